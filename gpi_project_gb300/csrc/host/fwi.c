/* fwi.c -- host side of one FWI gradient pass (MODE = FWI): the observed
 * data of a shot (inseis.c), the residuals that drive the backward run
 * (calc_res.c, LNORM = 2), the vp / vs / rho' gradients of the shot
 * (inversion.c:225-240) and their files (output_gradient.c, writemod.c with
 * format 3). Compiled as ISO C, so no product is contracted into a fused
 * multiply-add; the double constants of the reference's expressions are kept. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sofihost.h"

void sofih_set_error(const char *fmt, ...);

int sofih_fwi_read_data(const char *path, int ntr, int ns, float *out)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        sofih_set_error("Seismograms for inversion were not found: %s", path);
        return 1;
    }
    unsigned char h[240];
    unsigned short fns = 0;
    if (fread(h, 1, 240, fp) != 240) {
        fclose(fp);
        sofih_set_error("short read in SU file %s", path);
        return 1;
    }
    memcpy(&fns, h + 114, 2);
    const long tracelen = 240 + 4L * fns;
    int bad = fns < ns;
    for (int i = 0; i < ntr && !bad; i++)
        bad = fseek(fp, (long)i * tracelen + 240, SEEK_SET) != 0 ||
              fread(out + (size_t)i * ns, sizeof(float), (size_t)ns, fp) != (size_t)ns;
    fclose(fp);
    if (bad) {
        sofih_set_error("%s: %d traces of %d samples needed (file has %u samples per trace)", path, ntr, ns,
                        (unsigned)fns);
        return 1;
    }
    return 0;
}

int sofih_fwi_residual(const float *calc, const float *data, int ntr, int ns, int velocity, float dt, float *diff,
                       double *l2)
{
    if (!calc || !data || !diff || ntr < 0 || ns < 1) {
        sofih_set_error("invalid residual arguments");
        return 1;
    }
    float *ic = (float *)malloc(sizeof(float) * (size_t)ns * 2);
    if (!ic) {
        sofih_set_error("out of memory");
        return 1;
    }
    float *id = ic + ns;
    double sum = 0.0;
    for (int i = 0; i < ntr; i++) {
        const float *s = calc + (size_t)i * ns, *d = data + (size_t)i * ns;
        if (velocity == 0) { /* calc_res.c:138-145: displacement by a running sum */
            float as = 0.0f, ad = 0.0f;
            for (int j = 0; j < ns; j++) {
                as += s[j];
                ic[j] = as * dt;
                ad += d[j];
                id[j] = ad * dt;
            }
        } else {
            memcpy(ic, s, sizeof(float) * (size_t)ns);
            memcpy(id, d, sizeof(float) * (size_t)ns);
        }
        for (int j = 0; j < ns; j++) { /* calc_res.c:219-262: reversed in time */
            const float r = ic[j] - id[j];
            diff[(size_t)i * ns + (size_t)(ns - 1 - j)] = r;
            sum += (double)r * (double)r;
        }
    }
    free(ic);
    if (l2)
        *l2 = sum;
    return 0;
}

void sofih_fwi_model_gradients(size_t n, const float *lam, const float *mu, const float *rhos, const float *vp,
                               const float *vs, const float *rho, float *gvp, float *gvs, float *grho)
{
    for (size_t q = 0; q < n; q++) {
        gvp[q] = 2.0 * rho[q] * vp[q] * lam[q];
        /* the reference takes Vp0 in the mu term of the vs gradient */
        gvs[q] = (-4.0 * vs[q] * rho[q] * lam[q]) + 2.0 * rho[q] * vp[q] * mu[q];
        grho[q] = ((((vp[q] * vp[q]) - (2.0 * vs[q] * vs[q])) * lam[q]) + (vs[q] * vs[q] * mu[q]) + rhos[q]);
    }
}

int sofih_write_gradient(const char *path, const float *g, int nx, int ny, int idx, int idy)
{
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        sofih_set_error("Could not open model output file %s for writing.", path);
        return 1;
    }
    int bad = 0;
    idx = idx > 0 ? idx : 1, idy = idy > 0 ? idy : 1;
    for (int i = 0; i < nx && !bad; i += idx) /* writemod.c:40-42: x outer, y inner */
        for (int j = 0; j < ny && !bad; j += idy)
            bad = fwrite(g + (size_t)j * nx + i, sizeof(float), 1, fp) != 1;
    if (fclose(fp) || bad) {
        sofih_set_error("write error on %s", path);
        return 1;
    }
    return 0;
}
