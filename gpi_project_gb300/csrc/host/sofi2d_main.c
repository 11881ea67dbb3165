/*
 * sofi2d_main.c -- command-line forward modelling on one GPU.
 *
 *   sofi2d_gb300 par.json [device]
 *
 * Same inputs and outputs as the reference's forward mode (src/sofi2D.c
 * main(), MODE=FW, FDORDER_TIME 2 or 4): parameter file, binary model files,
 * source and receiver files; SU seismograms SEIS_FILE_<comp>.su (.shotN with
 * RUN_MULTIPLE_SHOTS) and binary snapshots. The domain is never decomposed,
 * so snapshots are written merged (the file snapmerge would produce,
 * SNAP_FILE.bin.<comp>). With RUN_MULTIPLE_SHOTS = 1 every shot is resident
 * in one context and advanced together instead of one after the other
 * (reference sofi2D.c:325 loops over shots).
 *
 * MODE = FWI runs the gradient pass of the first iteration (sofi2D.c:277-393
 * with inversion.c, ITERMAX treated as 1) for EL_ISO with LNORM = 2 and
 * DTINV = 1: per shot a forward run keeping the gradient quantities, its
 * seismograms (SEIS_FILE_<comp>.su.shot<n>), the residuals against
 * DATA_DIR_<comp>.su.shot<n>, the backward run, and the gradient files
 * GRADIENT_gradient.{vp,vs,rho}.shot<n>; after the last shot their sums
 * GRADIENT_gradient.{vp,vs,rho} (output_gradient.c). Model updates, step
 * length search and L-BFGS are not part of it.
 */
#include "sofigpu.h"
#include "sofihost.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define IROUND(x) ((int)floor((x) + 0.5))

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

#define DIE_H(...)                                                  \
    do {                                                            \
        fprintf(stderr, "sofi2d_gb300: %s\n", sofih_last_error());  \
        return 1;                                                   \
    } while (0)
#define CHECK_G(call)                                                           \
    do {                                                                        \
        if ((call) != 0) {                                                      \
            fprintf(stderr, "sofi2d_gb300: %s\n", sofi_last_error());           \
            return 1;                                                           \
        }                                                                       \
    } while (0)

/* [NX][NY] (model files) -> [NY][NX] */
static float *transpose_xy(const float *a, int nx, int ny)
{
    float *t = (float *)malloc(sizeof(float) * (size_t)nx * ny);
    if (!t) {
        fprintf(stderr, "sofi2d_gb300: out of host memory\n");
        exit(1);
    }
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++)
            t[(size_t)j * nx + i] = a[(size_t)i * ny + j];
    return t;
}

/* One FWI gradient pass over the shots (inversion.c, output_gradient.c). */
static int run_fwi(const sofih_par *p, sofi_ctx *ctx, int nsrc, const float *srcpos, const float *srcxy,
                   const float *sig, int ntr, const int *rix, const int *riy, const int *rtr, const float *vp,
                   const float *vs, const float *rho)
{
    if (p->weq != 2 || p->fwi_lnorm != 2 || p->fwi_dtinv != 1) {
        fprintf(stderr, "sofi2d_gb300: MODE = FWI needs WEQ = EL_ISO, LNORM = 2 and DTINV = 1\n");
        return 1;
    }
    if (!ntr || !nsrc) {
        fprintf(stderr, "sofi2d_gb300: MODE = FWI needs sources and receivers\n");
        return 1;
    }
    const int nx = p->nx, ny = p->ny, nt = p->nt;
    const size_t n = (size_t)nx * ny;
    float *mv = transpose_xy(vp, nx, ny), *ms = transpose_xy(vs, nx, ny), *mr = transpose_xy(rho, nx, ny);
    float *buf = (float *)calloc(12 * n + 6 * (size_t)ntr * nt, sizeof(float));
    float *lam = buf, *mu = buf + n, *rhos = buf + 2 * n, *g = buf + 3 * n, *sum = buf + 6 * n;
    float *cx = buf + 12 * n, *cy = cx + (size_t)ntr * nt, *dx = cy + (size_t)ntr * nt;
    float *dy = dx + (size_t)ntr * nt, *rx = dy + (size_t)ntr * nt, *ry = rx + (size_t)ntr * nt;
    const int nshots = p->run_multiple_shots ? nsrc : 1;
    const char *gn[3] = {"vp", "vs", "rho"};
    int rc = 0;
    for (int s = 0; s < nshots && !rc; s++) {
        if (nshots == 1) {
            CHECK_G(sofi_set_sources(ctx, 0, nsrc, srcpos, sig));
        } else {
            float one[12];
            for (int r = 0; r < 12; r++)
                one[r] = srcpos[r * nsrc + s];
            CHECK_G(sofi_set_sources(ctx, 0, 1, one, sig + (size_t)s * nt));
        }
        CHECK_G(sofi_fwi_begin(ctx, p->fwi_velocity, p->fwi_adjoint, mv, ms, mr));
        CHECK_G(sofi_reset(ctx, -1));
        CHECK_G(sofi_run(ctx, nt));
        CHECK_G(sofi_synchronize(ctx));
        CHECK_G(sofi_get_section(ctx, 0, 1, cx));
        CHECK_G(sofi_get_section(ctx, 0, 2, cy));
        char path[700];
        const int src = nshots == 1 ? 0 : s;
        for (int q = 0; q < 2; q++) { /* the forward seismograms, as the reference writes them in FWI mode */
            snprintf(path, sizeof path, "%s_%s.%s.shot%d", p->seis_file, q ? "vy" : "vx",
                     sofih_seis_ext(p->seis_format), s + 1);
            if (sofih_write_seis(path, q ? cy : cx, ntr, nt, rix, riy, rtr, srcxy[src], srcxy[nsrc + src], p, s + 1,
                                 q + 1))
                DIE_H();
        }
        double l2x = 0, l2y = 0;
        snprintf(path, sizeof path, "%s_vx.su.shot%d", p->data_dir, s + 1);
        if (sofih_fwi_read_data(path, ntr, nt, dx) ||
            sofih_fwi_residual(cx, dx, ntr, nt, p->fwi_velocity, p->dt, rx, &l2x))
            DIE_H();
        snprintf(path, sizeof path, "%s_vy.su.shot%d", p->data_dir, s + 1);
        if (sofih_fwi_read_data(path, ntr, nt, dy) ||
            sofih_fwi_residual(cy, dy, ntr, nt, p->fwi_velocity, p->dt, ry, &l2y))
            DIE_H();
        CHECK_G(sofi_fwi_backward(ctx, rx, ry));
        CHECK_G(sofi_fwi_gradients(ctx, lam, mu, rhos));
        sofih_fwi_model_gradients(n, lam, mu, rhos, mv, ms, mr, g, g + n, g + 2 * n);
        for (int k = 0; k < 3 && !rc; k++) {
            snprintf(path, sizeof path, "%s_gradient.%s.shot%d", p->gradient, gn[k], s + 1);
            rc = sofih_write_gradient(path, g + k * n, nx, ny, p->idx, p->idy);
            for (size_t q = 0; q < n; q++) /* inversion.c:243-251 */
                sum[k * n + q] += g[k * n + q];
        }
        printf("sofi2d_gb300: FWI shot %d: L2 (x, y) %.6e %.6e\n", s + 1, l2x, l2y);
    }
    for (int k = 0; k < 3 && !rc; k++) {
        char path[700];
        snprintf(path, sizeof path, "%s_gradient.%s", p->gradient, gn[k]);
        rc = sofih_write_gradient(path, sum + k * n, nx, ny, p->idx, p->idy);
    }
    if (rc)
        DIE_H();
    free(buf), free(mv), free(ms), free(mr);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s par.json [device]\n", argv[0]);
        return 2;
    }
    int device = argc > 2 ? atoi(argv[2]) : 0;
    double t0 = now_s();
    sofih_par p;
    if (sofih_read_par(argv[1], &p))
        DIE_H();
    float *mat[8] = {0};
    /* READMOD = 0: the reference's built-in model, no model files (readmod.c:60-83) */
    if (p.readmod && sofih_read_model(&p, p.mfile, mat, 8))
        DIE_H();
    const char *names[8];
    int nm = p.readmod ? sofih_model_suffixes(p.weq, names, 8) : 0;
    float *vp = NULL, *vs = NULL, *rho = NULL, *qp = NULL, *qs = NULL, *eps = NULL, *del = NULL, *tet = NULL;
    for (int k = 0; k < nm; k++) {
        float **dst = !strcmp(names[k], "vp") ? &vp : !strcmp(names[k], "vs") ? &vs : !strcmp(names[k], "rho") ? &rho
                    : !strcmp(names[k], "qp") ? &qp : !strcmp(names[k], "qs") ? &qs
                    : !strcmp(names[k], "epsilon") ? &eps : !strcmp(names[k], "delta") ? &del : &tet;
        *dst = mat[k];
    }
    sofih_prep *prep;
    if (sofih_prepare(&p, vp, vs, rho, qp, qs, eps, del, tet, 0, &prep))
        DIE_H();
    float dtmax;
    if (sofih_check_cfl(&p, prep, &dtmax))
        DIE_H();
    float *srcpos, *srcxy;
    int nsrc;
    if (sofih_read_sources(&p, p.source_file, &srcpos, &srcxy, &nsrc))
        DIE_H();
    float *sig = (float *)malloc(sizeof(float) * (size_t)(nsrc ? nsrc : 1) * p.nt);
    if (p.source_shape == 3 ? sofih_wavelet_file(p.signal_file, p.nt, p.dt, nsrc, srcpos, sig)
                            : sofih_wavelet(p.source_shape, p.nt, p.dt, nsrc, srcpos, sig))
        DIE_H();
    int *rix = NULL, *riy = NULL, *rtr = NULL, ntr = 0;
    if (p.seismo && sofih_read_receiver_traces(&p, p.rec_file, &rix, &riy, &rtr, &ntr))
        DIE_H();
    /* source wavelet files (initsrc.c:64-93): per shot, the first source of the
     * shot, at its grid position and with its coordinates */
    if (p.sigout == 1 && nsrc > 0) {
        int nsh = p.run_multiple_shots ? nsrc : 1;
        for (int s = 0; s < nsh; s++) {
            char path[600];
            if (sofih_write_signal(&p, s + 1, sig + (size_t)s * p.nt, p.nt, (int)srcpos[s], (int)srcpos[nsrc + s],
                                   srcxy[s], srcxy[nsrc + s], path, sizeof path))
                fprintf(stderr, "warning: %s - no signature written\n", sofih_last_error());
        }
    }
    int nshots = (p.run_multiple_shots && nsrc > 0 && !p.mode_fwi) ? nsrc : 1;  /* FWI: one shot at a time */

    sofi_config c;
    memset(&c, 0, sizeof c);
    c.weq = p.weq, c.nx = p.nx, c.ny = p.ny, c.fdorder = p.fdorder, c.maxrelerror = p.maxrelerror;
    c.L = p.L, c.dt = p.dt, c.dh = p.dh, c.nt = p.nt, c.fw = p.fw, c.abs_type = p.abs_type;
    c.free_surf = p.free_surf, c.boundary = p.boundary, c.seismo = p.seismo, c.ndt = p.ndt;
    c.snap = p.snap;
    c.snap_first = IROUND(p.tsnap1 / p.dt), c.snap_inc = IROUND(p.tsnapinc / p.dt), c.snap_last = IROUND(p.tsnap2 / p.dt);
    c.idx = p.idx, c.idy = p.idy, c.nshots = nshots, c.shared_model = 1;
    c.fdorder_time = p.fdorder_time;
    sofi_ctx *ctx;
    CHECK_G(sofi_create(&c, device, &ctx));
    float hc[7];
    if (sofih_holberg(p.fdorder, p.maxrelerror, hc))
        DIE_H();
    CHECK_G(sofi_set_hc(ctx, hc));
    for (int k = 0; k < sofih_prep_num_fields(prep); k++)
        CHECK_G(sofi_set_model_field(ctx, 0, sofih_prep_field_name(prep, k), sofih_prep_field(prep, k), p.nx, 1));
    const char *vecs[] = {"K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half", "K_y", "a_y", "b_y",
                          "K_y_half", "a_y_half", "b_y_half", "bip", "cip", "peta"};
    for (size_t k = 0; k < sizeof vecs / sizeof vecs[0]; k++) {
        const float *d;
        int n = sofih_prep_vector(prep, vecs[k], &d);
        if (n)
            CHECK_G(sofi_set_model_vector(ctx, vecs[k], d, n));
    }
    if (p.mode_fwi) {
        if (ntr)
            CHECK_G(sofi_set_receivers(ctx, 0, ntr, rix, riy));
        int rc = run_fwi(&p, ctx, nsrc, srcpos, srcxy, sig, ntr, rix, riy, rtr, vp, vs, rho);
        sofi_destroy(ctx);
        sofih_prep_free(prep);
        printf("sofi2d_gb300: total %.3f s\n", now_s() - t0);
        return rc;
    }
    for (int s = 0; s < nshots; s++) {
        if (nshots == 1) {
            CHECK_G(sofi_set_sources(ctx, 0, nsrc, srcpos, sig));
        } else {
            float one[12];
            for (int r = 0; r < 12; r++)
                one[r] = srcpos[r * nsrc + s];
            CHECK_G(sofi_set_sources(ctx, s, 1, one, sig + (size_t)s * p.nt));
        }
        if (ntr)
            CHECK_G(sofi_set_receivers(ctx, s, ntr, rix, riy));
    }
    CHECK_G(sofi_reset(ctx, -1));
    double t1 = now_s();
    CHECK_G(sofi_run(ctx, p.nt));
    CHECK_G(sofi_synchronize(ctx));
    double t2 = now_s();
    float ms = 0;
    sofi_last_run_ms(ctx, &ms);
    double cells = (double)p.nx * p.ny * p.nt * nshots;
    printf("sofi2d_gb300: %d shot(s), %dx%d, NT=%d: time loop %.3f s (device %.3f s), %.2f Gcell-updates/s\n",
           nshots, p.nx, p.ny, p.nt, t2 - t1, ms * 1e-3, cells / (ms * 1e-3) / 1e9);

    /* seismograms (saveseis_glob.c naming) */
    if (p.seismo && ntr) {
        int ns;
        sofi_num_samples(ctx, &ns);
        float *sec = (float *)malloc(sizeof(float) * (size_t)ntr * (ns ? ns : 1));
        const char *cn[6] = {0, "vx", "vy", "p", "div", "curl"};
        int comps[5], nc = 0;
        if (p.seismo == 1) comps[nc++] = 1, comps[nc++] = 2;
        if (p.seismo == 2) comps[nc++] = 3;
        if (p.seismo == 3) comps[nc++] = 4, comps[nc++] = 5;
        if (p.seismo == 4) for (int k = 1; k <= 5; k++) comps[nc++] = k;
        for (int s = 0; s < nshots; s++)
            for (int q = 0; q < nc; q++) {
                CHECK_G(sofi_get_section(ctx, s, comps[q], sec));
                char path[700];
                const char *ext = sofih_seis_ext(p.seis_format);
                if (p.run_multiple_shots)
                    snprintf(path, sizeof path, "%s_%s.%s.shot%d", p.seis_file, cn[comps[q]], ext, s + 1);
                else
                    snprintf(path, sizeof path, "%s_%s.%s", p.seis_file, cn[comps[q]], ext);
                int src = nshots == 1 ? 0 : s;
                if (sofih_write_seis(path, sec, ntr, ns, rix, riy, rtr, srcxy[src], srcxy[nsrc + src], &p, s + 1,
                                     comps[q]))
                    DIE_H();
            }
        free(sec);
    }
    /* snapshots: the frames of every shot that writes them, shot after shot (initsrc.c:96-98) */
    int nsnap = 0, fsz = 0;
    sofi_num_snapshots(ctx, &nsnap, &fsz);
    int *snap_shots = (int *)malloc(sizeof(int) * (size_t)nshots);
    const int nss = snap_shots ? sofih_snapshot_shots(&p, nshots, snap_shots) : 0;
    if (nsnap && nss) {
        float *frame = (float *)malloc(sizeof(float) * (size_t)fsz);
        const char *cn[6] = {0, "vx", "vy", "p", "div", "curl"};
        for (int comp = 1; comp <= 5; comp++) {
            int want = (p.snap == 4) || (p.snap == 1 && comp <= 2) || (p.snap == 2 && comp == 3) ||
                       (p.snap == 3 && comp >= 4);
            if (!want)
                continue;
            char path[700];
            snprintf(path, sizeof path, "%s.%s.%s", p.snap_file, p.snap_format == 2 ? "asc" : "bin", cn[comp]);
            for (int q = 0; q < nss; q++)
                for (int k = 0; k < nsnap; k++) {
                    CHECK_G(sofi_get_snapshot(ctx, snap_shots[q] - 1, k, comp, frame));
                    if (sofih_write_snap_format(path, frame, fsz, q > 0 || k > 0, p.snap_format))
                        DIE_H();
                }
        }
        free(frame);
    }
    sofi_destroy(ctx);
    sofih_prep_free(prep);
    printf("sofi2d_gb300: total %.3f s\n", now_s() - t0);
    return 0;
}
