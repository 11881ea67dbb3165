/*
 * prepare.c -- model preparation on the host (once per model).
 *
 * From the raw material of a model (model-file order, NX traces of NY
 * samples) to the arrays the time loop reads, following the reference:
 *   media conversion    readmod_elastic.c:112-136, readmod_visco.c:57-168,
 *                       readmod_elastic_vti.c:146-153, readmod_elastic_tti.c:151-176,
 *                       readmod_visco_vti.c:160-190, readmod_visco_tti.c:175-235
 *   halo of the model   matcopy_elastic.c (one rank: zero, or periodic in x with
 *                       BOUNDARY = 1), matcopy.c (VEL_ISO: periodic both ways)
 *   averaging           av_rho.c, av_mue.c (harmonic, in double), av_tau.c
 *   DT scaling          prepare_update_s_el/_visc/_vti/_tti.c, util.c dt_mult
 *   CPML profiles       PML_pro.c:86-334
 *   damping frame       absorb.c:34-121
 * Arithmetic keeps the reference's float variables and its double literals,
 * so the prepared arrays equal the reference's bit for bit on the same libm.
 * The viscoelastic defect planes (modulus * peta[l] * tau) are returned as the
 * l-independent factor (modulus * tau): the device multiplies by peta[l].
 */
#include "sofihost.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI M_PI
#define MAXF 40

void sofih_set_error(const char *fmt, ...);

struct sofih_prep {
    int nx, ny, nf;
    char names[MAXF][24];
    float *fields[MAXF];
    int nv;
    char vnames[16][16];
    float *vecs[16];
    int vlen[16];
    float vpmin, vpmax, vsmin, vsmax;
};

/* halo-1 work arrays: element (j, i), j = 0..NY+1, i = 0..NX+1 */
typedef struct {
    float *p;
    int pitch;
} h1;

#define H(a, j, i) ((a).p[(size_t)(j) * (size_t)(a).pitch + (size_t)(i)])

static h1 h1_new(int nx, int ny)
{
    h1 a;
    a.pitch = nx + 2;
    a.p = (float *)calloc((size_t)(nx + 2) * (size_t)(ny + 2), sizeof(float));
    return a;
}

static float *out_field(sofih_prep *m, const char *name)
{
    if (m->nf >= MAXF)
        return NULL;
    snprintf(m->names[m->nf], sizeof m->names[0], "%s", name);
    m->fields[m->nf] = (float *)malloc(sizeof(float) * (size_t)m->nx * (size_t)m->ny);
    return m->fields[m->nf++];
}

static void emit(sofih_prep *m, const char *name, h1 a)
{
    float *o = out_field(m, name);
    for (int j = 1; j <= m->ny; j++)
        memcpy(o + (size_t)(j - 1) * m->nx, &H(a, j, 1), sizeof(float) * (size_t)m->nx);
}

static void emit_product(sofih_prep *m, const char *name, h1 a, h1 b)
{
    float *o = out_field(m, name);
    for (int j = 1; j <= m->ny; j++)
        for (int i = 1; i <= m->nx; i++)
            o[(size_t)(j - 1) * m->nx + (i - 1)] = H(a, j, i) * H(b, j, i);
}

static float *out_vec(sofih_prep *m, const char *name, int n)
{
    snprintf(m->vnames[m->nv], sizeof m->vnames[0], "%s", name);
    m->vlen[m->nv] = n;
    m->vecs[m->nv] = (float *)calloc((size_t)(n + 1), sizeof(float)); /* 1-based */
    return m->vecs[m->nv++];
}

static int is_visco(int w) { return w == 3 || w == 5 || w == 7; }
static int is_tti(int w) { return w == 6 || w == 7; }

/* halo copy before averaging (one rank) */
static void model_halo(const sofih_par *p, h1 a, int full)
{
    int NX = p->nx, NY = p->ny;
    if (full)
        for (int i = 0; i <= NX + 1; i++) {
            H(a, NY + 1, i) = H(a, 1, i);
            H(a, 0, i) = H(a, NY, i);
        }
    if (full || p->boundary)
        for (int j = 0; j <= NY + 1; j++) {
            H(a, j, NX + 1) = H(a, j, 1);
            H(a, j, 0) = H(a, j, NX);
        }
}

static h1 harmonic4(const sofih_par *p, h1 u)
{
    h1 o = h1_new(p->nx, p->ny);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= p->ny; j++)
        for (int i = 1; i <= p->nx; i++) {
            if (H(u, j, i) == 0.f || H(u, j, i + 1) == 0.f || H(u, j + 1, i) == 0.f || H(u, j + 1, i + 1) == 0.f) {
                H(o, j, i) = 0.f;
            } else {
                double sum = (1.0 / H(u, j, i)) + (1.0 / H(u, j, i + 1)) + (1.0 / H(u, j + 1, i)) +
                             (1.0 / H(u, j + 1, i + 1));
                H(o, j, i) = (sum != 0.0) ? 4.0 / sum : 0.0;
            }
        }
    return o;
}

static h1 mean4(const sofih_par *p, h1 t)
{
    h1 o = h1_new(p->nx, p->ny);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= p->ny; j++)
        for (int i = 1; i <= p->nx; i++)
            H(o, j, i) = 0.25 * (H(t, j, i) + H(t, j, i + 1) + H(t, j + 1, i) + H(t, j + 1, i + 1));
    return o;
}

/* CPML profile point (PML_pro.c:101-150 / 196-236) */
static void pml_point(const sofih_par *p, float d0, float thick, float alpha_max, int clamp, float absc,
                      float absch, int h, float *K, float *Kh, float *d, float *dh, float *al, float *alh,
                      float *b, float *bh, float *a, float *ah)
{
    float NPOWER = p->npower, KMAX = p->k_max_cpml;
    K[h] = 1.0;
    Kh[h] = 1.0;
    if (absc >= 0.0) {
        float an = absc / thick;
        d[h] = d0 * pow(an, NPOWER);
        K[h] = 1.0 + (KMAX - 1.0) * pow(an, NPOWER);
        al[h] = alpha_max * (1.0 - an);
    }
    if (absch >= 0.0) {
        float an = absch / thick;
        dh[h] = d0 * pow(an, NPOWER);
        Kh[h] = 1.0 + (KMAX - 1.0) * pow(an, NPOWER);
        alh[h] = alpha_max * (1.0 - an);
    }
    if (clamp) {
        if (al[h] < 0.0)
            al[h] = 0.0;
        if (alh[h] < 0.0)
            alh[h] = 0.0;
    }
    b[h] = exp(-(d[h] / K[h] + al[h]) * p->dt);
    bh[h] = exp(-(dh[h] / Kh[h] + alh[h]) * p->dt);
    if (fabsf(d[h]) > 1.0e-6)
        a[h] = d[h] * (b[h] - 1.0) / (K[h] * (d[h] + K[h] * al[h]));
    if (fabsf(dh[h]) > 1.0e-6)
        ah[h] = dh[h] * (bh[h] - 1.0) / (Kh[h] * (dh[h] + Kh[h] * alh[h]));
}

static void cpml_profiles(const sofih_par *p, sofih_prep *m)
{
    int FW = p->fw, n = 2 * FW;
    float *K_x = out_vec(m, "K_x", n), *a_x = out_vec(m, "a_x", n), *b_x = out_vec(m, "b_x", n);
    float *K_xh = out_vec(m, "K_x_half", n), *a_xh = out_vec(m, "a_x_half", n), *b_xh = out_vec(m, "b_x_half", n);
    float *K_y = out_vec(m, "K_y", n), *a_y = out_vec(m, "a_y", n), *b_y = out_vec(m, "b_y", n);
    float *K_yh = out_vec(m, "K_y_half", n), *a_yh = out_vec(m, "a_y_half", n), *b_yh = out_vec(m, "b_y_half", n);
    float *d = calloc(n + 1, sizeof(float)), *dh = calloc(n + 1, sizeof(float));
    float *al = calloc(n + 1, sizeof(float)), *alh = calloc(n + 1, sizeof(float));
    float DH = p->dh;
    const float alpha_max_PML = 2.0 * PI * (p->fpml / 2.0);
    float thick = (float)FW * DH;
    float Rcoef = 0.001;
    float d0 = -(p->npower + 1) * p->vppml * log(Rcoef) / (2.0 * thick);
    float xl = thick, xr = (p->nx - 1) * DH - thick;
    for (int i = 1; i <= FW; i++) {
        float xval = DH * (i - 1);
        float ab = xl - xval, abh = xl - (xval + DH / 2.0);
        pml_point(p, d0, thick, alpha_max_PML, 1, ab, abh, i, K_x, K_xh, d, dh, al, alh, b_x, b_xh, a_x, a_xh);
    }
    for (int i = p->nx - FW + 1; i <= p->nx; i++) {
        int h = i - p->nx + 2 * FW;
        float xval = DH * (i - 1);
        float ab = xval - xr, abh = xval + DH / 2.0 - xr;
        pml_point(p, d0, thick, alpha_max_PML, 1, ab, abh, h, K_x, K_xh, d, dh, al, alh, b_x, b_xh, a_x, a_xh);
    }
    memset(d, 0, sizeof(float) * (n + 1)), memset(dh, 0, sizeof(float) * (n + 1));
    memset(al, 0, sizeof(float) * (n + 1)), memset(alh, 0, sizeof(float) * (n + 1));
    float yb = thick, yt = (p->ny - 1) * DH - thick;
    for (int i = 1; i <= FW; i++) {
        float yval = DH * (i - 1);
        float ab = yb - yval, abh = yb - (yval + DH / 2.0);
        pml_point(p, d0, thick, alpha_max_PML, 0, ab, abh, i, K_y, K_yh, d, dh, al, alh, b_y, b_yh, a_y, a_yh);
    }
    for (int i = p->ny - FW + 1; i <= p->ny; i++) {
        int h = i - p->ny + 2 * FW;
        float yval = DH * (i - 1);
        float ab = yval - yt, abh = yval + DH / 2.0 - yt;
        pml_point(p, d0, thick, alpha_max_PML, 0, ab, abh, h, K_y, K_yh, d, dh, al, alh, b_y, b_yh, a_y, a_yh);
    }
    free(d), free(dh), free(al), free(alh);
    /* shift to 0-based storage */
    for (int k = m->nv - 12; k < m->nv; k++)
        memmove(m->vecs[k], m->vecs[k] + 1, sizeof(float) * (size_t)n);
}

static void damping_frame(const sofih_par *p, sofih_prep *m)
{
    int FW = p->fw, NX = p->nx, NY = p->ny, FS = p->free_surf, BND = p->boundary;
    float amp = 1.0 - p->damping / 100.0;
    float *coeff = calloc((size_t)FW + 1, sizeof(float));
    float a = sqrt(-log(amp) / ((FW - 1) * (FW - 1)));
    for (int i = 1; i <= FW; i++)
        coeff[i] = exp(-(a * a * (FW - i) * (FW - i)));
    float *o = out_field(m, "absorb");
#define AB(j, i) o[(size_t)((j) - 1) * NX + (size_t)((i) - 1)]
    for (size_t k = 0; k < (size_t)NX * NY; k++)
        o[k] = 1.0;
    if (!BND) {
        for (int i = 1; i <= FW; i++) {
            int yb = FS ? 1 : i, ye = NY - i + 1;
            for (int j = yb; j <= ye; j++) {
                AB(j, i) = coeff[i];
                AB(j, NX - i + 1) = coeff[i];
            }
        }
    }
    for (int j = 1; j <= FW; j++) {
        int xb = BND ? 1 : j, xe = BND ? NX : NX - j + 1;
        for (int i = xb; i <= xe; i++) {
            if (!FS)
                AB(j, i) = coeff[j];
            AB(NY - j + 1, i) = coeff[j];
        }
    }
#undef AB
    free(coeff);
}

/* The reference's built-in models (READMOD = 0, readmod.c:60-83), MemModel
 * arrays as they leave it. hh_elastic.c / hh_visco.c: a half space below
 * y = 100 m (vp 3500, vs 2000, rho 2000) under a layer with vp 0, vs 1,
 * rho 1; the viscoelastic one with tau 0.01 (2.0 for 95 <= y <= 110 m).
 * hh_elastic_VTI.c / hh_elastic_TTI.c / hh_visco_VTI.c / hh_visco_TTI.c: a
 * homogeneous medium, c11 34.3, c33 22.7, c55 5.4, c13 10.7 GPa, rho 2000
 * (Jones and Wang 1981), tilted by 0 (elastic TTI) or 30 degrees
 * (viscoelastic TTI), tau = TAU. Float variables as the reference's. */
static void builtin_media(const sofih_par *p, int L, const float *pts, float ws, h1 prho, h1 ppi, h1 pu, h1 taus,
                          h1 taup, h1 c11, h1 c13, h1 c33, h1 c55, h1 c15, h1 c35, h1 t11, h1 t13, h1 t33, h1 t55,
                          h1 t15, h1 t35, float *vpmin, float *vpmax, float *vsmin, float *vsmax)
{
    const int weq = p->weq, NX = p->nx, NY = p->ny;
    if (weq == 2 || weq == 3) {
        const float vp1 = 0.0, vs1 = 1.0, rho1 = 1.0, h = 100.0;
        const float vp2 = 3500.0, vs2 = 2000.0, rho2 = 2000.0;
        const float tp1 = 0.01, ts1 = 0.01, tp2 = 0.01, ts2 = 0.01, h1_ = 95.0, h2_ = 110.0, tlp = 2.0, tls = 2.0;
        for (int i = 1; i <= NX; i++)
            for (int j = 1; j <= NY; j++) {
                const float y = (float)j * p->dh;
                const int top = y <= h;
                const float Vp = top ? vp1 : vp2, Vs = top ? vs1 : vs2, Rhov = top ? rho1 : rho2;
                if (weq == 2) {
                    H(pu, j, i) = Vs * Vs * Rhov;
                    H(ppi, j, i) = Vp * Vp * Rhov;
                } else {
                    float tp = top ? tp1 : tp2, ts = top ? ts1 : ts2;
                    if ((y >= h1_) && (y <= h2_))
                        tp = tlp, ts = tls;
                    float sumu = 0.0, sumpi = 0.0;
                    for (int l = 1; l <= L; l++) {
                        sumu = sumu + ((ws * ws * pts[l] * pts[l] * ts) / (1.0 + ws * ws * pts[l] * pts[l]));
                        sumpi = sumpi + ((ws * ws * pts[l] * pts[l] * tp) / (1.0 + ws * ws * pts[l] * pts[l]));
                    }
                    H(taus, j, i) = ts, H(taup, j, i) = tp;
                    H(pu, j, i) = Vs * Vs * Rhov / (1.0 + sumu);
                    H(ppi, j, i) = Vp * Vp * Rhov / (1.0 + sumpi);
                }
                H(prho, j, i) = Rhov;
            }
        *vpmin = *vpmax = vp2, *vsmin = *vsmax = vs2;
        return;
    }
    const float C11 = 34.3e9, C33 = 22.7e9, C55 = 5.4e9, C13 = 10.7e9, RHO = 2000.0;
    float c11v = C11, c33v = C33, c55v = C55, c13v = C13, tau11 = 0, tau13 = 0, tau55 = 0;
    if (L) {
        const float tau = p->tau;
        float sumc11 = 0.0, sumc33 = 0.0, sumc55 = 0.0, sumc13 = 0.0;
        for (int l = 1; l <= L; l++) {
            sumc11 = sumc11 + ((ws * ws * pts[l] * pts[l] * tau) / (1.0 + ws * ws * pts[l] * pts[l]));
            sumc33 = sumc33 + ((ws * ws * pts[l] * pts[l] * tau) / (1.0 + ws * ws * pts[l] * pts[l]));
            sumc55 = sumc55 + ((ws * ws * pts[l] * pts[l] * tau) / (1.0 + ws * ws * pts[l] * pts[l]));
        }
        c11v = c11v / (1.0 + sumc11);
        c33v = c33v / (1.0 + sumc33);
        c55v = c55v / (1.0 + sumc55);
        tau11 = tau, tau55 = tau;
        tau13 = (c11v * L * tau11 - 2.0 * c55v * L * tau55) / (c11v - 2.0 * c55v);
        for (int l = 1; l <= L; l++)
            sumc13 = sumc13 + ((ws * ws * pts[l] * pts[l] * tau13) / (1.0 + ws * ws * pts[l] * pts[l]));
        c13v = c13v / (1.0 + sumc13);
    }
    float o[6] = {c11v, c33v, c13v, c55v, 0.f, 0.f};
    if (is_tti(weq)) {
        const float THETA = weq == 7 ? 30.0 : 0.0;
        const float t = THETA * PI / 180.0;
        const float l1 = cos(t), l2 = sin(t);
        const float l12 = l1 * l1, l22 = l2 * l2, l14 = l12 * l12, l24 = l22 * l22, l13 = l1 * l12, l23 = l2 * l22;
        const float a1 = 2.0 * c13v + 4.0 * c55v, a3 = c11v + c33v - 4.0 * c55v, a4 = c11v + c33v - 2.0 * c13v;
        const float a5 = c13v - c11v + 2.0 * c55v, a6 = c13v - c33v + 2.0 * c55v;
        o[0] = c11v * l14 + c33v * l24 + a1 * l12 * l22;
        o[1] = c11v * l24 + c33v * l14 + a1 * l12 * l22;
        o[2] = a3 * l12 * l22 + c13v * (l14 + l24);
        o[3] = a4 * l12 * l22 + c55v * (l12 - l22) * (l12 - l22);
        o[4] = a5 * l13 * l2 - a6 * l1 * l23;
        o[5] = a5 * l23 * l1 - a6 * l2 * l13;
    }
    for (int i = 1; i <= NX; i++)
        for (int j = 1; j <= NY; j++) {
            H(prho, j, i) = RHO;
            H(c11, j, i) = o[0], H(c33, j, i) = o[1], H(c13, j, i) = o[2], H(c55, j, i) = o[3];
            if (is_tti(weq))
                H(c15, j, i) = o[4], H(c35, j, i) = o[5];
            if (L) {
                H(t11, j, i) = tau11, H(t33, j, i) = tau11, H(t13, j, i) = tau13, H(t55, j, i) = tau55;
                if (is_tti(weq))
                    H(t15, j, i) = tau13, H(t35, j, i) = tau13;
            }
        }
    /* phase velocities of the medium: vertical / horizontal P, S */
    const float vv = sqrtf(c33v / RHO), vh = sqrtf(c11v / RHO), vs = sqrtf(c55v / RHO);
    *vpmin = vv < vh ? vv : vh, *vpmax = vv > vh ? vv : vh, *vsmin = *vsmax = vs;
}

int sofih_prepare(const sofih_par *p, const float *vp, const float *vs, const float *rho, const float *qp,
                  const float *qs, const float *eps, const float *del, const float *theta, int nthreads,
                  sofih_prep **out)
{
    int weq = p->weq, NX = p->nx, NY = p->ny, L = is_visco(weq) ? p->L : 0;
    *out = NULL;
    if (weq < 0 || weq == 1 || weq > 7 || NX < 1 || NY < 1) {
        sofih_set_error("prepare: unsupported WEQ %d or empty grid", weq);
        return 1;
    }
    if (!p->readmod && (weq == 0 || p->mode_fwi)) {
        sofih_set_error("prepare: the built-in model (READMOD = 0) exists for WEQ 2..7 in MODE = FW only");
        return 1;
    }
    if (!p->readmod && (vp || vs || rho)) {
        sofih_set_error("prepare: READMOD = 0 selects the built-in model, but material arrays were given "
                        "(set READMOD = 1 to use them)");
        return 1;
    }
    if (p->readmod && (!vp || (!vs && weq != 0) || !rho || (L && (!qp || !qs)) || (weq >= 4 && (!eps || !del)) ||
                       (is_tti(weq) && !theta))) {
        sofih_set_error("prepare: missing material arrays for WEQ %d", weq);
        return 1;
    }
    if (is_visco(weq) && (L < 1 || L > SOFIH_MAX_L)) {
        sofih_set_error("prepare: viscoelastic media need 1 <= L <= %d", SOFIH_MAX_L);
        return 1;
    }
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    sofih_prep *m = (sofih_prep *)calloc(1, sizeof(sofih_prep));
    m->nx = NX, m->ny = NY;
    float DT = p->dt;
    /* relaxation mechanisms (readmod_visco.c:57-62) */
    float pts[SOFIH_MAX_L + 1] = {0}, peta[SOFIH_MAX_L + 1] = {0}, ws = 0.f;
    for (int l = 1; l <= L; l++) {
        pts[l] = 1.0 / (2.0 * PI * p->fl[l - 1]);
        peta[l] = DT / pts[l];
    }
    if (L)
        ws = 2.0 * PI * p->f_ref;
    h1 prho = h1_new(NX, NY), ppi = h1_new(NX, NY), pu = h1_new(NX, NY), taus = h1_new(NX, NY),
       taup = h1_new(NX, NY);
    h1 c11 = {0}, c13 = {0}, c33 = {0}, c55 = {0}, c15 = {0}, c35 = {0};
    h1 t11 = {0}, t13 = {0}, t33 = {0}, t55 = {0}, t15 = {0}, t35 = {0};
    if (weq >= 4) {
        c11 = h1_new(NX, NY), c13 = h1_new(NX, NY), c33 = h1_new(NX, NY), c55 = h1_new(NX, NY);
        if (is_tti(weq))
            c15 = h1_new(NX, NY), c35 = h1_new(NX, NY);
        if (L) {
            t11 = h1_new(NX, NY), t13 = h1_new(NX, NY), t33 = h1_new(NX, NY), t55 = h1_new(NX, NY);
            if (is_tti(weq))
                t15 = h1_new(NX, NY), t35 = h1_new(NX, NY);
        }
    }
    float vpmin = 1e30f, vpmax = 0.f, vsmin = 1e30f, vsmax = 0.f;
    if (!p->readmod) {
        builtin_media(p, L, pts, ws, prho, ppi, pu, taus, taup, c11, c13, c33, c55, c15, c35, t11, t13, t33, t55, t15,
                      t35, &vpmin, &vpmax, &vsmin, &vsmax);
    } else
#pragma omp parallel for schedule(static) reduction(min : vpmin, vsmin) reduction(max : vpmax, vsmax)
    for (int i = 1; i <= NX; i++)
        for (int j = 1; j <= NY; j++) {
            size_t k = (size_t)(i - 1) * NY + (j - 1);
            float v_p = vp[k], v_s = vs ? vs[k] : 0.0f, r = rho[k];
            if (v_p > 1.0f) {
                /* anisotropic media: horizontal P velocity vp*sqrt(1+2 eps) too
                 * (readmod_elastic_tti.c:128-131) */
                float v_h = weq >= 4 ? v_p * sqrtf(2.0f * eps[k] + 1.0f) : v_p;
                vpmin = v_p < vpmin ? v_p : vpmin;
                vpmax = v_p > vpmax ? v_p : vpmax;
                vpmax = v_h > vpmax ? v_h : vpmax;
            }
            if (v_s > 1.0f) {
                vsmin = v_s < vsmin ? v_s : vsmin;
                vsmax = v_s > vsmax ? v_s : vsmax;
            }
            H(prho, j, i) = r;
            if (weq == 0) {
                H(ppi, j, i) = v_p * v_p * r; /* readmod_acoustic.c:121 */
            } else if (weq == 2) {
                H(pu, j, i) = v_s * v_s * r;
                H(ppi, j, i) = v_p * v_p * r;
            } else if (weq == 3) {
                float tp = 2.0 / (qp[k] * L), ts = 2.0 / (qs[k] * L);
                float sumu = 0.0f, sumpi = 0.0f;
                for (int l = 1; l <= L; l++) {
                    sumu += ((ws * ws * pts[l] * pts[l] * ts) / (1.0 + ws * ws * pts[l] * pts[l]));
                    sumpi += ((ws * ws * pts[l] * pts[l] * tp) / (1.0 + ws * ws * pts[l] * pts[l]));
                }
                H(taus, j, i) = ts, H(taup, j, i) = tp;
                H(pu, j, i) = v_s * v_s * r / (1.0 + sumu);
                H(ppi, j, i) = v_p * v_p * r / (1.0 + sumpi);
            } else {
                float e = eps[k], d = del[k];
                float a33 = r * v_p * v_p, a55 = r * v_s * v_s;
                float a11 = a33 * (2.0 * e + 1.0);
                float a13 = sqrt((2.0 * d * a33 * (a33 - a55)) + ((a33 - a55) * (a33 - a55))) - a55;
                float tau11 = 0, tau13 = 0, tau55 = 0;
                if (L) {
                    float tp = 2.0 / (qp[k] * L), ts = 2.0 / (qs[k] * L);
                    float sumu = 0.0f, sumpi = 0.0f, sumc13 = 0.0f;
                    for (int l = 1; l <= L; l++) {
                        sumu += ((ws * ws * pts[l] * pts[l] * ts) / (1.0 + ws * ws * pts[l] * pts[l]));
                        sumpi += ((ws * ws * pts[l] * pts[l] * tp) / (1.0 + ws * ws * pts[l] * pts[l]));
                    }
                    tau11 = tp, tau55 = ts;
                    a11 = a11 / (1.0 + sumpi);
                    a33 = a33 / (1.0 + sumpi);
                    a55 = a55 / (1.0 + sumu);
                    tau13 = (a11 * L * tau11 - 2.0 * a55 * L * tau55) / (a11 - 2.0 * a55);
                    for (int l = 1; l <= L; l++)
                        sumc13 += ((ws * ws * pts[l] * pts[l] * tau13) / (1.0 + ws * ws * pts[l] * pts[l]));
                    a13 = a13 / (1.0 + sumc13);
                }
                if (is_tti(weq)) {
                    float t = theta[k] * PI / 180.0;
                    float l1 = cos(t), l2 = sin(t);
                    float l12 = l1 * l1, l22 = l2 * l2, l14 = l12 * l12, l24 = l22 * l22;
                    float l13 = l1 * l12, l23 = l2 * l22;
                    float b1 = 2.0 * a13 + 4.0 * a55, b3 = a11 + a33 - 4.0 * a55, b4 = a11 + a33 - 2.0 * a13;
                    float b5 = a13 - a11 + 2.0 * a55, b6 = a13 - a33 + 2.0 * a55;
                    H(c11, j, i) = a11 * l14 + a33 * l24 + b1 * l12 * l22;
                    H(c33, j, i) = a11 * l24 + a33 * l14 + b1 * l12 * l22;
                    H(c13, j, i) = b3 * l12 * l22 + a13 * (l14 + l24);
                    H(c55, j, i) = b4 * l12 * l22 + a55 * (l12 - l22) * (l12 - l22);
                    H(c15, j, i) = b5 * l13 * l2 - b6 * l1 * l23;
                    H(c35, j, i) = b5 * l23 * l1 - b6 * l2 * l13;
                } else {
                    H(c11, j, i) = a11, H(c13, j, i) = a13, H(c33, j, i) = a33, H(c55, j, i) = a55;
                }
                if (L) {
                    H(t11, j, i) = tau11, H(t33, j, i) = tau11, H(t13, j, i) = tau13, H(t55, j, i) = tau55;
                    if (is_tti(weq))
                        H(t15, j, i) = tau13, H(t35, j, i) = tau13;
                }
            }
        }
    m->vpmin = vpmin, m->vpmax = vpmax, m->vsmin = vsmin, m->vsmax = vsmax;

    /* halo + averaging (prepmod.c:42-120) */
    h1 rip = h1_new(NX, NY), rjp = h1_new(NX, NY);
    if (weq == 0) {
        model_halo(p, prho, 0), model_halo(p, ppi, 0); /* matcopy_elastic(prho, ppi, ppi), prepmod.c:41 */
    } else if (weq == 2 || weq == 3) {
        h1 hs[5] = {prho, ppi, pu, taus, taup};
        for (int k = 0; k < (weq == 3 ? 5 : 3); k++)
            model_halo(p, hs[k], weq == 3);
    } else {
        h1 hs[8] = {prho, c11, c55, c15, c35, t55, t15, t35};
        for (int k = 0; k < 8; k++)
            if (hs[k].p)
                model_halo(p, hs[k], 0);
    }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++) {
            H(rjp, j, i) = 1.0 / (0.5 * (H(prho, j, i) + H(prho, j + 1, i)));
            H(rip, j, i) = 1.0 / (0.5 * (H(prho, j, i) + H(prho, j, i + 1)));
        }
    emit(m, "prip", rip);
    emit(m, "prjp", rjp);
    if (weq == 0) {
        /* prepare_update_s_ac.c:27-34 */
        h1 g = h1_new(NX, NY);
#pragma omp parallel for schedule(static)
        for (int j = 1; j <= NY; j++)
            for (int i = 1; i <= NX; i++)
                H(g, j, i) = H(ppi, j, i) * DT;
        emit(m, "g", g);
        free(g.p);
    } else if (weq == 2 || weq == 3) {
        h1 uipjp = harmonic4(p, pu);
        h1 tsip = weq == 3 ? mean4(p, taus) : (h1){0};
        h1 g = h1_new(NX, NY), f = h1_new(NX, NY), fip = h1_new(NX, NY);
#pragma omp parallel for schedule(static)
        for (int j = 1; j <= NY; j++)
            for (int i = 1; i <= NX; i++) {
                if (weq == 2) {
                    H(fip, j, i) = H(uipjp, j, i) * DT;
                    H(f, j, i) = H(pu, j, i) * DT;
                    H(g, j, i) = H(ppi, j, i) * DT;
                } else {
                    H(fip, j, i) = H(uipjp, j, i) * DT * (1.0 + L * H(tsip, j, i));
                    H(f, j, i) = H(pu, j, i) * DT * (1.0 + L * H(taus, j, i));
                    H(g, j, i) = H(ppi, j, i) * DT * (1.0 + L * H(taup, j, i));
                }
            }
        emit(m, "g", g), emit(m, "f", f), emit(m, "fipjp", fip);
        emit(m, "ppi", ppi), emit(m, "pu", pu);
        if (weq == 3) {
            emit_product(m, "d_base", pu, taus);
            emit_product(m, "e_base", ppi, taup);
            emit_product(m, "dip_base", uipjp, tsip);
            if (p->free_surf)
                emit(m, "taus", taus), emit(m, "taup", taup);
            free(tsip.p);
        }
        free(uipjp.p), free(g.p), free(f.p), free(fip.p);
    } else {
        h1 c55ip = harmonic4(p, c55), c15ip = {0}, c35ip = {0}, t55ip = {0}, t15ip = {0}, t35ip = {0};
        if (is_tti(weq))
            c15ip = harmonic4(p, c15), c35ip = harmonic4(p, c35);
        if (L) {
            t55ip = mean4(p, t55);
            if (is_tti(weq))
                t15ip = mean4(p, t15), t35ip = mean4(p, t35);
        }
        /* ppi / pu alias c11 / c55 (initmem_model.c:87-91); elastic c11 is DT-scaled in place */
        struct {
            const char *name;
            h1 c, tau;
        } mods[8] = {{"c11", c11, t11}, {"c13", c13, t13}, {"c33", c33, t33}, {"c55ipjp", c55ip, t55ip},
                     {"c15", c15, t15}, {"c35", c35, t35}, {"c15ipjp", c15ip, t15ip}, {"c35ipjp", c35ip, t35ip}};
        int nm = is_tti(weq) ? 8 : 4;
        if (!L) {
            for (int k = 0; k < nm; k++) {
                float *o = out_field(m, mods[k].name);
                for (int j = 1; j <= NY; j++)
                    for (int i = 1; i <= NX; i++)
                        o[(size_t)(j - 1) * NX + (i - 1)] = H(mods[k].c, j, i) * DT;
            }
            /* ppi is c11 after dt_mult, pu is c55 (never scaled) */
            float *o = out_field(m, "ppi");
            for (int j = 1; j <= NY; j++)
                for (int i = 1; i <= NX; i++)
                    o[(size_t)(j - 1) * NX + (i - 1)] = H(c11, j, i) * DT;
            emit(m, "pu", c55);
        } else {
            for (int k = 0; k < nm; k++) {
                char nu[24], nb[32];
                snprintf(nu, sizeof nu, "%su", mods[k].name);
                snprintf(nb, sizeof nb, "%sd_base", mods[k].name);
                float *o = out_field(m, nu);
                for (int j = 1; j <= NY; j++)
                    for (int i = 1; i <= NX; i++)
                        o[(size_t)(j - 1) * NX + (i - 1)] = H(mods[k].c, j, i) * DT * (1.0 + L * H(mods[k].tau, j, i));
                emit_product(m, nb, mods[k].c, mods[k].tau);
            }
            emit(m, "ppi", c11);
            emit(m, "pu", c55);
        }
        h1 fr[] = {c55ip, c15ip, c35ip, t55ip, t15ip, t35ip};
        for (size_t k = 0; k < sizeof fr / sizeof fr[0]; k++)
            free(fr[k].p);
    }
    if (L) {
        float *bip = out_vec(m, "bip", L), *cip = out_vec(m, "cip", L), *pe = out_vec(m, "peta", L);
        for (int l = 1; l <= L; l++) {
            if (p->fdorder_time == 4) { /* prepare_update_s_visc_4.c:40-45 (c1 = 13/12) */
                const float c1 = 13.0 / 12.0;
                bip[l - 1] = 1.0 / (1.0 + (c1 * peta[l] * 0.5));
                cip[l - 1] = 1.0 - (c1 * peta[l] * 0.5);
            } else {
                bip[l - 1] = 1.0 / (1.0 + (peta[l] * 0.5));
                cip[l - 1] = 1.0 - (peta[l] * 0.5);
            }
            pe[l - 1] = peta[l];
        }
    }
    if (p->fw > 0 && p->abs_type == 1)
        cpml_profiles(p, m);
    if (p->fw > 0 && p->abs_type == 2)
        damping_frame(p, m);
    h1 all[] = {prho, ppi, pu, taus, taup, c11, c13, c33, c55, c15, c35, t11, t13, t33, t55, t15, t35, rip, rjp};
    for (size_t k = 0; k < sizeof all / sizeof all[0]; k++)
        free(all[k].p);
    *out = m;
    return 0;
}

void sofih_prep_free(sofih_prep *m)
{
    if (!m)
        return;
    for (int k = 0; k < m->nf; k++)
        free(m->fields[k]);
    for (int k = 0; k < m->nv; k++)
        free(m->vecs[k]);
    free(m);
}

int sofih_prep_num_fields(const sofih_prep *m) { return m ? m->nf : 0; }
const char *sofih_prep_field_name(const sofih_prep *m, int k) { return (m && k >= 0 && k < m->nf) ? m->names[k] : NULL; }
const float *sofih_prep_field(const sofih_prep *m, int k) { return (m && k >= 0 && k < m->nf) ? m->fields[k] : NULL; }

int sofih_prep_vector(const sofih_prep *m, const char *name, const float **data)
{
    for (int k = 0; m && k < m->nv; k++)
        if (!strcmp(m->vnames[k], name)) {
            *data = m->vecs[k];
            return m->vlen[k];
        }
    *data = NULL;
    return 0;
}

void sofih_prep_vrange(const sofih_prep *m, float *vpmin, float *vpmax, float *vsmin, float *vsmax)
{
    *vpmin = m->vpmin, *vpmax = m->vpmax, *vsmin = m->vsmin, *vsmax = m->vsmax;
}
