/*
 * sofi_oracle.c -- CPU restatement of SOFI2D's forward-modelling path.
 *
 * TEST INFRASTRUCTURE ONLY (see sofi_oracle.h). Not part of the product.
 *
 * Written from the reference's behaviour, one function per reference
 * routine, with the reference file:line cited on each. Arithmetic follows
 * the reference's C types: `real` is float in the f32 build, and wherever
 * the reference writes a double literal (2.0, 0.25, 1.0, PI ...) the same
 * literal is kept so that C's usual conversions promote the same
 * sub-expressions to double. In the f64 build every variable is double.
 *
 * Grid convention (reference util.c:231-262 `matrix`): 2-D arrays cover
 * rows -ND+1..NY+ND and columns -ND+1..NX+ND, x fastest, zero-initialised.
 * One rank (NPROCX = NPROCY = 1): exchange_v/exchange_s only act for
 * BOUNDARY = 1 (periodic in x), where they copy columns across the seam.
 */
#include "sofi_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL real;

#define PI M_PI
#define iround(x) ((int)(floor)((x) + 0.5))

typedef struct {
    real *p;
} arr2;

struct orc_ctx {
    orc_params P;
    int ND, pitch, rows;
    int NT;
    real DT, DH, DTDH;
    int GX[5], GY[5];
    real hc[7];
    char err[256];
    /* material / coefficients */
    arr2 prho, ppi, pu, ptaus, ptaup, prip, prjp, puipjp, ptausipjp, g, f, fipjp, absorb;
    arr2 pc11, pc13, pc33, pc55, pc15, pc35, pc55ipjp, pc15ipjp, pc35ipjp;
    arr2 ptau11, ptau13, ptau33, ptau55, ptau15, ptau35, ptau55ipjp, ptau15ipjp, ptau35ipjp;
    arr2 pc11u, pc13u, pc33u, pc55u, pc15u, pc35u, pc55ipjpu, pc15ipjpu, pc35ipjpu;
    arr2 dip[ORC_MAX_L + 1], d[ORC_MAX_L + 1], e[ORC_MAX_L + 1];
    arr2 pc11d[ORC_MAX_L + 1], pc13d[ORC_MAX_L + 1], pc33d[ORC_MAX_L + 1], pc55d[ORC_MAX_L + 1];
    arr2 pc15d[ORC_MAX_L + 1], pc35d[ORC_MAX_L + 1], pc55ipjpd[ORC_MAX_L + 1], pc15ipjpd[ORC_MAX_L + 1];
    arr2 pc35ipjpd[ORC_MAX_L + 1];
    real peta[ORC_MAX_L + 1], bip[ORC_MAX_L + 1], cip[ORC_MAX_L + 1];
    /* CPML profiles [1..2FW] */
    real *K_x, *K_x_half, *a_x, *a_x_half, *b_x, *b_x_half, *d_x, *d_x_half, *alpha_prime_x,
        *alpha_prime_x_half;
    real *K_y, *K_y_half, *a_y, *a_y_half, *b_y, *b_y_half, *d_y, *d_y_half, *alpha_prime_y,
        *alpha_prime_y_half;
    /* CPML memory: [1..NY][1..2FW] and [1..2FW][1..NX] */
    real *psi_sxx_x, *psi_sxy_x, *psi_vxx, *psi_vyx; /* NY x 2FW */
    real *psi_syy_y, *psi_sxy_y, *psi_vyy, *psi_vxy; /* 2FW x NX */
    /* wavefield */
    arr2 vx, vy, sxx, syy, sxy, vxx, vyy, vyx, vxy;
    arr2 pr[ORC_MAX_L + 1], pp[ORC_MAX_L + 1], pq[ORC_MAX_L + 1];
    /* FDORDER_TIME = 4 (Adams-Bashforth): histories of the stress-derivative
     * sums svx/svy and of the velocity derivatives, levels 1..4
     * (memw_struct.h: svx_1..4, vxx_1..4, ...), and levels 2..4 of the
     * memory variables ([k][l], k = 2..4; level 1 is pr/pp/pq) */
    int ab4;
    arr2 svx[5], svy[5], hxx[5], hyy[5], hxy[5], hyx[5];
    arr2 pr_h[5][ORC_MAX_L + 1], pp_h[5][ORC_MAX_L + 1], pq_h[5][ORC_MAX_L + 1];
    /* raw material input [NX][NY] */
    float *mat_vp, *mat_vs, *mat_rho, *mat_qp, *mat_qs, *mat_eps, *mat_del, *mat_tet;
    /* acquisition */
    int nsrc;
    float *srcpos; /* [12][nsrc] */
    real *signals; /* [nsrc][NT] (1-based nt at index nt-1) */
    int ntr;
    int *rx, *ry;
    int ns;
    float *sec[6]; /* comp 1..5: [ntr][ns] */
    /* snapshots */
    int nsnap, snap_cap, snap_nx, snap_ny, snapidx[5];
    float *snaps[6];
    int lsnap, isnap, esnap, lsamp;
    int step;
    int prepared;
    double tim[4];
    /* MODE = FWI, EL_ISO (inversion.c, snap_store.c, calc_conv.c): the
     * quantities wavefield_update_v.c:31-44 and wavefield_update_s_el.c:43-47
     * keep for the gradient, the forward ones of every step ([NT][5][NY][NX]),
     * the adjoint signals at the receivers ([2][ntr][NT]) and the per-shot
     * gradient sums ([NY][NX]) */
    int fwi, fwi_vel, fwi_adj, fwi_back;
    arr2 pvxp1, pvyp1, ux, uy, uxy;
    float *fwd;
    float *adj;
    float *g_lam, *g_mu, *g_rhos;
};

/* Adams-Bashforth coefficients of FDORDER_TIME = 4, float as the reference
 * declares them (wavefield_update_v_4.c:29-32) */
static const float AB1 = 13.0 / 12.0, AB2 = -5.0 / 24.0, AB3 = 1.0 / 6.0, AB4 = -1.0 / 24.0;

/* ----------------------------------------------------------------- helpers */

#define A(a, j, i) ((a).p[(size_t)((j) + c->ND - 1) * (size_t)c->pitch + (size_t)((i) + c->ND - 1)])
#define PSIX(a, j, h) ((a)[(size_t)((j) - 1) * (size_t)(2 * c->P.fw) + (size_t)((h) - 1)])
#define PSIY(a, h, i) ((a)[(size_t)((h) - 1) * (size_t)c->P.nx + (size_t)((i) - 1)])
#define MAT(m, j, i) ((m)[(size_t)((i) - 1) * (size_t)c->P.ny + (size_t)((j) - 1)])

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static arr2 alloc2(orc_ctx *c)
{
    arr2 a;
    a.p = (real *)calloc((size_t)c->pitch * (size_t)c->rows, sizeof(real));
    return a;
}

static void free2(arr2 *a)
{
    free(a->p);
    a->p = NULL;
}

static real *vec(int n)
{
    return (real *)calloc((size_t)(n + 1), sizeof(real));
}

static int is_visco(int weq)
{
    return weq == ORC_VEL_ISO || weq == ORC_VEL_VTI || weq == ORC_VEL_TTI;
}

static int is_iso(int weq)
{
    return weq == ORC_AC_ISO || weq == ORC_EL_ISO || weq == ORC_VEL_ISO;
}

static int is_ac(int weq)
{
    return weq == ORC_AC_ISO;
}

static int is_vti(int weq)
{
    return weq == ORC_EL_VTI || weq == ORC_VEL_VTI;
}

static int is_tti(int weq)
{
    return weq == ORC_EL_TTI || weq == ORC_VEL_TTI;
}

/* Holberg / Taylor coefficients: reference src/holbergcoeff.c:38-100.
 * Published tables (Taylor row = MAXRELERROR 0, Holberg 1987 rows 1-4);
 * element 0 is the operator's points-per-wavelength figure. */
static const double holberg_table[5][6][7] = {
    {{23.0, 1.0, 0, 0, 0, 0, 0},
     {8.0, 9.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0, 0, 0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0, 0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0, 35.0 / 294912.0, 0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0, -5445.0 / 1835008.0,
      847.0 / 2359296.0, -63.0 / 2883584.0}},
    {{49.7, 1.0010, 0, 0, 0, 0, 0},
     {8.32, 1.1382, -0.046414, 0, 0, 0, 0},
     {4.77, 1.1965, -0.078804, 0.0081781, 0, 0, 0},
     {3.69, 1.2257, -0.099537, 0.018063, -0.0026274, 0, 0},
     {3.19, 1.2415, -0.11231, 0.026191, -0.0064682, 0.001191, 0},
     {2.91, 1.2508, -0.12034, 0.032131, -0.010142, 0.0029857, -0.00066667}},
    {{22.2, 1.0050, 0, 0, 0, 0, 0},
     {5.65, 1.1534, -0.052806, 0, 0, 0, 0},
     {3.74, 1.2111, -0.088313, 0.011768, 0, 0, 0},
     {3.11, 1.2367, -0.10815, 0.023113, -0.0046905, 0, 0},
     {2.80, 1.2496, -0.11921, 0.031130, -0.0093272, 0.0025161, 0},
     {2.62, 1.2568, -0.12573, 0.036423, -0.013132, 0.0047484, -0.0015979}},
    {{15.8, 1.0100, 0, 0, 0, 0, 0},
     {4.80, 1.1640, -0.057991, 0, 0, 0, 0},
     {3.39, 1.2192, -0.094070, 0.014608, 0, 0, 0},
     {2.90, 1.2422, -0.11269, 0.026140, -0.0064054, 0, 0},
     {2.65, 1.2534, -0.12257, 0.033755, -0.011081, 0.0036784, 0},
     {2.51, 1.2596, -0.12825, 0.038550, -0.014763, 0.0058619, -0.0024538}},
    {{9.16, 1.0300, 0, 0, 0, 0, 0},
     {3.47, 1.1876, -0.072518, 0, 0, 0, 0},
     {2.91, 1.2341, -0.10569, 0.022589, 0, 0, 0},
     {2.61, 1.2516, -0.12085, 0.032236, -0.011459, 0, 0},
     {2.45, 1.2596, -0.12829, 0.038533, -0.014681, 0.0072580, 0},
     {2.36, 1.2640, -0.13239, 0.042217, -0.017803, 0.0081959, -0.0051848}},
};

/* ---------------------------------------------------------------- create */

orc_ctx *orc_create(const orc_params *p)
{
    if (p->fdorder < 2 || p->fdorder > 12 || (p->fdorder & 1) || p->maxrelerror < 0 || p->maxrelerror > 4 ||
        p->nx < 1 || p->ny < 1 || p->nt < 1 || p->L < 0 || p->L > ORC_MAX_L)
        return NULL;
    if (!(is_iso(p->weq) || is_vti(p->weq) || is_tti(p->weq)))
        return NULL;
    /* read_par_json.c:304-306: viscoelastic needs L >= 1. The viscoelastic
     * free surface (surface.c) reads ptaus/ptaup, which the anisotropic
     * viscoelastic readers never fill. */
    if ((is_visco(p->weq) && p->L < 1) || (p->free_surf && is_visco(p->weq) && !is_iso(p->weq)))
        return NULL;
    /* Acoustic media have no mu and no sxy (initmem_model.c:33-39,
     * initmem_wavefield.c:32-39); the free surface (surface_elastic.c) and
     * the div/curl outputs (seismo_ssg.c:49-59, snap_ssg.c:166) read them. */
    if (is_ac(p->weq) && (p->free_surf || p->seismo >= 3 || p->snap >= 3))
        return NULL;
    /* FDORDER_TIME = 4 exists for EL_ISO and VEL_ISO only (prepmod.c:160-186);
     * the free surface is not restated for it */
    if (p->fdorder_time == 4 && (!(p->weq == ORC_EL_ISO || p->weq == ORC_VEL_ISO) || p->free_surf))
        return NULL;
    if (p->fdorder_time != 0 && p->fdorder_time != 2 && p->fdorder_time != 4)
        return NULL;
    orc_ctx *c = (orc_ctx *)calloc(1, sizeof(orc_ctx));
    c->P = *p;
    if (!is_visco(p->weq))
        c->P.L = 0; /* read_par_json.c:308-311 */
    c->ND = p->fdorder / 2;           /* initmem.c:59 */
    c->ab4 = p->fdorder_time == 4;
    c->pitch = p->nx + 2 * c->ND;
    c->rows = p->ny + 2 * c->ND;
    c->NT = p->nt;
    c->DT = (real)p->dt;
    c->DH = (real)p->dh;
    c->DTDH = c->DT / c->DH;          /* prepmod.c:37 */
    for (int k = 0; k <= 6; k++) {
        float hf = (float)holberg_table[p->maxrelerror][p->fdorder / 2 - 1][k]; /* float hcall[] */
        c->hc[k] = (real)hf;
    }
    /* subgrid_bounds.c:65-66,260-270 for NPROCX = NPROCY = 1 */
    c->GY[1] = 1, c->GY[2] = p->fw, c->GY[3] = p->ny - p->fw, c->GY[4] = p->ny;
    c->GX[1] = 1, c->GX[2] = p->fw, c->GX[3] = p->nx - p->fw, c->GX[4] = p->nx;
    if (p->free_surf == 1)
        c->GY[2] = 0;
    if (p->boundary == 1) {
        c->GX[2] = 0;
        c->GX[3] = p->nx, c->GX[4] = p->nx - 1;
    }
#ifdef _OPENMP
    if (p->nthreads > 0)
        omp_set_num_threads(p->nthreads);
#endif
    int L = c->P.L;
    arr2 *all[] = {&c->prho, &c->ppi, &c->pu, &c->ptaus, &c->ptaup, &c->prip, &c->prjp, &c->puipjp,
                   &c->ptausipjp, &c->g, &c->f, &c->fipjp, &c->absorb, &c->pc11, &c->pc13, &c->pc33,
                   &c->pc55, &c->pc15, &c->pc35, &c->pc55ipjp, &c->pc15ipjp, &c->pc35ipjp, &c->ptau11,
                   &c->ptau13, &c->ptau33, &c->ptau55, &c->ptau15, &c->ptau35, &c->ptau55ipjp,
                   &c->ptau15ipjp, &c->ptau35ipjp, &c->pc11u, &c->pc13u, &c->pc33u, &c->pc55u, &c->pc15u,
                   &c->pc35u, &c->pc55ipjpu, &c->pc15ipjpu, &c->pc35ipjpu, &c->vx, &c->vy, &c->sxx,
                   &c->syy, &c->sxy, &c->vxx, &c->vyy, &c->vyx, &c->vxy};
    for (size_t k = 0; k < sizeof(all) / sizeof(all[0]); k++)
        *all[k] = alloc2(c);
    /* initmem_model.c:87-91,101-105,119-123,150-156: for anisotropic media
     * ppi, pu and puipjp are the same arrays as pc11, pc55 and pc55ipjp, so the
     * seismogram/snapshot/free-surface terms that read ppi/pu see c11 and c55. */
    if (!is_iso(p->weq)) {
        free2(&c->ppi), free2(&c->pu), free2(&c->puipjp);
        c->ppi = c->pc11, c->pu = c->pc55, c->puipjp = c->pc55ipjp;
    }
    /* initmem_wavefield.c:34: the acoustic psyy is psxx (one pressure field,
     * updated by g*vxx and then by g*vyy); sxy stays zero */
    if (is_ac(p->weq)) {
        free2(&c->syy);
        c->syy = c->sxx;
    }
    if (c->ab4) {
        for (int k = 1; k <= 4; k++) {
            c->svx[k] = alloc2(c), c->svy[k] = alloc2(c);
            c->hxx[k] = alloc2(c), c->hyy[k] = alloc2(c), c->hxy[k] = alloc2(c), c->hyx[k] = alloc2(c);
        }
        for (int l = 1; l <= L; l++)
            for (int k = 2; k <= 4; k++)
                c->pr_h[k][l] = alloc2(c), c->pp_h[k][l] = alloc2(c), c->pq_h[k][l] = alloc2(c);
    }
    for (int l = 1; l <= L; l++) {
        c->dip[l] = alloc2(c), c->d[l] = alloc2(c), c->e[l] = alloc2(c);
        c->pr[l] = alloc2(c), c->pp[l] = alloc2(c), c->pq[l] = alloc2(c);
        if (!is_iso(p->weq)) {
            c->pc11d[l] = alloc2(c), c->pc13d[l] = alloc2(c), c->pc33d[l] = alloc2(c);
            c->pc55d[l] = alloc2(c), c->pc15d[l] = alloc2(c), c->pc35d[l] = alloc2(c);
            c->pc55ipjpd[l] = alloc2(c), c->pc15ipjpd[l] = alloc2(c), c->pc35ipjpd[l] = alloc2(c);
        }
    }
    int n2 = 2 * (p->fw > 0 ? p->fw : 1);
    real **vv[] = {&c->K_x, &c->K_x_half, &c->a_x, &c->a_x_half, &c->b_x, &c->b_x_half, &c->d_x,
                   &c->d_x_half, &c->alpha_prime_x, &c->alpha_prime_x_half, &c->K_y, &c->K_y_half,
                   &c->a_y, &c->a_y_half, &c->b_y, &c->b_y_half, &c->d_y, &c->d_y_half,
                   &c->alpha_prime_y, &c->alpha_prime_y_half};
    for (size_t k = 0; k < sizeof(vv) / sizeof(vv[0]); k++)
        *vv[k] = vec(n2);
    size_t nxf = (size_t)p->ny * (size_t)n2, nyf = (size_t)n2 * (size_t)p->nx;
    c->psi_sxx_x = (real *)calloc(nxf, sizeof(real));
    c->psi_sxy_x = (real *)calloc(nxf, sizeof(real));
    c->psi_vxx = (real *)calloc(nxf, sizeof(real));
    c->psi_vyx = (real *)calloc(nxf, sizeof(real));
    c->psi_syy_y = (real *)calloc(nyf, sizeof(real));
    c->psi_sxy_y = (real *)calloc(nyf, sizeof(real));
    c->psi_vyy = (real *)calloc(nyf, sizeof(real));
    c->psi_vxy = (real *)calloc(nyf, sizeof(real));
    c->ns = p->ndt > 0 ? c->NT / p->ndt : 0; /* read_par_json.c:516: iround of an int quotient */
    /* snapshot schedule: time_loop.c:38-40, indices initproc.c:87-119 */
    if (p->snap) {
        c->snapidx[1] = 1;
        c->snapidx[3] = 1;
        c->snapidx[2] = -1, c->snapidx[4] = -1;
        for (int i = 1; i <= p->nx; i += p->idx)
            c->snapidx[2] = i;
        for (int j = 1; j <= p->ny; j += p->idy)
            c->snapidx[4] = j;
        c->snap_nx = (c->snapidx[2] - c->snapidx[1]) / p->idx + 1;
        c->snap_ny = (c->snapidx[4] - c->snapidx[3]) / p->idy + 1;
    }
    orc_reset(c);
    return c;
}

void orc_destroy(orc_ctx *c)
{
    if (!c)
        return;
    if (!is_iso(c->P.weq))
        c->ppi.p = c->pu.p = c->puipjp.p = NULL; /* aliases of pc11/pc55/pc55ipjp */
    if (is_ac(c->P.weq))
        c->syy.p = NULL; /* alias of sxx */
    arr2 *all[] = {&c->prho, &c->ppi, &c->pu, &c->ptaus, &c->ptaup, &c->prip, &c->prjp, &c->puipjp,
                   &c->ptausipjp, &c->g, &c->f, &c->fipjp, &c->absorb, &c->pc11, &c->pc13, &c->pc33,
                   &c->pc55, &c->pc15, &c->pc35, &c->pc55ipjp, &c->pc15ipjp, &c->pc35ipjp, &c->ptau11,
                   &c->ptau13, &c->ptau33, &c->ptau55, &c->ptau15, &c->ptau35, &c->ptau55ipjp,
                   &c->ptau15ipjp, &c->ptau35ipjp, &c->pc11u, &c->pc13u, &c->pc33u, &c->pc55u, &c->pc15u,
                   &c->pc35u, &c->pc55ipjpu, &c->pc15ipjpu, &c->pc35ipjpu, &c->vx, &c->vy, &c->sxx,
                   &c->syy, &c->sxy, &c->vxx, &c->vyy, &c->vyx, &c->vxy};
    for (size_t k = 0; k < sizeof(all) / sizeof(all[0]); k++)
        free2(all[k]);
    for (int k = 1; k <= 4; k++) {
        free2(&c->svx[k]), free2(&c->svy[k]);
        free2(&c->hxx[k]), free2(&c->hyy[k]), free2(&c->hxy[k]), free2(&c->hyx[k]);
        for (int l = 1; l <= c->P.L; l++)
            free2(&c->pr_h[k][l]), free2(&c->pp_h[k][l]), free2(&c->pq_h[k][l]);
    }
    for (int l = 1; l <= c->P.L; l++) {
        free2(&c->dip[l]), free2(&c->d[l]), free2(&c->e[l]);
        free2(&c->pr[l]), free2(&c->pp[l]), free2(&c->pq[l]);
        free2(&c->pc11d[l]), free2(&c->pc13d[l]), free2(&c->pc33d[l]), free2(&c->pc55d[l]);
        free2(&c->pc15d[l]), free2(&c->pc35d[l]), free2(&c->pc55ipjpd[l]), free2(&c->pc15ipjpd[l]);
        free2(&c->pc35ipjpd[l]);
    }
    real *vv[] = {c->K_x, c->K_x_half, c->a_x, c->a_x_half, c->b_x, c->b_x_half, c->d_x, c->d_x_half,
                  c->alpha_prime_x, c->alpha_prime_x_half, c->K_y, c->K_y_half, c->a_y, c->a_y_half,
                  c->b_y, c->b_y_half, c->d_y, c->d_y_half, c->alpha_prime_y, c->alpha_prime_y_half,
                  c->psi_sxx_x, c->psi_sxy_x, c->psi_vxx, c->psi_vyx, c->psi_syy_y, c->psi_sxy_y,
                  c->psi_vyy, c->psi_vxy, c->signals};
    for (size_t k = 0; k < sizeof(vv) / sizeof(vv[0]); k++)
        free(vv[k]);
    float *ff[] = {c->mat_vp, c->mat_vs, c->mat_rho, c->mat_qp, c->mat_qs, c->mat_eps, c->mat_del,
                   c->mat_tet, c->srcpos};
    for (size_t k = 0; k < sizeof(ff) / sizeof(ff[0]); k++)
        free(ff[k]);
    for (int k = 1; k <= 5; k++) {
        free(c->sec[k]);
        free(c->snaps[k]);
    }
    free(c->rx);
    free(c->ry);
    free2(&c->pvxp1), free2(&c->pvyp1), free2(&c->ux), free2(&c->uy), free2(&c->uxy);
    free(c->fwd), free(c->adj), free(c->g_lam), free(c->g_mu), free(c->g_rhos);
    free(c);
}

const char *orc_error(orc_ctx *c)
{
    return c ? c->err : "null context";
}

int orc_set_material(orc_ctx *c, const char *name, const float *data)
{
    float **dst = NULL;
    if (!strcmp(name, "vp")) dst = &c->mat_vp;
    else if (!strcmp(name, "vs")) dst = &c->mat_vs;
    else if (!strcmp(name, "rho")) dst = &c->mat_rho;
    else if (!strcmp(name, "qp")) dst = &c->mat_qp;
    else if (!strcmp(name, "qs")) dst = &c->mat_qs;
    else if (!strcmp(name, "epsilon")) dst = &c->mat_eps;
    else if (!strcmp(name, "delta")) dst = &c->mat_del;
    else if (!strcmp(name, "theta")) dst = &c->mat_tet;
    if (!dst) {
        snprintf(c->err, sizeof c->err, "unknown material %s", name);
        return 1;
    }
    size_t n = (size_t)c->P.nx * (size_t)c->P.ny;
    if (!*dst)
        *dst = (float *)malloc(n * sizeof(float));
    memcpy(*dst, data, n * sizeof(float));
    return 0;
}

/* ------------------------------------------------------------- model read */

/* Relaxation-mechanism vectors shared by the visco readers:
 * readmod_visco.c:57-62 (pts, peta, ws). */
static void visco_pts(orc_ctx *c, real *pts, real *ws)
{
    for (int l = 1; l <= c->P.L; l++) {
        pts[l] = 1.0 / (2.0 * PI * (real)c->P.fl[l - 1]);
        c->peta[l] = c->DT / pts[l];
    }
    *ws = 2.0 * PI * (real)c->P.f_ref;
}

/* readmod_elastic.c:112-136 */
static void readmod_elastic(orc_ctx *c)
{
    for (int i = 1; i <= c->P.nx; i++)
        for (int j = 1; j <= c->P.ny; j++) {
            real vp = MAT(c->mat_vp, j, i), vs = MAT(c->mat_vs, j, i), rho = MAT(c->mat_rho, j, i);
            A(c->pu, j, i) = vs * vs * rho;
            A(c->prho, j, i) = rho;
            A(c->ppi, j, i) = vp * vp * rho;
        }
}

/* readmod_acoustic.c:105-122 */
static void readmod_acoustic(orc_ctx *c)
{
    for (int i = 1; i <= c->P.nx; i++)
        for (int j = 1; j <= c->P.ny; j++) {
            real vp = MAT(c->mat_vp, j, i), rho = MAT(c->mat_rho, j, i);
            A(c->prho, j, i) = rho;
            A(c->ppi, j, i) = vp * vp * rho;
        }
}

/* readmod_visco.c:57-62,135-168 */
static void readmod_visco(orc_ctx *c)
{
    real pts[ORC_MAX_L + 1], ws;
    int L = c->P.L;
    visco_pts(c, pts, &ws);
    for (int i = 1; i <= c->P.nx; i++)
        for (int j = 1; j <= c->P.ny; j++) {
            real vp = MAT(c->mat_vp, j, i), vs = MAT(c->mat_vs, j, i), rho = MAT(c->mat_rho, j, i);
            real tp = 2.0 / (MAT(c->mat_qp, j, i) * L);
            real ts = 2.0 / (MAT(c->mat_qs, j, i) * L);
            real sumu = 0.0f, sumpi = 0.0f;
            for (int l = 1; l <= L; l++) {
                sumu += ((ws * ws * pts[l] * pts[l] * ts) / (1.0 + ws * ws * pts[l] * pts[l]));
                sumpi += ((ws * ws * pts[l] * pts[l] * tp) / (1.0 + ws * ws * pts[l] * pts[l]));
            }
            real muv = vs * vs * rho / (1.0 + sumu);
            real piv = vp * vp * rho / (1.0 + sumpi);
            A(c->ptaus, j, i) = ts;
            A(c->ptaup, j, i) = tp;
            A(c->pu, j, i) = muv;
            A(c->prho, j, i) = rho;
            A(c->ppi, j, i) = piv;
        }
}

/* Thomsen -> VTI stiffness: readmod_elastic_vti.c:146-149 */
static void thomsen_vti(real rho, real vp, real vs, real eps, real del, real *c11, real *c13, real *c33,
                        real *c55)
{
    *c33 = rho * vp * vp;
    *c55 = rho * vs * vs;
    *c11 = *c33 * (2.0 * eps + 1.0);
    *c13 = sqrt((2.0 * del * *c33 * (*c33 - *c55)) + ((*c33 - *c55) * (*c33 - *c55))) - *c55;
}

/* Bond transformation: readmod_elastic_tti.c:151-176 */
static void bond_tti(real c11, real c13, real c33, real c55, real tet, real *o)
{
    real t = tet * PI / 180.0;
    real l1 = cos(t), l2 = sin(t);
    real l12 = l1 * l1, l22 = l2 * l2;
    real l14 = l12 * l12, l24 = l22 * l22;
    real l13 = l1 * l12, l23 = l2 * l22;
    real a1 = 2.0 * c13 + 4.0 * c55;
    real a3 = c11 + c33 - 4.0 * c55;
    real a4 = c11 + c33 - 2.0 * c13;
    real a5 = c13 - c11 + 2.0 * c55;
    real a6 = c13 - c33 + 2.0 * c55;
    o[0] = c11 * l14 + c33 * l24 + a1 * l12 * l22;            /* c11t */
    o[1] = c11 * l24 + c33 * l14 + a1 * l12 * l22;            /* c33t */
    o[2] = a3 * l12 * l22 + c13 * (l14 + l24);                /* c13t */
    o[3] = a4 * l12 * l22 + c55 * (l12 - l22) * (l12 - l22);  /* c55t */
    o[4] = a5 * l13 * l2 - a6 * l1 * l23;                     /* c15t */
    o[5] = a5 * l23 * l1 - a6 * l2 * l13;                     /* c35t */
}

/* readmod_elastic_vti.c / readmod_elastic_tti.c / readmod_visco_vti.c:160-190 /
 * readmod_visco_tti.c:175-235 */
static void readmod_aniso(orc_ctx *c)
{
    int L = c->P.L, weq = c->P.weq;
    real pts[ORC_MAX_L + 1], ws = 0;
    if (is_visco(weq))
        visco_pts(c, pts, &ws);
    for (int i = 1; i <= c->P.nx; i++)
        for (int j = 1; j <= c->P.ny; j++) {
            real vp = MAT(c->mat_vp, j, i), vs = MAT(c->mat_vs, j, i), rho = MAT(c->mat_rho, j, i);
            real eps = MAT(c->mat_eps, j, i), del = MAT(c->mat_del, j, i);
            real c11, c13, c33, c55;
            thomsen_vti(rho, vp, vs, eps, del, &c11, &c13, &c33, &c55);
            real tau11 = 0, tau33 = 0, tau13 = 0, tau55 = 0;
            if (is_visco(weq)) {
                real tp = 2.0 / (MAT(c->mat_qp, j, i) * L);
                real ts = 2.0 / (MAT(c->mat_qs, j, i) * L);
                real sumu = 0.0f, sumpi = 0.0f, sumc13 = 0.0f;
                for (int l = 1; l <= L; l++) {
                    sumu += ((ws * ws * pts[l] * pts[l] * ts) / (1.0 + ws * ws * pts[l] * pts[l]));
                    sumpi += ((ws * ws * pts[l] * pts[l] * tp) / (1.0 + ws * ws * pts[l] * pts[l]));
                }
                tau11 = tau33 = tp;
                tau55 = ts;
                c11 = c11 / (1.0 + sumpi);
                c33 = c33 / (1.0 + sumpi);
                c55 = c55 / (1.0 + sumu);
                tau13 = (c11 * L * tau11 - 2.0 * c55 * L * tau55) / (c11 - 2.0 * c55);
                for (int l = 1; l <= L; l++)
                    sumc13 += ((ws * ws * pts[l] * pts[l] * tau13) / (1.0 + ws * ws * pts[l] * pts[l]));
                c13 = c13 / (1.0 + sumc13);
            }
            A(c->prho, j, i) = rho;
            if (is_tti(weq)) {
                real o[6];
                bond_tti(c11, c13, c33, c55, MAT(c->mat_tet, j, i), o);
                A(c->pc11, j, i) = o[0];
                A(c->pc33, j, i) = o[1];
                A(c->pc13, j, i) = o[2];
                A(c->pc55, j, i) = o[3];
                A(c->pc15, j, i) = o[4];
                A(c->pc35, j, i) = o[5];
            } else {
                A(c->pc11, j, i) = c11;
                A(c->pc13, j, i) = c13;
                A(c->pc33, j, i) = c33;
                A(c->pc55, j, i) = c55;
            }
            if (is_visco(weq)) {
                A(c->ptau11, j, i) = tau11;
                A(c->ptau33, j, i) = tau33;
                A(c->ptau13, j, i) = tau13;
                A(c->ptau55, j, i) = tau55;
                if (is_tti(weq)) {
                    A(c->ptau15, j, i) = tau13;
                    A(c->ptau35, j, i) = tau13;
                }
            }
        }
}

/* ----------------------------------------------------------- prepmod */

/* Halo copy of material before averaging with one rank.
 * matcopy_elastic.c:40-117: without BOUNDARY nothing is copied (ghost rows and
 * columns stay zero); with BOUNDARY = 1 columns 0 and NX+1 wrap.
 * matcopy.c (visco, VEL_ISO only): unconditional exchange = full periodic wrap. */
static void matcopy_wrap(orc_ctx *c, arr2 *arrs, int n, int full)
{
    int NX = c->P.nx, NY = c->P.ny;
    for (int k = 0; k < n; k++) {
        arr2 a = arrs[k];
        if (full)
            for (int i = 0; i <= NX + 1; i++) {
                A(a, NY + 1, i) = A(a, 1, i);
                A(a, 0, i) = A(a, NY, i);
            }
        if (full || c->P.boundary)
            for (int j = 0; j <= NY + 1; j++) {
                A(a, j, NX + 1) = A(a, j, 1);
                A(a, j, 0) = A(a, j, NX);
            }
    }
}

/* av_rho.c:28-36 */
static void av_rho(orc_ctx *c)
{
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++) {
            A(c->prjp, j, i) = 1.0 / (0.5 * (A(c->prho, j, i) + A(c->prho, j + 1, i)));
            A(c->prip, j, i) = 1.0 / (0.5 * (A(c->prho, j, i) + A(c->prho, j, i + 1)));
        }
}

/* av_mue.c:27-43 (harmonic mean of four neighbours, accumulated in double) */
static void av_mue(orc_ctx *c, arr2 u, arr2 uipjp)
{
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++) {
            if ((A(u, j, i) == 0.f) || (A(u, j, i + 1) == 0.f) || (A(u, j + 1, i) == 0.f) ||
                (A(u, j + 1, i + 1) == 0.f)) {
                A(uipjp, j, i) = 0.f;
            } else {
                double sum = (1.0 / A(u, j, i)) + (1.0 / A(u, j, i + 1)) + (1.0 / A(u, j + 1, i)) +
                             (1.0 / A(u, j + 1, i + 1));
                A(uipjp, j, i) = (sum != 0.0) ? 4.0 / sum : 0.0;
            }
        }
}

/* av_tau.c:27-34 */
static void av_tau(orc_ctx *c, arr2 t, arr2 tipjp)
{
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++)
            A(tipjp, j, i) = 0.25 * (A(t, j, i) + A(t, j, i + 1) + A(t, j + 1, i) + A(t, j + 1, i + 1));
}

/* util.c:37-46 */
static void dt_mult(orc_ctx *c, arr2 a)
{
    for (int i = 1; i <= c->P.nx; i++)
        for (int j = 1; j <= c->P.ny; j++)
            A(a, j, i) = A(a, j, i) * c->DT;
}

/* prepare_update_s_el.c / _visc.c:27-47 / _vti.c / _tti.c */
static void prepare_update(orc_ctx *c)
{
    int L = c->P.L, weq = c->P.weq;
    real DT = c->DT;
    for (int l = 1; l <= L; l++) {
        if (c->ab4) { /* prepare_update_s_visc_4.c:40-45 */
            c->bip[l] = 1.0 / (1.0 + (AB1 * c->peta[l] * 0.5));
            c->cip[l] = 1.0 - (AB1 * c->peta[l] * 0.5);
        } else {
            c->bip[l] = 1.0 / (1.0 + (c->peta[l] * 0.5));
            c->cip[l] = 1.0 - (c->peta[l] * 0.5);
        }
    }
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++) {
            if (weq == ORC_AC_ISO) {
                A(c->g, j, i) = A(c->ppi, j, i) * DT; /* prepare_update_s_ac.c:27-34 */
            } else if (weq == ORC_EL_ISO) {
                A(c->fipjp, j, i) = A(c->puipjp, j, i) * DT;
                A(c->f, j, i) = A(c->pu, j, i) * DT;
                A(c->g, j, i) = A(c->ppi, j, i) * DT;
            } else if (weq == ORC_VEL_ISO) {
                A(c->fipjp, j, i) = A(c->puipjp, j, i) * DT * (1.0 + L * A(c->ptausipjp, j, i));
                A(c->f, j, i) = A(c->pu, j, i) * DT * (1.0 + L * A(c->ptaus, j, i));
                A(c->g, j, i) = A(c->ppi, j, i) * DT * (1.0 + L * A(c->ptaup, j, i));
                for (int l = 1; l <= L; l++) {
                    A(c->dip[l], j, i) = A(c->puipjp, j, i) * c->peta[l] * A(c->ptausipjp, j, i);
                    A(c->d[l], j, i) = A(c->pu, j, i) * c->peta[l] * A(c->ptaus, j, i);
                    A(c->e[l], j, i) = A(c->ppi, j, i) * c->peta[l] * A(c->ptaup, j, i);
                }
            } else if (weq == ORC_VEL_VTI) {
                A(c->pc55ipjpu, j, i) = A(c->pc55ipjp, j, i) * DT * (1.0 + L * A(c->ptau55ipjp, j, i));
                A(c->pc13u, j, i) = A(c->pc13, j, i) * DT * (1.0 + L * A(c->ptau13, j, i));
                A(c->pc11u, j, i) = A(c->pc11, j, i) * DT * (1.0 + L * A(c->ptau11, j, i));
                A(c->pc33u, j, i) = A(c->pc33, j, i) * DT * (1.0 + L * A(c->ptau33, j, i));
                for (int l = 1; l <= L; l++) {
                    A(c->pc55ipjpd[l], j, i) = A(c->pc55ipjp, j, i) * c->peta[l] * A(c->ptau55ipjp, j, i);
                    A(c->pc13d[l], j, i) = A(c->pc13, j, i) * c->peta[l] * A(c->ptau13, j, i);
                    A(c->pc33d[l], j, i) = A(c->pc33, j, i) * c->peta[l] * A(c->ptau33, j, i);
                    A(c->pc11d[l], j, i) = A(c->pc11, j, i) * c->peta[l] * A(c->ptau11, j, i);
                }
            } else if (weq == ORC_VEL_TTI) {
                A(c->pc11u, j, i) = A(c->pc11, j, i) * DT * (1.0 + L * A(c->ptau11, j, i));
                A(c->pc33u, j, i) = A(c->pc33, j, i) * DT * (1.0 + L * A(c->ptau33, j, i));
                A(c->pc13u, j, i) = A(c->pc13, j, i) * DT * (1.0 + L * A(c->ptau13, j, i));
                A(c->pc55u, j, i) = A(c->pc55, j, i) * DT * (1.0 + L * A(c->ptau55, j, i));
                A(c->pc15u, j, i) = A(c->pc15, j, i) * DT * (1.0 + L * A(c->ptau15, j, i));
                A(c->pc35u, j, i) = A(c->pc35, j, i) * DT * (1.0 + L * A(c->ptau35, j, i));
                A(c->pc55ipjpu, j, i) = A(c->pc55ipjp, j, i) * DT * (1.0 + L * A(c->ptau55ipjp, j, i));
                A(c->pc15ipjpu, j, i) = A(c->pc15ipjp, j, i) * DT * (1.0 + L * A(c->ptau15ipjp, j, i));
                A(c->pc35ipjpu, j, i) = A(c->pc35ipjp, j, i) * DT * (1.0 + L * A(c->ptau35ipjp, j, i));
                for (int l = 1; l <= L; l++) {
                    A(c->pc55ipjpd[l], j, i) = A(c->pc55ipjp, j, i) * c->peta[l] * A(c->ptau55ipjp, j, i);
                    A(c->pc15ipjpd[l], j, i) = A(c->pc15ipjp, j, i) * c->peta[l] * A(c->ptau15ipjp, j, i);
                    A(c->pc35ipjpd[l], j, i) = A(c->pc35ipjp, j, i) * c->peta[l] * A(c->ptau35ipjp, j, i);
                    A(c->pc11d[l], j, i) = A(c->pc11, j, i) * c->peta[l] * A(c->ptau11, j, i);
                    A(c->pc33d[l], j, i) = A(c->pc33, j, i) * c->peta[l] * A(c->ptau33, j, i);
                    A(c->pc13d[l], j, i) = A(c->pc13, j, i) * c->peta[l] * A(c->ptau13, j, i);
                    A(c->pc55d[l], j, i) = A(c->pc55, j, i) * c->peta[l] * A(c->ptau55, j, i);
                    A(c->pc15d[l], j, i) = A(c->pc15, j, i) * c->peta[l] * A(c->ptau15, j, i);
                    A(c->pc35d[l], j, i) = A(c->pc35, j, i) * c->peta[l] * A(c->ptau35, j, i);
                }
            }
        }
}

/* prepmod.c:37-193 */
static void prepmod(orc_ctx *c)
{
    int weq = c->P.weq;
    switch (weq) {
      case ORC_AC_ISO: {
          arr2 m[3] = {c->prho, c->ppi, c->ppi}; /* prepmod.c:40-43 */
          matcopy_wrap(c, m, 3, 0);
          av_rho(c);
          break;
      }
      case ORC_EL_ISO: {
          arr2 m[3] = {c->prho, c->ppi, c->pu};
          matcopy_wrap(c, m, 3, 0);
          av_mue(c, c->pu, c->puipjp);
          av_rho(c);
          break;
      }
      case ORC_VEL_ISO: {
          arr2 m[5] = {c->prho, c->ppi, c->pu, c->ptaus, c->ptaup};
          matcopy_wrap(c, m, 5, 1);
          av_mue(c, c->pu, c->puipjp);
          av_rho(c);
          av_tau(c, c->ptaus, c->ptausipjp);
          break;
      }
      case ORC_EL_VTI: {
          arr2 m[3] = {c->prho, c->pc11, c->pc55};
          matcopy_wrap(c, m, 3, 0);
          av_mue(c, c->pc55, c->pc55ipjp);
          av_rho(c);
          break;
      }
      case ORC_VEL_VTI: {
          arr2 m[3] = {c->prho, c->ptau55, c->pc55};
          matcopy_wrap(c, m, 3, 0);
          av_mue(c, c->pc55, c->pc55ipjp);
          av_rho(c);
          av_tau(c, c->ptau55, c->ptau55ipjp);
          break;
      }
      case ORC_EL_TTI: {
          arr2 m[5] = {c->prho, c->pc11, c->pc55, c->pc15, c->pc35};
          matcopy_wrap(c, m, 5, 0);
          av_mue(c, c->pc55, c->pc55ipjp);
          av_mue(c, c->pc15, c->pc15ipjp);
          av_mue(c, c->pc35, c->pc35ipjp);
          av_rho(c);
          break;
      }
      case ORC_VEL_TTI: {
          arr2 m[7] = {c->prho, c->ptau55, c->pc55, c->ptau15, c->pc15, c->ptau35, c->pc35};
          matcopy_wrap(c, m, 7, 0);
          av_mue(c, c->pc55, c->pc55ipjp);
          av_mue(c, c->pc15, c->pc15ipjp);
          av_mue(c, c->pc35, c->pc35ipjp);
          av_rho(c);
          av_tau(c, c->ptau55, c->ptau55ipjp);
          av_tau(c, c->ptau15, c->ptau15ipjp);
          av_tau(c, c->ptau35, c->ptau35ipjp);
          break;
      }
    }
    /* prepmod.c:135-151 */
    if (weq == ORC_EL_VTI) {
        dt_mult(c, c->pc11), dt_mult(c, c->pc33), dt_mult(c, c->pc13), dt_mult(c, c->pc55ipjp);
    } else if (weq == ORC_EL_TTI) {
        dt_mult(c, c->pc11), dt_mult(c, c->pc33), dt_mult(c, c->pc13), dt_mult(c, c->pc15);
        dt_mult(c, c->pc35), dt_mult(c, c->pc55ipjp), dt_mult(c, c->pc35ipjp), dt_mult(c, c->pc15ipjp);
    } else {
        prepare_update(c);
    }
}

/* ----------------------------------------------------------- boundaries */

/* One side of a CPML profile: PML_pro.c:101-150 (x) / 196-236 (y).
 * `grid_dist` = abscissa of grid points, `half_dist` = of half points. */
static void pml_point(orc_ctx *c, real d0, real thickness, real alpha_max, int clamp_alpha, real absc,
                      real absc_half, int h, real *K, real *Kh, real *dd, real *dh_, real *al, real *alh,
                      real *b, real *bh, real *a, real *ah)
{
    real NPOWER = c->P.npower, KMAX = c->P.k_max_cpml;
    K[h] = 1.0;
    Kh[h] = 1.0;
    if (absc >= 0.0) {
        real an = absc / thickness;
        dd[h] = d0 * pow(an, NPOWER);
        K[h] = 1.0 + (KMAX - 1.0) * pow(an, NPOWER);
        al[h] = alpha_max * (1.0 - an);
    }
    if (absc_half >= 0.0) {
        real an = absc_half / thickness;
        dh_[h] = d0 * pow(an, NPOWER);
        Kh[h] = 1.0 + (KMAX - 1.0) * pow(an, NPOWER);
        alh[h] = alpha_max * (1.0 - an);
    }
    if (clamp_alpha) {
        if (al[h] < 0.0)
            al[h] = 0.0;
        if (alh[h] < 0.0)
            alh[h] = 0.0;
    }
    b[h] = exp(-(dd[h] / K[h] + al[h]) * c->DT);
    bh[h] = exp(-(dh_[h] / Kh[h] + alh[h]) * c->DT);
    if (fabs((double)dd[h]) > 1.0e-6)
        a[h] = dd[h] * (b[h] - 1.0) / (K[h] * (dd[h] + K[h] * al[h]));
    if (fabs((double)dh_[h]) > 1.0e-6)
        ah[h] = dh_[h] * (bh[h] - 1.0) / (Kh[h] * (dh_[h] + Kh[h] * alh[h]));
}

/* PML_pro.c:86-334 */
static void pml_pro(orc_ctx *c)
{
    int FW = c->P.fw, NXG = c->P.nx, NYG = c->P.ny;
    real DH = c->DH;
    const real alpha_max_PML = 2.0 * PI * (c->P.fpml / 2.0);
    real thickness_x = (real)FW * DH, thickness_y = (real)FW * DH;
    real Rcoef = 0.001;
    real NPOWER = c->P.npower, VPPML = c->P.vppml;
    real d0_x = -(NPOWER + 1) * VPPML * log(Rcoef) / (2.0 * thickness_x);
    real d0_y = -(NPOWER + 1) * VPPML * log(Rcoef) / (2.0 * thickness_y);
    real xoriginleft = thickness_x;
    real xoriginright = (NXG - 1) * DH - thickness_x;
    for (int i = 1; i <= FW; i++) {
        real xval = DH * (i - 1);
        real absc = xoriginleft - xval;
        real absch = xoriginleft - (xval + DH / 2.0);
        pml_point(c, d0_x, thickness_x, alpha_max_PML, 1, absc, absch, i, c->K_x, c->K_x_half, c->d_x,
                  c->d_x_half, c->alpha_prime_x, c->alpha_prime_x_half, c->b_x, c->b_x_half, c->a_x,
                  c->a_x_half);
    }
    for (int i = NXG - FW + 1; i <= NXG; i++) {
        int h = i - NXG + 2 * FW;
        real xval = DH * (i - 1);
        real absc = xval - xoriginright;
        real absch = xval + DH / 2.0 - xoriginright;
        pml_point(c, d0_x, thickness_x, alpha_max_PML, 1, absc, absch, h, c->K_x, c->K_x_half, c->d_x,
                  c->d_x_half, c->alpha_prime_x, c->alpha_prime_x_half, c->b_x, c->b_x_half, c->a_x,
                  c->a_x_half);
    }
    real yoriginbottom = thickness_y;
    real yorigintop = (NYG - 1) * DH - thickness_y;
    for (int i = 1; i <= FW; i++) {
        real yval = DH * (i - 1);
        real absc = yoriginbottom - yval;
        real absch = yoriginbottom - (yval + DH / 2.0);
        pml_point(c, d0_y, thickness_y, alpha_max_PML, 0, absc, absch, i, c->K_y, c->K_y_half, c->d_y,
                  c->d_y_half, c->alpha_prime_y, c->alpha_prime_y_half, c->b_y, c->b_y_half, c->a_y,
                  c->a_y_half);
    }
    for (int i = NYG - FW + 1; i <= NYG; i++) {
        int h = i - NYG + 2 * FW;
        real yval = DH * (i - 1);
        real absc = yval - yorigintop;
        real absch = yval + DH / 2.0 - yorigintop;
        pml_point(c, d0_y, thickness_y, alpha_max_PML, 0, absc, absch, h, c->K_y, c->K_y_half, c->d_y,
                  c->d_y_half, c->alpha_prime_y, c->alpha_prime_y_half, c->b_y, c->b_y_half, c->a_y,
                  c->a_y_half);
    }
}

/* absorb.c:34-121 (one rank) */
static void absorb(orc_ctx *c)
{
    int FW = c->P.fw, NX = c->P.nx, NY = c->P.ny, FS = c->P.free_surf, BND = c->P.boundary;
    real amp = 1.0 - c->P.damping / 100.0;
    real coeff[FW + 1];
    real a = sqrt(-log(amp) / ((FW - 1) * (FW - 1)));
    for (int i = 1; i <= FW; i++)
        coeff[i] = exp(-(a * a * (FW - i) * (FW - i)));
    for (int j = 1; j <= NY; j++)
        for (int i = 1; i <= NX; i++)
            A(c->absorb, j, i) = 1.0;
    if (!BND) {
        int yb = 1, ye = NY;
        for (int i = 1; i <= FW; i++) {
            if (!FS)
                yb = i;
            ye = NY - i + 1;
            for (int j = yb; j <= ye; j++)
                A(c->absorb, j, i) = coeff[i];
        }
        yb = 1, ye = NY;
        for (int i = 1; i <= FW; i++) {
            int ii = NX - i + 1;
            if (!FS)
                yb = i;
            ye = NY - i + 1;
            for (int j = yb; j <= ye; j++)
                A(c->absorb, j, ii) = coeff[i];
        }
    }
    if (!FS) {
        int xb = 1, xe = NX;
        for (int j = 1; j <= FW; j++) {
            if (!BND)
                xb = j;
            if (!BND)
                xe = NX - j + 1;
            for (int i = xb; i <= xe; i++)
                A(c->absorb, j, i) = coeff[j];
        }
    }
    {
        int xb = 1, xe = NX;
        for (int j = 1; j <= FW; j++) {
            int jj = NY - j + 1;
            if (!BND)
                xb = j;
            if (!BND)
                xe = NX - j + 1;
            for (int i = xb; i <= xe; i++)
                A(c->absorb, jj, i) = coeff[j];
        }
    }
}

/* The built-in models of readmod.c:60-83 (READMOD = 0): hh_elastic.c:31-71,
 * hh_visco.c:31-104, hh_elastic_VTI.c, hh_elastic_TTI.c (Bond transformation
 * at THETA = 0), hh_visco_VTI.c:31-107, hh_visco_TTI.c (THETA = 30). */
static int hh_model(orc_ctx *c)
{
    int weq = c->P.weq, L = c->P.L;
    real pts[ORC_MAX_L + 1], ws = 0;
    if (is_visco(weq))
        visco_pts(c, pts, &ws);
    if (weq == ORC_EL_ISO || weq == ORC_VEL_ISO) {
        const real vp1 = 0.0, vs1 = 1.0, rho1 = 1.0, tp1 = 0.01, ts1 = 0.01, h = 100.0;
        const real vp2 = 3500.0, vs2 = 2000.0, rho2 = 2000.0, tp2 = 0.01, ts2 = 0.01;
        const real h1 = 95.0, h2 = 110.0, tlp = 2.0, tls = 2.0;
        for (int i = 1; i <= c->P.nx; i++)
            for (int j = 1; j <= c->P.ny; j++) {
                real y = (real)j * c->DH, Vp, Vs, Rhov, tp, ts;
                if (y <= h)
                    Vp = vp1, Vs = vs1, Rhov = rho1, tp = tp1, ts = ts1;
                else
                    Vp = vp2, Vs = vs2, Rhov = rho2, tp = tp2, ts = ts2;
                if (weq == ORC_EL_ISO) {
                    A(c->pu, j, i) = Vs * Vs * Rhov;
                    A(c->ppi, j, i) = Vp * Vp * Rhov;
                } else {
                    if ((y >= h1) && (y <= h2))
                        tp = tlp, ts = tls;
                    real sumu = 0.0, sumpi = 0.0;
                    for (int l = 1; l <= L; l++) {
                        sumu = sumu + ((ws * ws * pts[l] * pts[l] * ts) / (1.0 + ws * ws * pts[l] * pts[l]));
                        sumpi = sumpi + ((ws * ws * pts[l] * pts[l] * tp) / (1.0 + ws * ws * pts[l] * pts[l]));
                    }
                    A(c->ptaus, j, i) = ts;
                    A(c->ptaup, j, i) = tp;
                    A(c->pu, j, i) = Vs * Vs * Rhov / (1.0 + sumu);
                    A(c->ppi, j, i) = Vp * Vp * Rhov / (1.0 + sumpi);
                }
                A(c->prho, j, i) = Rhov;
            }
        return 0;
    }
    if (is_iso(weq)) {
        snprintf(c->err, sizeof c->err, "Internal model for your chosen WEQ not implemented.");
        return 1;
    }
    /* Jones and Wang (1981) */
    const real C11 = 34.3e9, C33 = 22.7e9, C55 = 5.4e9, C13 = 10.7e9, RHO = 2000.0;
    real c11 = C11, c33 = C33, c55 = C55, c13 = C13, tau11 = 0, tau13 = 0, tau55 = 0;
    if (is_visco(weq)) {
        const real TAU = c->P.tau;
        real sumc11 = 0.0, sumc33 = 0.0, sumc55 = 0.0, sumc13 = 0.0;
        for (int l = 1; l <= L; l++) {
            sumc11 = sumc11 + ((ws * ws * pts[l] * pts[l] * TAU) / (1.0 + ws * ws * pts[l] * pts[l]));
            sumc33 = sumc33 + ((ws * ws * pts[l] * pts[l] * TAU) / (1.0 + ws * ws * pts[l] * pts[l]));
            sumc55 = sumc55 + ((ws * ws * pts[l] * pts[l] * TAU) / (1.0 + ws * ws * pts[l] * pts[l]));
        }
        c11 = c11 / (1.0 + sumc11);
        c33 = c33 / (1.0 + sumc33);
        c55 = c55 / (1.0 + sumc55);
        tau11 = TAU, tau55 = TAU;
        tau13 = (c11 * L * tau11 - 2.0 * c55 * L * tau55) / (c11 - 2.0 * c55);
        for (int l = 1; l <= L; l++)
            sumc13 = sumc13 + ((ws * ws * pts[l] * pts[l] * tau13) / (1.0 + ws * ws * pts[l] * pts[l]));
        c13 = c13 / (1.0 + sumc13);
    }
    real o[6] = {c11, c33, c13, c55, 0, 0};
    if (is_tti(weq))
        bond_tti(c11, c13, c33, c55, weq == ORC_VEL_TTI ? 30.0 : 0.0, o);
    for (int i = 1; i <= c->P.nx; i++)
        for (int j = 1; j <= c->P.ny; j++) {
            A(c->prho, j, i) = RHO;
            A(c->pc11, j, i) = o[0];
            A(c->pc33, j, i) = o[1];
            A(c->pc13, j, i) = o[2];
            A(c->pc55, j, i) = o[3];
            if (is_tti(weq)) {
                A(c->pc15, j, i) = o[4];
                A(c->pc35, j, i) = o[5];
            }
            if (is_visco(weq)) {
                A(c->ptau11, j, i) = tau11;
                A(c->ptau33, j, i) = tau11;
                A(c->ptau13, j, i) = tau13;
                A(c->ptau55, j, i) = tau55;
                if (is_tti(weq)) {
                    A(c->ptau15, j, i) = tau13;
                    A(c->ptau35, j, i) = tau13;
                }
            }
        }
    return 0;
}

int orc_prepare(orc_ctx *c)
{
    int weq = c->P.weq;
    if (!c->P.readmod) {
        if (hh_model(c))
            return 1;
        goto prepared_media;
    }
    if (!c->mat_vp || (!c->mat_vs && !is_ac(weq)) || !c->mat_rho) {
        snprintf(c->err, sizeof c->err, "vp/vs/rho missing");
        return 1;
    }
    if (is_visco(weq) && (!c->mat_qp || !c->mat_qs)) {
        snprintf(c->err, sizeof c->err, "qp/qs missing");
        return 1;
    }
    if (!is_iso(weq) && (!c->mat_eps || !c->mat_del || (is_tti(weq) && !c->mat_tet))) {
        snprintf(c->err, sizeof c->err, "anisotropy parameters missing");
        return 1;
    }
    if (weq == ORC_AC_ISO)
        readmod_acoustic(c);
    else if (weq == ORC_EL_ISO)
        readmod_elastic(c);
    else if (weq == ORC_VEL_ISO)
        readmod_visco(c);
    else
        readmod_aniso(c);
prepared_media:
    if (c->P.fw > 0 && c->P.abs_type == 1)
        pml_pro(c);
    if (c->P.fw > 0 && c->P.abs_type == 2)
        absorb(c);
    prepmod(c);
    c->prepared = 1;
    return 0;
}

/* ------------------------------------------------------------- wavelet */

/* wavelet.c:48-142 for one source k: `file` holds the samples of a
 * SOURCE_SHAPE 3 signal (read_srcsig.c), nfile of them. Float variables,
 * double constants and libm calls as the reference mixes them. */
static int wavelet_one(int shape, int nt, float dt, int nsrc, int k, const float *srcpos, const float *file,
                       int nfile, float *out)
{
    float tshift = srcpos[3 * nsrc + k];
    float fc = srcpos[4 * nsrc + k];
    float a = srcpos[5 * nsrc + k];
    float ts = 1.0 / fc;
    float sigmax = 0.0;
    for (int n = 1; n <= nt; n++) {
        float t = (float)n * dt;
        float amp = 0.0, tau;
        switch (shape) {
          case 1:
              tau = PI * (t - 1.5 * ts - tshift) / (ts);
              amp = (((1.0 - 2.0 * tau * tau) * exp(-tau * tau)));
              break;
          case 2:
              if ((t < tshift) || (t > (tshift + ts)))
                  amp = 0.0;
              else
                  amp = (sin(2.0 * PI * (t - tshift) * fc) - 0.5 * sin(4.0 * PI * (t - tshift) * fc));
              break;
          case 3: /* wavelet.c:70-75 */
              amp = n <= nfile ? file[n - 1] : 0.0;
              break;
          case 4:
              if ((t < tshift) || (t > (tshift + ts)))
                  amp = 0.0;
              else
                  amp = pow(sin(PI * (t - tshift) / ts), 3.0);
              break;
          case 5: { /* Berlage, wavelet.c:82-96: rows 9, 10, 11 */
              float ex = srcpos[8 * nsrc + k], alpha = srcpos[9 * nsrc + k];
              float phi0 = srcpos[10 * nsrc + k] * PI / 180;
              if (ex <= 0)
                  return 1;
              if (t < tshift)
                  amp = 0.0;
              else
                  amp = a * pow((t - tshift), ex) * exp(-alpha * (t - tshift)) * cos(2 * PI * fc * (t - tshift) + phi0);
              break;
          }
          case 6: { /* Klauder, wavelet.c:97-125: rows 9..12. The carrier
                     * exp(2 pi i fc t') goes through the real exp() of
                     * <math.h> (no <tgmath.h> in the reference), which takes
                     * the argument's real part, 0: the factor is 1. */
              float fmin = srcpos[8 * nsrc + k], fmax = srcpos[9 * nsrc + k];
              float T = srcpos[10 * nsrc + k], width = srcpos[11 * nsrc + k];
              float f2 = (fmax - fmin) / T, taper;
              tau = (width / fc);
              if ((t < tshift) || (t > (tau * 2) + tshift)) {
                  amp = 0.0;
              } else if (t < (tau * 0.2) + tshift) {
                  amp = sin(PI * f2 * (t - tau - tshift) * (T - (t - tau - tshift))) / (PI * f2 * (t - tau - tshift)) *
                        exp(0.0);
                  taper = (1 - cos(((t - tshift) / tau / 0.2) * PI)) / 2;
                  amp = amp * taper;
              } else if (t > (tau * 1.8) + tshift) {
                  amp = sin(PI * f2 * (t - tau - tshift) * (T - (t - tau - tshift))) / (PI * f2 * (t - tau - tshift)) *
                        exp(0.0);
                  taper = (1 - cos(((2 * tau + tshift - t) / 0.2 / tau) * PI)) / 2;
                  amp = amp * taper;
              } else {
                  amp = sin(PI * f2 * (t - tau - tshift) * (T - (t - tau - tshift))) / (PI * f2 * (t - tau - tshift)) *
                        exp(0.0);
              }
              break;
          }
          default:
              return 1;
        }
        if (fabs(amp) > sigmax)
            sigmax = fabs(amp);
        out[n - 1] = amp * a;
    }
    if (0.0 == sigmax) /* wavelet.c:135-136 */
        return 2;
    if (shape == 5 || shape == 6)
        for (int n = 1; n <= nt; n++)
            out[n - 1] = out[n - 1] / sigmax;
    return 0;
}

int orc_wavelet(int shape, int nt, float dt, int nsrc, const float *srcpos, float *out)
{
    /* wavelet.c:46-142; srcpos rows are 1-based in the reference: row r -> srcpos[(r-1)*nsrc + k] */
    if (shape == 3)
        return 1;
    for (int k = 0; k < nsrc; k++) {
        int rc = wavelet_one(shape, nt, dt, nsrc, k, srcpos, NULL, 0, out + (size_t)k * nt);
        if (rc)
            return rc;
    }
    return 0;
}

int orc_wavelet_samples(int nt, float dt, int nsrc, const float *srcpos, const float *samples, int ns, float *out)
{
    for (int k = 0; k < nsrc; k++) {
        int rc = wavelet_one(3, nt, dt, nsrc, k, srcpos, samples, ns, out + (size_t)k * nt);
        if (rc)
            return rc;
    }
    return 0;
}

int orc_set_sources(orc_ctx *c, int nsrc, const float *srcpos, const float *signals)
{
    free(c->srcpos);
    free(c->signals);
    c->nsrc = nsrc;
    c->srcpos = (float *)malloc(sizeof(float) * 12 * (size_t)(nsrc > 0 ? nsrc : 1));
    memcpy(c->srcpos, srcpos, sizeof(float) * 12 * (size_t)nsrc);
    c->signals = (real *)malloc(sizeof(real) * (size_t)(nsrc > 0 ? nsrc : 1) * (size_t)c->NT);
    for (size_t k = 0; k < (size_t)nsrc * (size_t)c->NT; k++)
        c->signals[k] = signals[k];
    return 0;
}

int orc_set_receivers(orc_ctx *c, int ntr, const int *ix, const int *iy)
{
    free(c->rx);
    free(c->ry);
    c->ntr = ntr;
    c->rx = (int *)malloc(sizeof(int) * (size_t)(ntr > 0 ? ntr : 1));
    c->ry = (int *)malloc(sizeof(int) * (size_t)(ntr > 0 ? ntr : 1));
    memcpy(c->rx, ix, sizeof(int) * (size_t)ntr);
    memcpy(c->ry, iy, sizeof(int) * (size_t)ntr);
    for (int k = 1; k <= 5; k++) {
        free(c->sec[k]);
        c->sec[k] = (float *)calloc((size_t)(ntr > 0 ? ntr : 1) * (size_t)(c->ns > 0 ? c->ns : 1), sizeof(float));
    }
    return 0;
}

#define SRC(row, l) (c->srcpos[(size_t)((row) - 1) * (size_t)c->nsrc + (size_t)((l) - 1)])
#define SIG(l, n) (c->signals[(size_t)((l) - 1) * (size_t)c->NT + (size_t)((n) - 1)])

/* ----------------------------------------------------------- operators */

/* op_v_fdN, initfd.c:97-183: stress derivatives for the velocity update (unscaled). */
static inline void op_v(orc_ctx *c, int i, int j, real *sxx_x, real *sxy_x, real *sxy_y, real *syy_y)
{
    const real *hc = c->hc;
    real a = 0, b = 0, d = 0, e = 0;
    for (int m = 1; m <= c->ND; m++) {
        real ta = hc[m] * (A(c->sxx, j, i + m) - A(c->sxx, j, i - m + 1));
        real tb = hc[m] * (A(c->sxy, j, i + m - 1) - A(c->sxy, j, i - m));
        real td = hc[m] * (A(c->sxy, j + m - 1, i) - A(c->sxy, j - m, i));
        real te = hc[m] * (A(c->syy, j + m, i) - A(c->syy, j - m + 1, i));
        if (m == 1) {
            a = ta, b = tb, d = td, e = te;
        } else {
            a += ta, b += tb, d += td, e += te;
        }
    }
    *sxx_x = a, *sxy_x = b, *sxy_y = d, *syy_y = e;
}

/* op_s_fdN, initfd.c:9-95: velocity derivatives, scaled by dhi = 1/DH (float). */
static inline void op_s(orc_ctx *c, real dhi, int i, int j, real *vxx, real *vyx, real *vxy, real *vyy)
{
    const real *hc = c->hc;
    real a = 0, b = 0, d = 0, e = 0;
    for (int m = 1; m <= c->ND; m++) {
        real ta = hc[m] * (A(c->vx, j, i + m - 1) - A(c->vx, j, i - m));
        real tb = hc[m] * (A(c->vy, j, i + m) - A(c->vy, j, i - m + 1));
        real td = hc[m] * (A(c->vx, j + m, i) - A(c->vx, j - m + 1, i));
        real te = hc[m] * (A(c->vy, j + m - 1, i) - A(c->vy, j - m, i));
        if (m == 1) {
            a = ta, b = tb, d = td, e = te;
        } else {
            a += ta, b += tb, d += td, e += te;
        }
    }
    *vxx = a * dhi, *vyx = b * dhi, *vxy = d * dhi, *vyy = e * dhi;
}

/* cpml_update.c:50-66 (h indexes the profile and the psi column/row) */
static inline void cpml_v_x(orc_ctx *c, int h, int j, real *sxx_x, real *sxy_x)
{
    real *ps = &PSIX(c->psi_sxx_x, j, h), *py = &PSIX(c->psi_sxy_x, j, h);
    *ps = c->b_x_half[h] * *ps + c->a_x_half[h] * (*sxx_x);
    *sxx_x = (*sxx_x) / c->K_x_half[h] + *ps;
    *py = c->b_x[h] * *py + c->a_x[h] * (*sxy_x);
    *sxy_x = (*sxy_x) / c->K_x[h] + *py;
}

static inline void cpml_v_y(orc_ctx *c, int i, int h, real *sxy_y, real *syy_y)
{
    real *ps = &PSIY(c->psi_syy_y, h, i), *py = &PSIY(c->psi_sxy_y, h, i);
    *ps = c->b_y_half[h] * *ps + c->a_y_half[h] * (*syy_y);
    *syy_y = (*syy_y) / c->K_y_half[h] + *ps;
    *py = c->b_y[h] * *py + c->a_y[h] * (*sxy_y);
    *sxy_y = (*sxy_y) / c->K_y[h] + *py;
}

/* cpml_update.c:30-46: in-place stretch of the stored velocity derivatives */
static inline void cpml_s_x(orc_ctx *c, int i, int j, int h1)
{
    real *p = &PSIX(c->psi_vxx, j, h1), *q = &PSIX(c->psi_vyx, j, h1);
    *p = c->b_x[h1] * *p + c->a_x[h1] * (A(c->vxx, j, i));
    A(c->vxx, j, i) = (A(c->vxx, j, i)) / c->K_x[h1] + *p;
    *q = c->b_x_half[h1] * *q + c->a_x_half[h1] * (A(c->vyx, j, i));
    A(c->vyx, j, i) = (A(c->vyx, j, i)) / c->K_x_half[h1] + *q;
}

static inline void cpml_s_y(orc_ctx *c, int i, int j, int h2)
{
    real *p = &PSIY(c->psi_vyy, h2, i), *q = &PSIY(c->psi_vxy, h2, i);
    *p = c->b_y[h2] * *p + c->a_y[h2] * (A(c->vyy, j, i));
    A(c->vyy, j, i) = (A(c->vyy, j, i)) / c->K_y[h2] + *p;
    *q = c->b_y_half[h2] * *q + c->a_y_half[h2] * (A(c->vxy, j, i));
    A(c->vxy, j, i) = (A(c->vxy, j, i)) / c->K_y_half[h2] + *q;
}

/* wavefield_update_v.c:46-47 */
static inline void wf_update_v(orc_ctx *c, int i, int j, real sxx_x, real sxy_x, real sxy_y, real syy_y)
{
    if (c->fwi) {
        /* wavefield_update_v.c:31-44 */
        if (!c->fwi_back) {
            A(c->pvxp1, j, i) = A(c->prip, j, i) * (sxx_x + sxy_y) / c->DH;
            A(c->pvyp1, j, i) = A(c->prjp, j, i) * (sxy_x + syy_y) / c->DH;
        } else if (c->fwi_vel == 0) {
            A(c->pvxp1, j, i) += A(c->vx, j, i) * c->DT;
            A(c->pvyp1, j, i) += A(c->vy, j, i) * c->DT;
        } else {
            A(c->pvxp1, j, i) = A(c->vx, j, i);
            A(c->pvyp1, j, i) = A(c->vy, j, i);
        }
    }
    A(c->vx, j, i) += (sxx_x + sxy_y) * c->DTDH * A(c->prip, j, i);
    A(c->vy, j, i) += (sxy_x + syy_y) * c->DTDH * A(c->prjp, j, i);
}

/* shift_var2 / shift_var3 (util.c:89-109): level 4 <- 3 <- 2 <- 1, the old
 * level 4 array becomes level 1 */
static void shift4(arr2 *h)
{
    arr2 t = h[4];
    h[4] = h[3], h[3] = h[2], h[2] = h[1], h[1] = t;
}

/* wavefield_update_v_4.c:26-46 */
static inline void wf_update_v4(orc_ctx *c, int i, int j, real sxx_x, real sxy_x, real sxy_y, real syy_y)
{
    A(c->svx[1], j, i) = sxx_x + sxy_y;
    A(c->svy[1], j, i) = sxy_x + syy_y;
    A(c->vx, j, i) += (AB1 * A(c->svx[1], j, i) + AB2 * A(c->svx[2], j, i) + AB3 * A(c->svx[3], j, i) +
                       AB4 * A(c->svx[4], j, i)) * c->DTDH * A(c->prip, j, i);
    A(c->vy, j, i) += (AB1 * A(c->svy[1], j, i) + AB2 * A(c->svy[2], j, i) + AB3 * A(c->svy[3], j, i) +
                       AB4 * A(c->svy[4], j, i)) * c->DTDH * A(c->prjp, j, i);
}

/* ------------------------------------------------------- velocity update */

/* update_v_interior.c:49-71: force sources before the velocity loop */
static void force_sources(orc_ctx *c, int nt)
{
    if (c->fwi_back) {
        /* update_v_interior.c:72-90: the time-reversed residuals at the
         * receivers, unscaled (ADJOINT_TYPE 1: x and y, 2: y, 3: x) */
        for (int l = 1; l <= c->ntr; l++) {
            int i = c->rx[l - 1], j = c->ry[l - 1];
            float sx = c->adj[((size_t)(l - 1)) * (size_t)c->NT + (size_t)(nt - 1)];
            float sy = c->adj[((size_t)(c->ntr + l - 1)) * (size_t)c->NT + (size_t)(nt - 1)];
            if (c->fwi_adj == 1 || c->fwi_adj == 3)
                A(c->vx, j, i) += sx;
            if (c->fwi_adj == 1 || c->fwi_adj == 2)
                A(c->vy, j, i) += sy;
        }
        return;
    }
    for (int l = 1; l <= c->nsrc; l++) {
        int i = (int)SRC(1, l), j = (int)SRC(2, l);
        real azi_rad = SRC(7, l) * PI / 180;
        real amp = (c->DT * SIG(l, nt)) / (c->DH * c->DH);
        int type = (int)SRC(8, l);
        switch (type) {
          case 2:
              A(c->vx, j, i) += A(c->prip, j, i) * amp;
              break;
          case 3:
              A(c->vy, j, i) += A(c->prjp, j, i) * amp;
              break;
          case 4:
              A(c->vx, j, i) += sin(azi_rad) * (A(c->prip, j, i) * amp);
              A(c->vy, j, i) += cos(azi_rad) * (A(c->prjp, j, i) * amp);
              break;
        }
    }
}

/* Velocity update of one region (update_v_interior.c:92-98, update_v_PML.c:41-140,
 * update_v_abs.c:37-120). mode: 0 interior, 1 CPML x, 2 CPML y, 3 CPML x+y, 4 damping. */
static void v_region(orc_ctx *c, int j0, int j1, int i0, int i1, int modex, int modey, int damp)
{
    int NX = c->P.nx, NY = c->P.ny, FW = c->P.fw;
#pragma omp parallel for schedule(static)
    for (int j = j0; j <= j1; j++)
        for (int i = i0; i <= i1; i++) {
            real sxx_x, sxy_x, sxy_y, syy_y;
            op_v(c, i, j, &sxx_x, &sxy_x, &sxy_y, &syy_y);
            if (modex == 1)
                cpml_v_x(c, i, j, &sxx_x, &sxy_x);
            else if (modex == 2)
                cpml_v_x(c, i - NX + 2 * FW, j, &sxx_x, &sxy_x);
            if (modey == 1)
                cpml_v_y(c, i, j, &sxy_y, &syy_y);
            else if (modey == 2)
                cpml_v_y(c, i, j - NY + 2 * FW, &sxy_y, &syy_y);
            wf_update_v(c, i, j, sxx_x, sxy_x, sxy_y, syy_y);
            if (damp) {
                A(c->vx, j, i) *= A(c->absorb, j, i); /* abs_update.c:46-50 */
                A(c->vy, j, i) *= A(c->absorb, j, i);
            }
        }
}

/* The FDORDER_TIME = 4 drivers (update_v_interior_4.c, update_v_PML_4.c,
 * update_v_abs_4.c). upd = 0: the region gets its CPML pass but no update --
 * update_v_PML_4.c leaves the velocity of the left frame and of all four
 * corners untouched. */
static void v_region4(orc_ctx *c, int j0, int j1, int i0, int i1, int modex, int modey, int damp, int upd)
{
    int NX = c->P.nx, NY = c->P.ny, FW = c->P.fw;
#pragma omp parallel for schedule(static)
    for (int j = j0; j <= j1; j++)
        for (int i = i0; i <= i1; i++) {
            real sxx_x, sxy_x, sxy_y, syy_y;
            op_v(c, i, j, &sxx_x, &sxy_x, &sxy_y, &syy_y);
            if (modex == 1)
                cpml_v_x(c, i, j, &sxx_x, &sxy_x);
            else if (modex == 2)
                cpml_v_x(c, i - NX + 2 * FW, j, &sxx_x, &sxy_x);
            if (modey == 1)
                cpml_v_y(c, i, j, &sxy_y, &syy_y);
            else if (modey == 2)
                cpml_v_y(c, i, j - NY + 2 * FW, &sxy_y, &syy_y);
            if (upd)
                wf_update_v4(c, i, j, sxx_x, sxy_x, sxy_y, syy_y);
            if (damp) {
                A(c->vx, j, i) *= A(c->absorb, j, i); /* abs_update.c:46-50 */
                A(c->vy, j, i) *= A(c->absorb, j, i);
            }
        }
}

static void update_v4(orc_ctx *c)
{
    int *GX = c->GX, *GY = c->GY;
    v_region4(c, GY[2] + 1, GY[3], GX[2] + 1, GX[3], 0, 0, 0, 1);
    if (c->P.fw && (c->P.abs_type == 1 || c->P.abs_type == 2)) {
        int pml = c->P.abs_type == 1, dmp = c->P.abs_type == 2;
        v_region4(c, GY[2] + 1, GY[3], GX[1], GX[2], pml ? 1 : 0, 0, dmp, dmp);
        v_region4(c, GY[2] + 1, GY[3], GX[3] + 1, GX[4], pml ? 2 : 0, 0, dmp, 1);
        v_region4(c, GY[1], GY[2], GX[2] + 1, GX[3], 0, pml ? 1 : 0, dmp, 1);
        v_region4(c, GY[3] + 1, GY[4], GX[2] + 1, GX[3], 0, pml ? 2 : 0, dmp, 1);
        v_region4(c, GY[1], GY[2], GX[1], GX[2], pml ? 1 : 0, pml ? 1 : 0, dmp, dmp);
        v_region4(c, GY[3] + 1, GY[4], GX[1], GX[2], pml ? 1 : 0, pml ? 2 : 0, dmp, dmp);
        v_region4(c, GY[1], GY[2], GX[3] + 1, GX[4], pml ? 2 : 0, pml ? 1 : 0, dmp, dmp);
        v_region4(c, GY[3] + 1, GY[4], GX[3] + 1, GX[4], pml ? 2 : 0, pml ? 2 : 0, dmp, dmp);
    }
    /* time_loop.c:89-91 */
    shift4(c->svx);
    shift4(c->svy);
}

static void update_v(orc_ctx *c, int nt)
{
    int *GX = c->GX, *GY = c->GY;
    force_sources(c, nt);
    if (c->ab4) {
        update_v4(c);
        return;
    }
    v_region(c, GY[2] + 1, GY[3], GX[2] + 1, GX[3], 0, 0, 0);
    if (c->P.fw) {
        int pml = c->P.abs_type == 1, dmp = c->P.abs_type == 2;
        if (!pml && !dmp)
            return;
        /* order: left, right, top, bottom, left-top, left-bottom, right-top, right-bottom */
        v_region(c, GY[2] + 1, GY[3], GX[1], GX[2], pml ? 1 : 0, 0, dmp);
        v_region(c, GY[2] + 1, GY[3], GX[3] + 1, GX[4], pml ? 2 : 0, 0, dmp);
        v_region(c, GY[1], GY[2], GX[2] + 1, GX[3], 0, pml ? 1 : 0, dmp);
        v_region(c, GY[3] + 1, GY[4], GX[2] + 1, GX[3], 0, pml ? 2 : 0, dmp);
        v_region(c, GY[1], GY[2], GX[1], GX[2], pml ? 1 : 0, pml ? 1 : 0, dmp);
        v_region(c, GY[3] + 1, GY[4], GX[1], GX[2], pml ? 1 : 0, pml ? 2 : 0, dmp);
        v_region(c, GY[1], GY[2], GX[3] + 1, GX[4], pml ? 2 : 0, pml ? 1 : 0, dmp);
        v_region(c, GY[3] + 1, GY[4], GX[3] + 1, GX[4], pml ? 2 : 0, pml ? 2 : 0, dmp);
    }
}

/* exchange_v.c:88-148 with BOUNDARY = 1 and one rank: a pair (a = "vx", b = "vy")
 * gets its ghost columns from the opposite edge. */
static void exchange_pair_periodic(orc_ctx *c, arr2 ax, arr2 ay)
{
    int NX = c->P.nx, ND = c->ND;
    for (int j = 1; j <= c->P.ny; j++) {
        real bl[16], br[16];
        int n = 0;
        for (int l = 1; l <= ND; l++) bl[n++] = A(ay, j, l);
        for (int l = 1; l <= ND - 1; l++) bl[n++] = A(ax, j, l);
        n = 0;
        for (int l = 1; l <= ND - 1; l++) br[n++] = A(ay, j, NX - l + 1);
        for (int l = 1; l <= ND; l++) br[n++] = A(ax, j, NX - l + 1);
        n = 0;
        for (int l = 1; l <= ND; l++) A(ay, j, NX + l) = bl[n++];
        for (int l = 1; l <= ND - 1; l++) A(ax, j, NX + l) = bl[n++];
        n = 0;
        for (int l = 1; l <= ND - 1; l++) A(ay, j, 1 - l) = br[n++];
        for (int l = 1; l <= ND; l++) A(ax, j, 1 - l) = br[n++];
    }
}

/* exchange_s.c:79-121 with BOUNDARY = 1 and one rank */
static void exchange_s_periodic(orc_ctx *c)
{
    int NX = c->P.nx, ND = c->ND;
    for (int j = 1; j <= c->P.ny; j++) {
        real bl[16], br[16];
        int n = 0;
        for (int l = 1; l <= ND - 1; l++) bl[n++] = A(c->sxy, j, l);
        for (int l = 1; l <= ND; l++) bl[n++] = A(c->sxx, j, l);
        n = 0;
        for (int l = 1; l <= ND; l++) br[n++] = A(c->sxy, j, NX - l + 1);
        for (int l = 1; l <= ND - 1; l++) br[n++] = A(c->sxx, j, NX - l + 1);
        n = 0;
        for (int l = 1; l <= ND - 1; l++) A(c->sxy, j, NX + l) = bl[n++];
        for (int l = 1; l <= ND; l++) A(c->sxx, j, NX + l) = bl[n++];
        n = 0;
        for (int l = 1; l <= ND; l++) A(c->sxy, j, 1 - l) = br[n++];
        for (int l = 1; l <= ND - 1; l++) A(c->sxx, j, 1 - l) = br[n++];
    }
}

/* v_derivatives.c:27-50 (full grid) */
static void v_derivatives(orc_ctx *c)
{
    real dhi = 1.f / c->DH; /* initfd.c:302 */
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++) {
            real vxx, vyx, vxy, vyy;
            op_s(c, dhi, i, j, &vxx, &vyx, &vxy, &vyy);
            A(c->vxx, j, i) = vxx;
            A(c->vyy, j, i) = vyy;
            A(c->vyx, j, i) = vyx;
            A(c->vxy, j, i) = vxy;
        }
}

/* --------------------------------------------------------- stress update */

/* wavefield_update_s_el.c:28-48 */
static inline void wf_s_el(orc_ctx *c, int i, int j)
{
    real vxx = A(c->vxx, j, i), vyy = A(c->vyy, j, i), vyx = A(c->vyx, j, i), vxy = A(c->vxy, j, i);
    real u1 = A(c->fipjp, j, i) * (vyx + vxy);
    real u2 = (A(c->g, j, i) * (vxx + vyy)) - (2.0 * A(c->f, j, i) * vyy);
    real u3 = (A(c->g, j, i) * (vxx + vyy)) - (2.0 * A(c->f, j, i) * vxx);
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
    if (c->fwi) { /* wavefield_update_s_el.c:43-47 */
        A(c->uxy, j, i) = u1 / c->DT;
        A(c->ux, j, i) = u2 / c->DT;
        A(c->uy, j, i) = u3 / c->DT;
    }
}

/* wavefield_update_s_visc.c:27-68 */
static inline void wf_s_visc(orc_ctx *c, int i, int j)
{
    real dthalbe = c->DT / 2.0;
    real sumr_old = 0.0f, sump_old = 0.0f, sumq_old = 0.0f, sumr = 0.0f, sump = 0.0f, sumq = 0.0f;
    real vxx = A(c->vxx, j, i), vyy = A(c->vyy, j, i), vyx = A(c->vyx, j, i), vxy = A(c->vxy, j, i);
    for (int l = 1; l <= c->P.L; l++) {
        real *r = &A(c->pr[l], j, i), *p = &A(c->pp[l], j, i), *q = &A(c->pq[l], j, i);
        sumr_old += *r;
        sump_old += *p;
        sumq_old += *q;
        *r = c->bip[l] * (*r * c->cip[l] - (A(c->dip[l], j, i) * (vxy + vyx)));
        *p = c->bip[l] * (*p * c->cip[l] - (A(c->e[l], j, i) * (vxx + vyy)) + (2.0 * A(c->d[l], j, i) * vyy));
        *q = c->bip[l] * (*q * c->cip[l] - (A(c->e[l], j, i) * (vxx + vyy)) + (2.0 * A(c->d[l], j, i) * vxx));
        sumr += *r;
        sump += *p;
        sumq += *q;
    }
    real u1 = (A(c->fipjp, j, i) * (vxy + vyx)) + (dthalbe * (sumr_old + sumr));
    real u2 = (A(c->g, j, i) * (vxx + vyy)) - (2.0 * A(c->f, j, i) * vyy) + (dthalbe * (sump_old + sump));
    real u3 = (A(c->g, j, i) * (vxx + vyy)) - (2.0 * A(c->f, j, i) * vxx) + (dthalbe * (sumq_old + sumq));
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

/* wavefield_update_s_el_vti.c:27-47 */
static inline void wf_s_el_vti(orc_ctx *c, int i, int j)
{
    real vxx = A(c->vxx, j, i), vyy = A(c->vyy, j, i), vyx = A(c->vyx, j, i), vxy = A(c->vxy, j, i);
    real u1 = (A(c->pc55ipjp, j, i) * (vxy + vyx));
    real u2 = ((A(c->pc11, j, i) * vxx) + (A(c->pc13, j, i) * vyy));
    real u3 = ((A(c->pc13, j, i) * vxx) + (A(c->pc33, j, i) * vyy));
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

/* wavefield_update_s_visc_VTI.c:27-66 */
static inline void wf_s_visc_vti(orc_ctx *c, int i, int j)
{
    real dthalbe = c->DT / 2.0;
    real sumr_old = 0.0f, sump_old = 0.0f, sumq_old = 0.0f, sumr = 0.0f, sump = 0.0f, sumq = 0.0f;
    real vxx = A(c->vxx, j, i), vyy = A(c->vyy, j, i), vyx = A(c->vyx, j, i), vxy = A(c->vxy, j, i);
    for (int l = 1; l <= c->P.L; l++) {
        real *r = &A(c->pr[l], j, i), *p = &A(c->pp[l], j, i), *q = &A(c->pq[l], j, i);
        sumr_old += *r;
        sump_old += *p;
        sumq_old += *q;
        *r = c->bip[l] * (*r * c->cip[l] - (A(c->pc55ipjpd[l], j, i) * (vxy + vyx)));
        *p = c->bip[l] * (*p * c->cip[l] - (A(c->pc11d[l], j, i) * vxx) - (A(c->pc13d[l], j, i) * vyy));
        *q = c->bip[l] * (*q * c->cip[l] - (A(c->pc13d[l], j, i) * vxx) - (A(c->pc33d[l], j, i) * vyy));
        sumr += *r;
        sump += *p;
        sumq += *q;
    }
    real u1 = (A(c->pc55ipjpu, j, i) * (vxy + vyx)) + (dthalbe * (sumr_old + sumr));
    real u2 = (A(c->pc11u, j, i) * vxx) + (A(c->pc13u, j, i) * vyy) + (dthalbe * (sump_old + sump));
    real u3 = (A(c->pc13u, j, i) * vxx) + (A(c->pc33u, j, i) * vyy) + (dthalbe * (sumq_old + sumq));
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

/* wavefield_update_s_el_tti.c:27-52 */
static inline void wf_s_el_tti(orc_ctx *c, int i, int j)
{
    real vxxipjp = 0.25 * (A(c->vxx, j, i) + A(c->vxx, j + 1, i) + A(c->vxx, j, i + 1) + A(c->vxx, j + 1, i + 1));
    real vyyipjp = 0.25 * (A(c->vyy, j, i) + A(c->vyy, j + 1, i) + A(c->vyy, j, i + 1) + A(c->vyy, j + 1, i + 1));
    real vij = (0.25 * (A(c->vyx, j, i) + A(c->vyx, j - 1, i) + A(c->vyx, j, i - 1) + A(c->vyx, j - 1, i - 1))) +
               (0.25 * (A(c->vxy, j, i) + A(c->vxy, j - 1, i) + A(c->vxy, j, i - 1) + A(c->vxy, j - 1, i - 1)));
    real v = A(c->vxy, j, i) + A(c->vyx, j, i);
    real u1 = ((A(c->pc55ipjp, j, i) * v) + (A(c->pc15ipjp, j, i) * vxxipjp) + (A(c->pc35ipjp, j, i) * vyyipjp));
    real u2 = ((A(c->pc11, j, i) * A(c->vxx, j, i)) + (A(c->pc13, j, i) * A(c->vyy, j, i)) + (A(c->pc15, j, i) * vij));
    real u3 = ((A(c->pc13, j, i) * A(c->vxx, j, i)) + (A(c->pc33, j, i) * A(c->vyy, j, i)) + (A(c->pc35, j, i) * vij));
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

/* wavefield_update_s_visc_TTI.c:27-84 */
static inline void wf_s_visc_tti(orc_ctx *c, int i, int j)
{
    real dthalbe = c->DT / 2.0;
    real sumr_old = 0.0f, sump_old = 0.0f, sumq_old = 0.0f, sumr = 0.0f, sump = 0.0f, sumq = 0.0f;
    real vxxipjp, vyyipjp, vyxij, vxyij, vij, v;
    vxxipjp = 0.25 * (A(c->vxx, j, i) + A(c->vxx, j + 1, i) + A(c->vxx, j, i + 1) + A(c->vxx, j + 1, i + 1));
    vyyipjp = 0.25 * (A(c->vyy, j, i) + A(c->vyy, j + 1, i) + A(c->vyy, j, i + 1) + A(c->vyy, j + 1, i + 1));
    vyxij = 0.25 * (A(c->vyx, j, i) + A(c->vyx, j - 1, i) + A(c->vyx, j, i - 1) + A(c->vyx, j - 1, i - 1));
    vxyij = 0.25 * (A(c->vxy, j, i) + A(c->vxy, j - 1, i) + A(c->vxy, j, i - 1) + A(c->vxy, j - 1, i - 1));
    vij = vyxij + vxyij;
    v = A(c->vxy, j, i) + A(c->vyx, j, i);
    real vxx = A(c->vxx, j, i), vyy = A(c->vyy, j, i);
    for (int l = 1; l <= c->P.L; l++) {
        real *r = &A(c->pr[l], j, i), *p = &A(c->pp[l], j, i), *q = &A(c->pq[l], j, i);
        sumr_old += *r;
        sump_old += *p;
        sumq_old += *q;
        *r = c->bip[l] * (*r * c->cip[l] - (A(c->pc55ipjpd[l], j, i) * v) - (A(c->pc15ipjpd[l], j, i) * vxxipjp) -
                          (A(c->pc35ipjpd[l], j, i) * vyyipjp));
        *p = c->bip[l] * (*p * c->cip[l] - (A(c->pc11d[l], j, i) * vxx) - (A(c->pc13d[l], j, i) * vyy) -
                          (A(c->pc15d[l], j, i) * vij));
        *q = c->bip[l] * (*q * c->cip[l] - (A(c->pc13d[l], j, i) * vxx) - (A(c->pc33d[l], j, i) * vyy) -
                          (A(c->pc35d[l], j, i) * vij));
        sumr += *r;
        sump += *p;
        sumq += *q;
    }
    real u1 = (A(c->pc55ipjpu, j, i) * v) + (A(c->pc15ipjpu, j, i) * vxxipjp) + (A(c->pc35ipjpu, j, i) * vyyipjp) +
              (dthalbe * (sumr_old + sumr));
    real u2 = (A(c->pc11u, j, i) * vxx) + (A(c->pc13u, j, i) * vyy) + +(A(c->pc15u, j, i) * vij) +
              (dthalbe * (sump_old + sump));
    real u3 = (A(c->pc13u, j, i) * vxx) + (A(c->pc33u, j, i) * vyy) + (A(c->pc35u, j, i) * vij) +
              (dthalbe * (sumq_old + sumq));
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

/* wavefield_update_s_ac.c:27-33: sxx and syy are one array, so the pressure
 * gets g*vxx and then g*vyy */
static inline void wf_s_ac(orc_ctx *c, int i, int j)
{
    A(c->sxx, j, i) += (A(c->g, j, i) * A(c->vxx, j, i));
    A(c->syy, j, i) += (A(c->g, j, i) * A(c->vyy, j, i));
}

/* wavefield_update_s_el_4.c:26-60 (the stored derivatives times DH, their
 * Adams-Bashforth sums, the update scaled back by dhi) */
static inline void wf_s_el4(orc_ctx *c, int i, int j)
{
    real dhi = 1.0 / c->DH;
    A(c->hxx[1], j, i) = A(c->vxx, j, i) * c->DH;
    A(c->hyy[1], j, i) = A(c->vyy, j, i) * c->DH;
    A(c->hxy[1], j, i) = A(c->vxy, j, i) * c->DH;
    A(c->hyx[1], j, i) = A(c->vyx, j, i) * c->DH;
    real sumxx = AB1 * A(c->hxx[1], j, i) + AB2 * A(c->hxx[2], j, i) + AB3 * A(c->hxx[3], j, i) + AB4 * A(c->hxx[4], j, i);
    real sumyy = AB1 * A(c->hyy[1], j, i) + AB2 * A(c->hyy[2], j, i) + AB3 * A(c->hyy[3], j, i) + AB4 * A(c->hyy[4], j, i);
    real sumxy = AB1 * A(c->hxy[1], j, i) + AB2 * A(c->hxy[2], j, i) + AB3 * A(c->hxy[3], j, i) + AB4 * A(c->hxy[4], j, i);
    real sumyx = AB1 * A(c->hyx[1], j, i) + AB2 * A(c->hyx[2], j, i) + AB3 * A(c->hyx[3], j, i) + AB4 * A(c->hyx[4], j, i);
    real u1 = A(c->fipjp, j, i) * (sumxy + sumyx) * dhi;
    real u2 = ((A(c->g, j, i) * (sumxx + sumyy)) - (2.0 * A(c->f, j, i) * sumyy)) * dhi;
    real u3 = ((A(c->g, j, i) * (sumxx + sumyy)) - (2.0 * A(c->f, j, i) * sumxx)) * dhi;
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

/* wavefield_update_s_visc_4.c:27-91: memory variables of level 4 are
 * overwritten with the new values (they become level 1 after the shift) */
static inline void wf_s_visc4(orc_ctx *c, int i, int j)
{
    real sumr_old = 0.0f, sump_old = 0.0f, sumq_old = 0.0f, sumr = 0.0f, sump = 0.0f, sumq = 0.0f;
    real dhi = 1.0 / c->DH;
    real dthalbe = c->DT / 2.0;
    A(c->hxx[1], j, i) = A(c->vxx, j, i) * c->DH;
    A(c->hyy[1], j, i) = A(c->vyy, j, i) * c->DH;
    A(c->hxy[1], j, i) = A(c->vxy, j, i) * c->DH;
    A(c->hyx[1], j, i) = A(c->vyx, j, i) * c->DH;
    real sumxx = AB1 * A(c->hxx[1], j, i) + AB2 * A(c->hxx[2], j, i) + AB3 * A(c->hxx[3], j, i) + AB4 * A(c->hxx[4], j, i);
    real sumyy = AB1 * A(c->hyy[1], j, i) + AB2 * A(c->hyy[2], j, i) + AB3 * A(c->hyy[3], j, i) + AB4 * A(c->hyy[4], j, i);
    real sumxy = AB1 * A(c->hxy[1], j, i) + AB2 * A(c->hxy[2], j, i) + AB3 * A(c->hxy[3], j, i) + AB4 * A(c->hxy[4], j, i);
    real sumyx = AB1 * A(c->hyx[1], j, i) + AB2 * A(c->hyx[2], j, i) + AB3 * A(c->hyx[3], j, i) + AB4 * A(c->hyx[4], j, i);
    for (int l = 1; l <= c->P.L; l++) {
        real r = A(c->pr[l], j, i), r2 = A(c->pr_h[2][l], j, i), r3 = A(c->pr_h[3][l], j, i), r4 = A(c->pr_h[4][l], j, i);
        real p = A(c->pp[l], j, i), p2 = A(c->pp_h[2][l], j, i), p3 = A(c->pp_h[3][l], j, i), p4 = A(c->pp_h[4][l], j, i);
        real q = A(c->pq[l], j, i), q2 = A(c->pq_h[2][l], j, i), q3 = A(c->pq_h[3][l], j, i), q4 = A(c->pq_h[4][l], j, i);
        sumr_old += AB1 * r + AB2 * r2 + AB3 * r3 + AB4 * r4;
        sump_old += AB1 * p + AB2 * p2 + AB3 * p3 + AB4 * p4;
        sumq_old += AB1 * q + AB2 * q2 + AB3 * q3 + AB4 * q4;
        real ctemp = 2 * (1 - c->cip[l]) / AB1;
        real nr = c->bip[l] * (r * c->cip[l] - ctemp * AB2 * (r + r2) - ctemp * AB3 * (r2 + r3) -
                               ctemp * AB4 * (r3 + r4) - (A(c->dip[l], j, i) * (sumxy + sumyx) * dhi));
        real np = c->bip[l] * (p * c->cip[l] - ctemp * AB2 * (p + p2) - ctemp * AB3 * (p2 + p3) -
                               ctemp * AB4 * (p3 + p4) - (A(c->e[l], j, i) * (sumxx + sumyy) * dhi) +
                               (2.0 * A(c->d[l], j, i) * sumyy * dhi));
        real nq = c->bip[l] * (q * c->cip[l] - ctemp * AB2 * (q + q2) - ctemp * AB3 * (q2 + q3) -
                               ctemp * AB4 * (q3 + q4) - (A(c->e[l], j, i) * (sumxx + sumyy) * dhi) +
                               (2.0 * A(c->d[l], j, i) * sumxx * dhi));
        A(c->pr_h[4][l], j, i) = nr;
        A(c->pp_h[4][l], j, i) = np;
        A(c->pq_h[4][l], j, i) = nq;
        sumr += AB1 * nr + AB2 * r + AB3 * r2 + AB4 * r3;
        sump += AB1 * np + AB2 * p + AB3 * p2 + AB4 * p3;
        sumq += AB1 * nq + AB2 * q + AB3 * q2 + AB4 * q3;
    }
    real u1 = (A(c->fipjp, j, i) * (sumxy + sumyx)) * dhi + (dthalbe * (sumr_old + sumr));
    real u2 = (A(c->g, j, i) * (sumxx + sumyy) * dhi) - (2.0 * A(c->f, j, i) * sumyy * dhi) +
              (dthalbe * (sump_old + sump));
    real u3 = (A(c->g, j, i) * (sumxx + sumyy) * dhi) - (2.0 * A(c->f, j, i) * sumxx * dhi) +
              (dthalbe * (sumq_old + sumq));
    A(c->sxy, j, i) += u1;
    A(c->sxx, j, i) += u2;
    A(c->syy, j, i) += u3;
}

static inline void wf_s(orc_ctx *c, int i, int j)
{
    if (c->ab4) {
        if (c->P.weq == ORC_VEL_ISO)
            wf_s_visc4(c, i, j);
        else
            wf_s_el4(c, i, j);
        return;
    }
    switch (c->P.weq) {
      case ORC_AC_ISO: wf_s_ac(c, i, j); break;
      case ORC_EL_ISO: wf_s_el(c, i, j); break;
      case ORC_VEL_ISO: wf_s_visc(c, i, j); break;
      case ORC_EL_VTI: wf_s_el_vti(c, i, j); break;
      case ORC_VEL_VTI: wf_s_visc_vti(c, i, j); break;
      case ORC_EL_TTI: wf_s_el_tti(c, i, j); break;
      case ORC_VEL_TTI: wf_s_visc_tti(c, i, j); break;
    }
}

/* CPML pass over one region (cpml_update_s_x/_y with the driver's h1/h2 rules) */
static void s_cpml_region(orc_ctx *c, int j0, int j1, int i0, int i1, int modex, int modey)
{
    int NX = c->P.nx, NY = c->P.ny, FW = c->P.fw;
#pragma omp parallel for schedule(static)
    for (int j = j0; j <= j1; j++)
        for (int i = i0; i <= i1; i++) {
            if (modex == 1) cpml_s_x(c, i, j, i);
            else if (modex == 2) cpml_s_x(c, i, j, i - NX + 2 * FW);
            if (modey == 1) cpml_s_y(c, i, j, j);
            else if (modey == 2) cpml_s_y(c, i, j, j - NY + 2 * FW);
        }
}

/* Stress update of one region; cpml applied cell by cell (non-TTI drivers,
 * e.g. update_s_elastic_PML.c:41-120) or not at all; damp = abs_update_s. */
static void s_region(orc_ctx *c, int j0, int j1, int i0, int i1, int modex, int modey, int damp)
{
    int NX = c->P.nx, NY = c->P.ny, FW = c->P.fw;
#pragma omp parallel for schedule(static)
    for (int j = j0; j <= j1; j++)
        for (int i = i0; i <= i1; i++) {
            if (modex == 1) cpml_s_x(c, i, j, i);
            else if (modex == 2) cpml_s_x(c, i, j, i - NX + 2 * FW);
            if (modey == 1) cpml_s_y(c, i, j, j);
            else if (modey == 2) cpml_s_y(c, i, j, j - NY + 2 * FW);
            wf_s(c, i, j);
            if (damp && is_ac(c->P.weq)) { /* abs_update.c:28-31 (abs_update_s_ac2): once */
                A(c->sxx, j, i) *= A(c->absorb, j, i);
            } else if (damp) { /* abs_update.c:39-44 */
                A(c->sxy, j, i) *= A(c->absorb, j, i);
                A(c->syy, j, i) *= A(c->absorb, j, i);
                A(c->sxx, j, i) *= A(c->absorb, j, i);
            }
        }
}

static void update_s_regions(orc_ctx *c);

static void update_s(orc_ctx *c)
{
    update_s_regions(c);
    if (c->ab4) {
        /* time_loop.c:228-230, 241-244 */
        for (int l = 1; l <= c->P.L; l++) {
            arr2 hr[5] = {{0}, c->pr[l], c->pr_h[2][l], c->pr_h[3][l], c->pr_h[4][l]};
            arr2 hp[5] = {{0}, c->pp[l], c->pp_h[2][l], c->pp_h[3][l], c->pp_h[4][l]};
            arr2 hq[5] = {{0}, c->pq[l], c->pq_h[2][l], c->pq_h[3][l], c->pq_h[4][l]};
            shift4(hr), shift4(hp), shift4(hq);
            c->pr[l] = hr[1], c->pr_h[2][l] = hr[2], c->pr_h[3][l] = hr[3], c->pr_h[4][l] = hr[4];
            c->pp[l] = hp[1], c->pp_h[2][l] = hp[2], c->pp_h[3][l] = hp[3], c->pp_h[4][l] = hp[4];
            c->pq[l] = hq[1], c->pq_h[2][l] = hq[2], c->pq_h[3][l] = hq[3], c->pq_h[4][l] = hq[4];
        }
        shift4(c->hxx), shift4(c->hyy), shift4(c->hxy), shift4(c->hyx);
    }
}

static void update_s_regions(orc_ctx *c)
{
    int *GX = c->GX, *GY = c->GY;
    s_region(c, GY[2] + 1, GY[3], GX[2] + 1, GX[3], 0, 0, 0);
    if (!c->P.fw || (c->P.abs_type != 1 && c->P.abs_type != 2))
        return;
    int pml = c->P.abs_type == 1, dmp = c->P.abs_type == 2;
    if (pml && is_tti(c->P.weq)) {
        /* update_s_elastic_TTI_PML.c:36-144 / update_s_visc_TTI_PML.c: per region a
         * CPML pass over the whole region, then the update without the outer 2 cells */
        int rb = (c->P.weq == ORC_EL_TTI) ? GY[4] - 1 : GY[4];
        s_cpml_region(c, GY[2] + 1, GY[3], GX[1], GX[2], 1, 0);
        s_region(c, GY[2] + 1, GY[3], GX[1] + 2, GX[2], 0, 0, 0);
        s_cpml_region(c, GY[2] + 1, GY[3], GX[3] + 1, GX[4], 2, 0);
        s_region(c, GY[2] + 1, GY[3], GX[3] + 1, GX[4] - 2, 0, 0, 0);
        s_cpml_region(c, GY[1], GY[2], GX[2] + 1, GX[3], 0, 1);
        s_region(c, GY[1] + 2, GY[2], GX[2] + 1, GX[3], 0, 0, 0);
        s_cpml_region(c, GY[3] + 1, GY[4], GX[2] + 1, GX[3], 0, 2);
        s_region(c, GY[3] + 1, GY[4] - 2, GX[2] + 1, GX[3], 0, 0, 0);
        s_cpml_region(c, GY[1], GY[2], GX[1], GX[2], 1, 1);
        s_region(c, GY[1] + 2, GY[2], GX[1] + 2, GX[2], 0, 0, 0);
        s_cpml_region(c, GY[3] + 1, GY[4], GX[1], GX[2], 1, 2);
        s_region(c, GY[3] + 1, GY[4] - 2, GX[1] + 2, GX[2], 0, 0, 0);
        s_cpml_region(c, GY[1], GY[2], GX[3] + 1, GX[4], 2, 1);
        s_region(c, GY[1] + 2, GY[2], GX[3] + 1, GX[4] - 2, 0, 0, 0);
        s_cpml_region(c, GY[3] + 1, rb, GX[3] + 1, GX[4], 2, 2);
        s_region(c, GY[3] + 1, GY[4] - 2, GX[3] + 1, GX[4] - 2, 0, 0, 0);
        return;
    }
    s_region(c, GY[2] + 1, GY[3], GX[1], GX[2], pml ? 1 : 0, 0, dmp);
    s_region(c, GY[2] + 1, GY[3], GX[3] + 1, GX[4], pml ? 2 : 0, 0, dmp);
    s_region(c, GY[1], GY[2], GX[2] + 1, GX[3], 0, pml ? 1 : 0, dmp);
    s_region(c, GY[3] + 1, GY[4], GX[2] + 1, GX[3], 0, pml ? 2 : 0, dmp);
    s_region(c, GY[1], GY[2], GX[1], GX[2], pml ? 1 : 0, pml ? 1 : 0, dmp);
    s_region(c, GY[3] + 1, GY[4], GX[1], GX[2], pml ? 1 : 0, pml ? 2 : 0, dmp);
    s_region(c, GY[1], GY[2], GX[3] + 1, GX[4], pml ? 2 : 0, pml ? 1 : 0, dmp);
    s_region(c, GY[3] + 1, GY[4], GX[3] + 1, GX[4], pml ? 2 : 0, pml ? 2 : 0, dmp);
}

/* Type that time_loop.c:248-253 tests: gv->SOURCE_TYPE, which
 * update_v_interior.c:57 overwrites with each source's type in turn, so after
 * the velocity update it holds the last source's type. */
static int last_source_type(orc_ctx *c)
{
    return c->nsrc > 0 ? (int)SRC(8, c->nsrc) : 0;
}

/* psource.c:27-54 (explosive; applied to every source) */
static void psource(orc_ctx *c, int nt)
{
    int NT = c->NT;
    if (last_source_type(c) != 1 || c->fwi_back) /* time_loop.c:248: sw == 0 only */
        return;
    for (int l = 1; l <= c->nsrc; l++) {
        int i = (int)SRC(1, l), j = (int)SRC(2, l);
        real amp = (SIG(l, nt)) / (c->DH * c->DH);
        if (nt == 1)
            amp = SIG(l, nt + 1) / (2.0 * c->DH * c->DH);
        if ((nt > 1) && (nt < NT))
            amp = (SIG(l, nt + 1) - SIG(l, nt - 1)) / (2.0 * c->DH * c->DH);
        if (nt == NT)
            amp = -SIG(l, nt - 1) / (2.0 * c->DH * c->DH);
        A(c->sxx, j, i) += amp;
        A(c->syy, j, i) += amp;
    }
}

/* eqsource.c:25-52 (moment tensor; applied to every source) */
static void eqsource(orc_ctx *c, int nt)
{
    if (last_source_type(c) != 5 || c->fwi_back) /* time_loop.c:252: sw == 0 only */
        return;
    for (int l = 1; l <= c->nsrc; l++) {
        int i = (int)SRC(1, l), j = (int)SRC(2, l);
        real dip = SRC(7, l) * PI / 180.0;
        real scale_amp = c->DT / (c->DH * c->DH);
        real amp = SRC(6, l) * scale_amp * SIG(l, nt);
        real m11 = -sin(2 * dip), m12 = -cos(2 * dip), m22 = sin(2 * dip);
        A(c->sxx, j, i) += amp * m11;
        A(c->sxy, j, i) += 0.3 * amp * m12;
        A(c->sxy, j - 1, i) += 0.3 * amp * m12;
        A(c->sxy, j, i - 1) += 0.3 * amp * m12;
        A(c->syy, j, i) += amp * m22;
    }
}

/* Free-surface velocity derivatives at row j and the second psi_vxx update
 * (surface_elastic.c:44-74, surface.c:55-85). */
static void surf_derivs(orc_ctx *c, int i, int j, real *pvxx, real *pvyy)
{
    int fdoh = c->P.fdorder / 2, NX = c->P.nx, FW = c->P.fw;
    real dhi = 1.0 / c->DH;
    real vxx = 0.0, vyy = 0.0;
    for (int m = 1; m <= fdoh; m++) {
        A(c->syy, j - m, i) = -A(c->syy, j + m, i);
        A(c->sxy, j - m, i) = -A(c->sxy, j + m - 1, i);
        vxx += c->hc[m] * (A(c->vx, j, i + m - 1) - A(c->vx, j, i - m));
        vyy += c->hc[m] * (A(c->vy, j + m - 1, i) - A(c->vy, j - m, i));
    }
    vxx *= dhi;
    vyy *= dhi;
    if (c->P.abs_type == 1 && c->P.fw > 0) {
        if ((!c->P.boundary) && (i <= FW)) {
            real *p = &PSIX(c->psi_vxx, j, i);
            *p = c->b_x[i] * *p + c->a_x[i] * vxx;
            vxx = vxx / c->K_x[i] + *p;
        }
        if ((!c->P.boundary) && (i >= NX - FW + 1)) {
            int h1 = (i - NX + 2 * FW);
            real *p = &PSIX(c->psi_vxx, j, h1);
            *p = c->b_x[h1] * *p + c->a_x[h1] * vxx;
            vxx = vxx / c->K_x[h1] + *p;
        }
    }
    *pvxx = vxx, *pvyy = vyy;
}

/* surface_elastic.c:27-90 */
static void surface_elastic(orc_ctx *c)
{
    int j = 1;
    for (int i = 1; i <= c->P.nx; i++) {
        real vxx, vyy;
        A(c->syy, j, i) = 0.0;
        surf_derivs(c, i, j, &vxx, &vyy);
        real fjm = A(c->pu, j, i) * 2.0;
        real g = A(c->ppi, j, i);
        A(c->sxx, j, i) += -(c->DT * (g - fjm) * (g - fjm) * vxx / g) - (c->DT * (g - fjm) * vyy);
    }
}

/* surface.c:27-113 (viscoelastic) */
static void surface_visc(orc_ctx *c)
{
    int j = 1, L = c->P.L;
    real dthalbe = c->DT / 2.0;
    for (int i = 1; i <= c->P.nx; i++) {
        real vxx, vyy, sump;
        A(c->syy, j, i) = 0.0;
        for (int l = 1; l <= L; l++)
            A(c->pq[l], j, i) = 0.0;
        surf_derivs(c, i, j, &vxx, &vyy);
        sump = 0.0;
        for (int l = 1; l <= L; l++)
            sump += A(c->pp[l], j, i);
        real fjm = A(c->pu, j, i) * 2.0 * (1.0 + L * A(c->ptaus, j, i));
        real g = A(c->ppi, j, i) * (1.0 + L * A(c->ptaup, j, i));
        A(c->sxx, j, i) += -(c->DT * (g - fjm) * (g - fjm) * vxx / g) - (c->DT * (g - fjm) * vyy) - (dthalbe * sump);
        sump = 0.0;
        for (int l = 1; l <= L; l++) {
            real bjm = c->peta[l] / (1.0 + (c->peta[l] * 0.5));
            real djm = 2.0 * A(c->pu, j, i) * A(c->ptaus, j, i);
            real e = A(c->ppi, j, i) * A(c->ptaup, j, i);
            A(c->pp[l], j, i) += bjm * (((djm - e) * ((fjm / g) - 1.0) * vxx) - ((djm - e) * vyy));
            sump += A(c->pp[l], j, i);
        }
        A(c->sxx, j, i) += (dthalbe * sump);
    }
}

/* seismo_ssg.c:28-67 */
static void seismo(orc_ctx *c, int lsamp)
{
    int ins = lsamp / c->P.ndt;
    for (int itr = 1; itr <= c->ntr; itr++) {
        int nx = c->rx[itr - 1], ny = c->ry[itr - 1];
        size_t o = (size_t)(itr - 1) * (size_t)c->ns + (size_t)(ins - 1);
        int s = c->P.seismo;
        if (s == 1 || s == 4) {
            c->sec[1][o] = A(c->vx, ny, nx);
            c->sec[2][o] = A(c->vy, ny, nx);
        }
        if (s == 2)
            c->sec[3][o] = -A(c->sxx, ny, nx) - A(c->syy, ny, nx);
        if (s == 3 || s == 4) {
            c->sec[4][o] = (A(c->vxx, ny, nx) + A(c->vyy, ny, nx)) * sqrt(A(c->ppi, ny, nx));
            c->sec[5][o] = (A(c->vxy, ny, nx) - A(c->vyx, ny, nx)) * sqrt(A(c->pu, ny, nx));
        }
        if (s == 4) {
            real ppi = A(c->ppi, ny, nx), pu = A(c->pu, ny, nx);
            c->sec[3][o] = ((3.0 * ppi - 4.0 * pu) / (2.0 * ppi - 2.0 * pu)) *
                           (-A(c->sxx, ny, nx) - A(c->syy, ny, nx)) / 3;
        }
    }
}

/* snap_ssg.c:28-209: one frame per component in file order (x outer, y inner) */
static void snap(orc_ctx *c)
{
    int type = c->P.snap;
    int k = c->nsnap++;
    size_t fs = (size_t)c->snap_nx * (size_t)c->snap_ny;
    if (c->nsnap > c->snap_cap) {
        c->snap_cap = c->nsnap * 2;
        for (int q = 1; q <= 5; q++)
            c->snaps[q] = (float *)realloc(c->snaps[q], fs * (size_t)c->snap_cap * sizeof(float));
    }
    real dhi = 1.0 / c->DH;
    int fdoh = c->P.fdorder / 2;
    size_t o = fs * (size_t)k;
    for (int i = c->snapidx[1]; i <= c->snapidx[2]; i += c->P.idx)
        for (int j = c->snapidx[3]; j <= c->snapidx[4]; j += c->P.idy) {
            if (type == 1 || type == 4) {
                c->snaps[1][o] = A(c->vx, j, i);
                c->snaps[2][o] = A(c->vy, j, i);
            }
            if (type == 2 || type == 4) {
                real amp = -A(c->sxx, j, i) - A(c->syy, j, i);
                c->snaps[3][o] = amp;
            }
            if (type == 3 || type == 4) {
                real vyx = 0, vxy = 0, vxx = 0, vyy = 0;
                for (int m = 1; m <= fdoh; m++) {
                    vyx += c->hc[m] * (A(c->vy, j, i + m) - A(c->vy, j, i - m + 1));
                    vxy += c->hc[m] * (A(c->vx, j + m, i) - A(c->vx, j - m + 1, i));
                }
                vyx *= dhi;
                vxy *= dhi;
                real curl = (vxy - vyx) * sqrt(A(c->pu, j, i));
                for (int m = 1; m <= fdoh; m++) {
                    vxx += c->hc[m] * (A(c->vx, j, i + m - 1) - A(c->vx, j, i - m));
                    vyy += c->hc[m] * (A(c->vy, j + m - 1, i) - A(c->vy, j - m, i));
                }
                vxx *= dhi;
                vyy *= dhi;
                real div = (vxx + vyy) * sqrt(A(c->ppi, j, i));
                c->snaps[5][o] = curl;
                c->snaps[4][o] = div;
            }
            o++;
        }
}

/* ------------------------------------------------------------- time loop */

/* snap_store.c:26-45 (DTINV = 1: every step, slot nt) */
static void fwi_store(orc_ctx *c, int nt)
{
    size_t n = (size_t)c->P.nx * (size_t)c->P.ny;
    float *slot = c->fwd + (size_t)(nt - 1) * 5 * n;
    arr2 *src[5] = {&c->pvxp1, &c->pvyp1, c->fwi_vel ? &c->ux : &c->sxx, c->fwi_vel ? &c->uy : &c->syy,
                    c->fwi_vel ? &c->uxy : &c->sxy};
    for (int k = 0; k < 5; k++)
        for (int j = 1; j <= c->P.ny; j++)
            for (int i = 1; i <= c->P.nx; i++)
                slot[(size_t)k * n + (size_t)(j - 1) * c->P.nx + (size_t)(i - 1)] = (float)A(*src[k], j, i);
}

/* calc_conv.c:34-71 at backward step nt: the forward quantities of step
 * NT - nt + 1 against the adjoint ones. The reference declares muss / lamss
 * float and the constants double, so lamss and the lambda / mu terms are
 * formed in double and rounded into the float sums. */
static void fwi_conv(orc_ctx *c, int nt)
{
    size_t n = (size_t)c->P.nx * (size_t)c->P.ny;
    const float *slot = c->fwd + (size_t)(c->NT - nt) * 5 * n;
    const float DT = (float)c->DT;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++) {
            const size_t q = (size_t)(j - 1) * c->P.nx + (size_t)(i - 1);
            const float rx = slot[q], ry = slot[n + q], fx = slot[2 * n + q], fy = slot[3 * n + q],
                        fu = slot[4 * n + q];
            const float vs0 = MAT(c->mat_vs, j, i), vp0 = MAT(c->mat_vp, j, i), rho0 = MAT(c->mat_rho, j, i);
            const float muss = vs0 * vs0 * rho0;
            const float lamss = vp0 * vp0 * rho0 - 2.0 * muss;
            const float sxx = (float)A(c->sxx, j, i), syy = (float)A(c->syy, j, i), sxy = (float)A(c->sxy, j, i);
            c->g_rhos[q] += -DT * (((float)A(c->pvxp1, j, i) * rx) + ((float)A(c->pvyp1, j, i) * ry));
            c->g_lam[q] += -DT * (1.0 / (4.0 * (lamss + muss) * (lamss + muss))) * ((fx + fy) * (sxx + syy));
            if (A(c->pu, j, i) > 0.0)
                c->g_mu[q] += -DT * (((1.0 / (muss * muss)) * (fu * sxy)) +
                                     ((1.0 / 4.0) * ((fx + fy) * (sxx + syy)) / ((lamss + muss) * (lamss + muss))) +
                                     ((1.0 / 4.0) * ((fx - fy) * (sxx - syy)) / (muss * muss)));
        }
}

int orc_fwi_begin(orc_ctx *c, int velocity, int adjoint_type)
{
    if (c->P.weq != 2) {
        snprintf(c->err, sizeof c->err, "FWI gradients need WEQ = EL_ISO");
        return 1;
    }
    if (adjoint_type < 1 || adjoint_type > 3 || (velocity != 0 && velocity != 1)) {
        snprintf(c->err, sizeof c->err, "ADJOINT_TYPE 1-3 and VELOCITY 0/1 only");
        return 1;
    }
    size_t n = (size_t)c->P.nx * (size_t)c->P.ny;
    if (!c->fwd) {
        c->fwd = (float *)calloc((size_t)c->NT * 5 * n, sizeof(float));
        c->g_lam = (float *)calloc(n, sizeof(float));
        c->g_mu = (float *)calloc(n, sizeof(float));
        c->g_rhos = (float *)calloc(n, sizeof(float));
        c->pvxp1 = alloc2(c), c->pvyp1 = alloc2(c), c->ux = alloc2(c), c->uy = alloc2(c), c->uxy = alloc2(c);
        if (!c->fwd || !c->g_lam || !c->g_mu || !c->g_rhos) {
            snprintf(c->err, sizeof c->err, "out of memory for the forward wavefields");
            return 1;
        }
    }
    memset(c->g_lam, 0, n * sizeof(float));
    memset(c->g_mu, 0, n * sizeof(float));
    memset(c->g_rhos, 0, n * sizeof(float));
    c->fwi = 1, c->fwi_vel = velocity, c->fwi_adj = adjoint_type, c->fwi_back = 0;
    return 0;
}

int orc_fwi_backward(orc_ctx *c, const float *adj_x, const float *adj_y)
{
    if (!c->fwi || c->step != c->NT) {
        snprintf(c->err, sizeof c->err, "FWI backward pass needs a completed forward pass (orc_fwi_begin, NT steps)");
        return 1;
    }
    size_t m = (size_t)(c->ntr > 0 ? c->ntr : 1) * (size_t)c->NT;
    free(c->adj);
    c->adj = (float *)malloc(2 * m * sizeof(float));
    memcpy(c->adj, adj_x, m * sizeof(float));
    memcpy(c->adj + m, adj_y, m * sizeof(float));
    orc_reset(c); /* zero_wavefield.c */
    c->fwi_back = 1;
    int rc = orc_run(c, c->NT);
    c->fwi_back = 0;
    return rc;
}

int orc_fwi_gradients(orc_ctx *c, float *lam, float *mu, float *rhos)
{
    if (!c->fwi) {
        snprintf(c->err, sizeof c->err, "FWI not begun");
        return 1;
    }
    size_t n = (size_t)c->P.nx * (size_t)c->P.ny;
    memcpy(lam, c->g_lam, n * sizeof(float));
    memcpy(mu, c->g_mu, n * sizeof(float));
    memcpy(rhos, c->g_rhos, n * sizeof(float));
    return 0;
}

int orc_reset(orc_ctx *c)
{
    /* zero_wavefield.c */
    size_t n2 = (size_t)c->pitch * (size_t)c->rows;
    arr2 *w[] = {&c->vx, &c->vy, &c->sxx, &c->syy, &c->sxy, &c->vxx, &c->vyy, &c->vyx, &c->vxy};
    for (size_t k = 0; k < sizeof(w) / sizeof(w[0]); k++)
        memset(w[k]->p, 0, n2 * sizeof(real));
    for (int l = 1; l <= c->P.L; l++) {
        memset(c->pr[l].p, 0, n2 * sizeof(real));
        memset(c->pp[l].p, 0, n2 * sizeof(real));
        memset(c->pq[l].p, 0, n2 * sizeof(real));
    }
    for (int k = 1; c->ab4 && k <= 4; k++) {
        arr2 *h[] = {&c->svx[k], &c->svy[k], &c->hxx[k], &c->hyy[k], &c->hxy[k], &c->hyx[k]};
        for (size_t q = 0; q < sizeof(h) / sizeof(h[0]); q++)
            memset(h[q]->p, 0, n2 * sizeof(real));
        for (int l = 1; k >= 2 && l <= c->P.L; l++) {
            memset(c->pr_h[k][l].p, 0, n2 * sizeof(real));
            memset(c->pp_h[k][l].p, 0, n2 * sizeof(real));
            memset(c->pq_h[k][l].p, 0, n2 * sizeof(real));
        }
    }
    int fw2 = 2 * (c->P.fw > 0 ? c->P.fw : 1);
    size_t nxf = (size_t)c->P.ny * fw2, nyf = (size_t)fw2 * c->P.nx;
    memset(c->psi_sxx_x, 0, nxf * sizeof(real));
    memset(c->psi_sxy_x, 0, nxf * sizeof(real));
    memset(c->psi_vxx, 0, nxf * sizeof(real));
    memset(c->psi_vyx, 0, nxf * sizeof(real));
    memset(c->psi_syy_y, 0, nyf * sizeof(real));
    memset(c->psi_sxy_y, 0, nyf * sizeof(real));
    memset(c->psi_vyy, 0, nyf * sizeof(real));
    memset(c->psi_vxy, 0, nyf * sizeof(real));
    c->step = 0;
    c->nsnap = 0;
    c->lsamp = c->P.ndt;
    if (c->P.snap) {
        c->lsnap = iround(c->P.tsnap1 / c->P.dt);
        c->isnap = iround(c->P.tsnapinc / c->P.dt);
        c->esnap = iround(c->P.tsnap2 / c->P.dt);
    }
    for (int k = 1; k <= 5; k++)
        if (c->sec[k])
            memset(c->sec[k], 0, sizeof(float) * (size_t)c->ntr * (size_t)c->ns);
    memset(c->tim, 0, sizeof c->tim);
    arr2 *fw[] = {&c->pvxp1, &c->pvyp1, &c->ux, &c->uy, &c->uxy};
    for (size_t k = 0; k < sizeof(fw) / sizeof(fw[0]); k++)
        if (fw[k]->p)
            memset(fw[k]->p, 0, n2 * sizeof(real));
    return 0;
}

int orc_run(orc_ctx *c, int nsteps)
{
    if (!c->prepared) {
        snprintf(c->err, sizeof c->err, "orc_prepare not called");
        return 1;
    }
    for (int s = 0; s < nsteps; s++) {
        int nt = ++c->step;
        if (nt > c->NT) {
            snprintf(c->err, sizeof c->err, "past NT");
            return 1;
        }
        double t0 = now_s();
        update_v(c, nt);
        if (c->P.boundary)
            exchange_pair_periodic(c, c->vx, c->vy);
        double t1 = now_s();
        v_derivatives(c);
        if (c->P.boundary) {
            exchange_pair_periodic(c, c->vxx, c->vyy);
            exchange_pair_periodic(c, c->vyx, c->vxy);
        }
        double t2 = now_s();
        update_s(c);
        psource(c, nt);
        eqsource(c, nt);
        if (c->P.free_surf) {
            if (c->P.L)
                surface_visc(c);
            else
                surface_elastic(c);
        }
        if (c->P.boundary)
            exchange_s_periodic(c);
        double t3 = now_s();
        if (c->P.seismo && nt == c->lsamp && nt < c->NT) {
            seismo(c, c->lsamp);
            c->lsamp += c->P.ndt;
        }
        if (c->fwi) { /* time_loop.c:288-296 */
            if (!c->fwi_back)
                fwi_store(c, nt);
            else
                fwi_conv(c, nt);
        }
        if (c->P.snap && nt == c->lsnap && nt <= c->esnap) {
            snap(c);
            c->lsnap += c->isnap;
        }
        c->tim[0] += t1 - t0;
        c->tim[1] += t2 - t1;
        c->tim[2] += t3 - t2;
        c->tim[3] += now_s() - t0;
    }
    return 0;
}

int orc_current_step(orc_ctx *c)
{
    return c->step;
}

void orc_timings(orc_ctx *c, double out[4])
{
    memcpy(out, c->tim, sizeof c->tim);
}

/* ---------------------------------------------------------------- access */

static arr2 *field_by_name(orc_ctx *c, const char *name)
{
    struct {
        const char *n;
        arr2 *a;
    } tab[] = {{"vx", &c->vx}, {"vy", &c->vy}, {"sxx", &c->sxx}, {"syy", &c->syy}, {"sxy", &c->sxy},
               {"vxx", &c->vxx}, {"vyy", &c->vyy}, {"vyx", &c->vyx}, {"vxy", &c->vxy},
               {"prip", &c->prip}, {"prjp", &c->prjp}, {"g", &c->g}, {"f", &c->f}, {"fipjp", &c->fipjp},
               {"ppi", &c->ppi}, {"pu", &c->pu}, {"prho", &c->prho}, {"puipjp", &c->puipjp},
               {"taus", &c->ptaus}, {"taup", &c->ptaup}, {"tausipjp", &c->ptausipjp},
               {"absorb", &c->absorb}, {"c11", &c->pc11}, {"c13", &c->pc13}, {"c33", &c->pc33},
               {"c55", &c->pc55}, {"c15", &c->pc15}, {"c35", &c->pc35}, {"c55ipjp", &c->pc55ipjp},
               {"c15ipjp", &c->pc15ipjp}, {"c35ipjp", &c->pc35ipjp}, {"c11u", &c->pc11u},
               {"c13u", &c->pc13u}, {"c33u", &c->pc33u}, {"c55u", &c->pc55u}, {"c15u", &c->pc15u},
               {"c35u", &c->pc35u}, {"c55ipjpu", &c->pc55ipjpu}, {"c15ipjpu", &c->pc15ipjpu},
               {"c35ipjpu", &c->pc35ipjpu}, {"tau11", &c->ptau11}, {"tau13", &c->ptau13},
               {"tau33", &c->ptau33}, {"tau55", &c->ptau55}, {"tau15", &c->ptau15}, {"tau35", &c->ptau35},
               {"tau55ipjp", &c->ptau55ipjp}, {"tau15ipjp", &c->ptau15ipjp}, {"tau35ipjp", &c->ptau35ipjp}};
    for (size_t k = 0; k < sizeof(tab) / sizeof(tab[0]); k++)
        if (!strcmp(tab[k].n, name))
            return tab[k].a;
    /* per-mechanism planes: name followed by l */
    size_t n = strlen(name);
    if (n >= 2 && name[n - 1] >= '1' && name[n - 1] <= '8') {
        int l = name[n - 1] - '0';
        if (l > c->P.L)
            return NULL;
        char base[32];
        if (n - 1 >= sizeof base)
            return NULL;
        memcpy(base, name, n - 1);
        base[n - 1] = 0;
        struct {
            const char *n;
            arr2 *a;
        } t3[] = {{"r", c->pr}, {"p", c->pp}, {"q", c->pq}, {"dip", c->dip}, {"d", c->d}, {"e", c->e},
                  {"c11d", c->pc11d}, {"c13d", c->pc13d}, {"c33d", c->pc33d}, {"c55d", c->pc55d},
                  {"c15d", c->pc15d}, {"c35d", c->pc35d}, {"c55ipjpd", c->pc55ipjpd},
                  {"c15ipjpd", c->pc15ipjpd}, {"c35ipjpd", c->pc35ipjpd}};
        for (size_t k = 0; k < sizeof(t3) / sizeof(t3[0]); k++)
            if (!strcmp(t3[k].n, base))
                return t3[k].a[l].p ? &t3[k].a[l] : NULL;
    }
    return NULL;
}

int orc_get_field(orc_ctx *c, const char *name, float *out)
{
    arr2 *a = field_by_name(c, name);
    if (!a || !a->p) {
        snprintf(c->err, sizeof c->err, "unknown field %s", name);
        return 1;
    }
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++)
            out[(size_t)(j - 1) * c->P.nx + (i - 1)] = (float)A(*a, j, i);
    return 0;
}

int orc_set_field(orc_ctx *c, const char *name, const float *in)
{
    arr2 *a = field_by_name(c, name);
    if (!a || !a->p) {
        snprintf(c->err, sizeof c->err, "unknown field %s", name);
        return 1;
    }
    for (int j = 1; j <= c->P.ny; j++)
        for (int i = 1; i <= c->P.nx; i++)
            A(*a, j, i) = in[(size_t)(j - 1) * c->P.nx + (i - 1)];
    return 0;
}

int orc_get_vector(orc_ctx *c, const char *name, float *out, int n)
{
    struct {
        const char *n;
        real *v;
        int len;
    } tab[] = {{"K_x", c->K_x, 2 * c->P.fw}, {"K_x_half", c->K_x_half, 2 * c->P.fw},
               {"a_x", c->a_x, 2 * c->P.fw}, {"a_x_half", c->a_x_half, 2 * c->P.fw},
               {"b_x", c->b_x, 2 * c->P.fw}, {"b_x_half", c->b_x_half, 2 * c->P.fw},
               {"K_y", c->K_y, 2 * c->P.fw}, {"K_y_half", c->K_y_half, 2 * c->P.fw},
               {"a_y", c->a_y, 2 * c->P.fw}, {"a_y_half", c->a_y_half, 2 * c->P.fw},
               {"b_y", c->b_y, 2 * c->P.fw}, {"b_y_half", c->b_y_half, 2 * c->P.fw},
               {"bip", c->bip, c->P.L}, {"cip", c->cip, c->P.L}, {"peta", c->peta, c->P.L}};
    if (!strcmp(name, "hc")) {
        for (int k = 0; k < n && k < 7; k++)
            out[k] = (float)c->hc[k];
        return 0;
    }
    for (size_t k = 0; k < sizeof(tab) / sizeof(tab[0]); k++)
        if (!strcmp(tab[k].n, name)) {
            for (int q = 0; q < n && q < tab[k].len; q++)
                out[q] = (float)tab[k].v[q + 1];
            return 0;
        }
    snprintf(c->err, sizeof c->err, "unknown vector %s", name);
    return 1;
}

int orc_get_section(orc_ctx *c, int comp, float *out)
{
    if (comp < 1 || comp > 5 || !c->sec[comp])
        return 1;
    memcpy(out, c->sec[comp], sizeof(float) * (size_t)c->ntr * (size_t)c->ns);
    return 0;
}

int orc_num_samples(orc_ctx *c)
{
    return c->ns;
}

int orc_num_snapshots(orc_ctx *c)
{
    return c->nsnap;
}

int orc_snapshot_size(orc_ctx *c)
{
    return c->snap_nx * c->snap_ny;
}

int orc_get_snapshot(orc_ctx *c, int k, int comp, float *out)
{
    if (k < 0 || k >= c->nsnap || comp < 1 || comp > 5 || !c->snaps[comp])
        return 1;
    size_t fs = (size_t)c->snap_nx * (size_t)c->snap_ny;
    memcpy(out, c->snaps[comp] + fs * (size_t)k, fs * sizeof(float));
    return 0;
}
