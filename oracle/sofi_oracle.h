/*
 * sofi_oracle.h -- CPU restatement of the SOFI2D forward-modelling path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the CUDA path is compared
 * with; nothing in the product (gpi_project_gb300/, include/) may include,
 * link or call it. Only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg / reference arm use it.
 *
 * It restates, in plain C, the reference's per-time-step algorithm
 * (src/time_loop.c:27-326 with NPROCX = NPROCY = 1) and the set-up that feeds
 * it (readmod_*.c conversions, prepmod.c, PML_pro.c, absorb.c,
 * holbergcoeff.c, wavelet.c Ricker/Fuchs-Mueller/sin^3).  Each function in
 * sofi_oracle.c cites the reference file:line it follows.
 *
 * Built twice from one source:
 *   liboracle_f32.so  ORC_REAL=float  -- the reference's own float arithmetic,
 *                     including the places where a C double literal promotes a
 *                     sub-expression to double (e.g. `2.0 * f * vyy`).
 *   liboracle_f64.so  ORC_REAL=double -- the same stencil in FP64 (arbiter).
 *
 * Pinning: tests/test_oracle_golden.py checks the f32 build against the
 * reference's shipped golden seismograms/snapshots (examples/weqN_ref) and
 * against the reference compiled here (oracle/_ref, fixtures in tests/golden/).
 */
#ifndef SOFI_ORACLE_H
#define SOFI_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_L 8

/* wave equation codes: reference src/enums.h:22-31 */
enum { ORC_AC_ISO = 0, ORC_VAC_ISO, ORC_EL_ISO, ORC_VEL_ISO, ORC_EL_VTI, ORC_VEL_VTI, ORC_EL_TTI, ORC_VEL_TTI };

typedef struct {
    int weq, nx, ny, fdorder, maxrelerror, L;
    float dt, dh;
    int nt;
    int fw, abs_type, free_surf, boundary;
    float npower, k_max_cpml, vppml, fpml, damping;
    float f_ref;
    float fl[ORC_MAX_L];
    int seismo, ndt;
    int snap;               /* 0 = off, 1..4 as the reference's SNAP */
    float tsnap1, tsnap2, tsnapinc;
    int idx, idy;
    int nthreads;           /* OpenMP threads for the cell loops (0 = default) */
    int fdorder_time;       /* 2 (or 0) leapfrog, 4 Adams-Bashforth (gv->FDORDER_TIME) */
    int readmod;            /* 1: materials from orc_set_material, 0: the reference's built-in model (READMOD) */
    float tau;              /* gv->TAU of the built-in anisotropic viscoelastic models */
} orc_params;

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const orc_params *p);
void orc_destroy(orc_ctx *c);
const char *orc_error(orc_ctx *c);

/* Raw material of one model, in model-file order: NX traces of NY samples
 * (x-major, y fastest), as the reference reads them (readmod_elastic.c:103-111).
 * names: vp vs rho qp qs epsilon delta theta */
int orc_set_material(orc_ctx *c, const char *name, const float *data);

/* readmod conversion + PML_pro/absorb + prepmod (reference sofi2D.c:250-266,318). */
int orc_prepare(orc_ctx *c);

/* Sources: srcpos is the reference's srcpos_loc matrix rows 1..12 flattened
 * row-major [12][nsrc] (row 1 = grid x index, 2 = grid y index, 7 = azimuth /
 * dip [deg], 8 = SOURCE_TYPE, 6 = amplitude ...); signals is [nsrc][nt]. */
int orc_set_sources(orc_ctx *c, int nsrc, const float *srcpos, const float *signals);
/* Receivers: grid indices ix[ntr], iy[ntr] (1-based). */
int orc_set_receivers(orc_ctx *c, int ntr, const int *ix, const int *iy);

/* Wavelet (reference src/wavelet.c:33-149), shapes 1 (Ricker), 2 (Fuchs-Mueller),
 * 4 (sin^3). srcpos as above; out is [nsrc][nt]. */
int orc_wavelet(int shape, int nt, float dt, int nsrc, const float *srcpos, float *out);
/* SOURCE_SHAPE 3: the samples of the signal file (read_srcsig.c) times each source's amplitude */
int orc_wavelet_samples(int nt, float dt, int nsrc, const float *srcpos, const float *samples, int ns, float *out);

/* zero_wavefield + snapshot counter reset, then steps nt = 1..nsteps of the
 * reference time loop (continuing from the current step on later calls). */
int orc_reset(orc_ctx *c);
int orc_run(orc_ctx *c, int nsteps);
int orc_current_step(orc_ctx *c);

/* Interior (1..NY x 1..NX, x fastest) of a named array; f64 builds round to float.
 * names: vx vy sxx syy sxy vxx vyy vyx vxy prip prjp g f fipjp ppi pu prho
 *        c11 c13 c33 c55 c15 c35 c55ipjp c15ipjp c35ipjp (+u suffix for unrelaxed)
 *        taus taup absorb ; memory variables "r<l>" "p<l>" "q<l>" and
 *        coefficient planes "dip<l>" "d<l>" "e<l>" "c11d<l>" ... (l = 1..L). */
int orc_get_field(orc_ctx *c, const char *name, float *out);
int orc_set_field(orc_ctx *c, const char *name, const float *in);
/* 1-D arrays: K_x a_x b_x K_x_half ... (2FW), bip cip peta (L), hc (7) */
int orc_get_vector(orc_ctx *c, const char *name, float *out, int n);

/* Seismogram section of one component: 1 vx, 2 vy, 3 p, 4 div, 5 curl; out [ntr][ns]. */
int orc_get_section(orc_ctx *c, int comp, float *out);
int orc_num_samples(orc_ctx *c);

/* Snapshots taken so far; comp 1 vx 2 vy 3 p 4 div 5 curl. One frame holds
 * the values in the reference's file order (x outer, y inner, strides IDX/IDY). */
int orc_num_snapshots(orc_ctx *c);
int orc_snapshot_size(orc_ctx *c);
int orc_get_snapshot(orc_ctx *c, int k, int comp, float *out);

/* Time-loop phase timings of the last run, seconds: v, v-derivatives, s, total. */
void orc_timings(orc_ctx *c, double out[4]);

/* MODE = FWI, EL_ISO (inversion.c, snap_store.c, calc_conv.c; DTINV = 1):
 * orc_fwi_begin makes the next forward run of NT steps keep the gradient's
 * forward quantities of every step (VELOCITY 1: rho-weighted accelerations
 * and stress rates, 0: accelerations and stresses). orc_fwi_backward then
 * zeroes the wavefield and runs NT steps with the adjoint signals ([ntr][NT]
 * each, already time-reversed, as calc_res.c leaves them) injected at the
 * receivers (ADJOINT_TYPE 1: x and y, 2: y, 3: x), correlating every step
 * with the forward step NT - nt + 1. orc_fwi_gradients returns the per-shot
 * sums gradLam_shot, gradMu_shot, gradRhos_shot ([NY][NX], row-major). */
int orc_fwi_begin(orc_ctx *c, int velocity, int adjoint_type);
int orc_fwi_backward(orc_ctx *c, const float *adj_x, const float *adj_y);
int orc_fwi_gradients(orc_ctx *c, float *lam, float *mu, float *rhos);

#ifdef __cplusplus
}
#endif
#endif
