/*
 * sofigpu.h -- C ABI of the GB300 time-stepping library (libsofigpu.so).
 *
 * The library replaces the per-shot time loop of SOFI2D,
 *     void time_loop(int iter, int ishot, int snapcheck, float *hc, float **srcpos_loc,
 *                    float **signalx, float **signaly, int nsrc, int sw, AcqVar *acq,
 *                    MemModel *mpm, MemWavefield *mpw, MemInv *minv, GlobVar *gv,
 *                    GlobVarInv *vinv, Perform *perf)
 * (reference src/fd.h:335-337, src/time_loop.c:27-326), by device kernels on one
 * GPU. Inputs are what time_loop() reads: the prepared model arrays of MemModel
 * (after prepmod.c / PML_pro.c / absorb.c), the sources and signals of the shot,
 * the receiver grid positions; outputs are what it writes: the seismogram
 * sections (gv->SECTIONVX/VY/P/DIV/CURL), the final wavefield and the snapshots.
 *
 * Conventions
 *  - Every call returns 0 on success or a SOFI_E_* code; sofi_last_error() gives
 *    the message of the calling thread's last failure. Nothing calls exit().
 *  - Grid indices are the reference's: i = 1..NX (x), j = 1..NY (y, depth).
 *  - 2-D host arrays are passed as a pointer to element (j=1, i=1) plus a row
 *    stride and a column stride in floats, so a reference matrix m can be passed
 *    as (&m[1][1], NX + 2*ND, 1) and an f3tensor plane l as
 *    (&t[1][1][l], (NX + 2*ND) * L, L).
 *  - One context holds `nshots` resident shots of one configuration; the model
 *    is shared by all shots or given per shot (sofi_config.shared_model).
 *  - A context is used by one host thread at a time. All device work of a
 *    context is ordered on its own CUDA stream.
 */
#ifndef SOFIGPU_H
#define SOFIGPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SOFI_ABI_VERSION 2

/* status codes */
#define SOFI_OK 0
#define SOFI_E_ARG 1       /* invalid argument or configuration */
#define SOFI_E_CUDA 2      /* a CUDA runtime call failed */
#define SOFI_E_STATE 3     /* call out of order (e.g. run before sources) */
#define SOFI_E_NOMEM 4     /* device allocation failed */
#define SOFI_E_UNSTABLE 5  /* NaN at the probe cell: reference time_loop.c:44-47 */
#define SOFI_E_NODEV 6     /* no CUDA device / driver */
#define SOFI_E_BUSY 7      /* device work of the context still in flight */

/* wave equations: reference src/enums.h:22-31 */
#define SOFI_AC_ISO 0      /* acoustic: one pressure field; no free surface, no div/curl */
#define SOFI_EL_ISO 2
#define SOFI_VEL_ISO 3
#define SOFI_EL_VTI 4
#define SOFI_VEL_VTI 5
#define SOFI_EL_TTI 6
#define SOFI_VEL_TTI 7

/* seismogram components (gv->SECTIONVX, VY, P, DIV, CURL) */
#define SOFI_COMP_VX 1
#define SOFI_COMP_VY 2
#define SOFI_COMP_P 3
#define SOFI_COMP_DIV 4
#define SOFI_COMP_CURL 5

typedef struct sofi_ctx sofi_ctx;

/* The GlobVar fields time_loop() reads (reference src/globvar_struct.h:40-203). */
typedef struct {
    int weq;            /* SOFI_EL_ISO .. SOFI_VEL_TTI                         (gv->WEQ) */
    int nx, ny;         /* interior grid                                    (gv->NX, NY) */
    int fdorder;        /* 2,4,...,12                                       (gv->FDORDER) */
    int maxrelerror;    /* 0..4 Holberg table row                       (gv->MAXRELERROR) */
    int L;              /* relaxation mechanisms (viscoelastic only)             (gv->L) */
    float dt, dh;       /*                                                 (gv->DT, DH) */
    int nt;             /* time steps per shot                                  (gv->NT) */
    int fw;             /* absorbing frame width                                (gv->FW) */
    int abs_type;       /* 1 CPML, 2 exponential damping                  (gv->ABS_TYPE) */
    int free_surf;      /* stress-free top edge                          (gv->FREE_SURF) */
    int boundary;       /* 1 = periodic in x                              (gv->BOUNDARY) */
    int seismo;         /* 0 off, 1 v, 2 p, 3 div/curl, 4 all               (gv->SEISMO) */
    int ndt;            /* sampling interval in steps                          (gv->NDT) */
    int snap;           /* 0 off, 1 v, 2 p, 3 div/curl, 4 all                 (gv->SNAP) */
    int snap_first;     /* first snapshot step  iround(TSNAP1/DT)  (time_loop.c:38) */
    int snap_inc;       /* snapshot increment   iround(TSNAPINC/DT)(time_loop.c:39) */
    int snap_last;      /* last snapshot step   iround(TSNAP2/DT)  (time_loop.c:40) */
    int idx, idy;       /* snapshot subsampling                          (gv->IDX, IDY) */
    int nshots;         /* resident shots in this context (>= 1) */
    int shared_model;   /* 1: one model for all shots, 0: one model per shot */
    int fdorder_time;   /* 2 (or 0): leapfrog; 4: Adams-Bashforth, EL_ISO / VEL_ISO
                           without free surface                 (gv->FDORDER_TIME) */
} sofi_config;

/* ---- context ---------------------------------------------------------- */

/* Check the configuration, select `device`, allocate every device array the
 * time loop needs (wavefields zeroed) and create the context's stream. */
int sofi_create(const sofi_config *cfg, int device, sofi_ctx **out);
/* sofi_create with a stream priority (CUDA convention: lower is more urgent;
 * clamped to the device's range). The block scheduler prefers the work of
 * higher-priority streams when several contexts share the GPU. */
int sofi_create_with_priority(const sofi_config *cfg, int device, int priority, sofi_ctx **out);
/* The device's stream priorities: least urgent and most urgent. */
int sofi_stream_priority_range(int device, int *least, int *greatest);
/* Free and total device memory in bytes (cudaMemGetInfo on `device`). */
int sofi_device_memory(int device, long long *free_bytes, long long *total_bytes);
int sofi_destroy(sofi_ctx *ctx);
const char *sofi_last_error(void);
int sofi_abi_version(void);
/* Device bytes the context holds (for admission by HBM budget). */
int sofi_device_bytes(const sofi_config *cfg, long long *bytes);

/* ---- model: the prepared MemModel arrays (reference src/memm_struct.h) ---- */

/* Holberg coefficients hc[0..6] (reference holbergcoeff.c:38-100). Set by
 * sofi_create from (fdorder, maxrelerror); this call overrides them. */
int sofi_set_hc(sofi_ctx *ctx, const float *hc);

/* A 2-D model array, interior 1..NY x 1..NX. `model` is 0 for a shared model,
 * else the shot index. Names follow MemModel:
 *   prip prjp                 reciprocal averaged density (av_rho.c)
 *   g f fipjp                 DT-scaled (unrelaxed) moduli (prepare_update_s_*.c)
 *   ppi pu                    pi, mu (free surface, div/curl, p sampling); for
 *                             anisotropic media these are c11 and c55
 *                             (initmem_model.c:87-91 aliases them)
 *   taus taup                 (viscoelastic free surface, surface.c)
 *   c11 c13 c33 c15 c35 c55ipjp c15ipjp c35ipjp            (elastic VTI/TTI, DT-scaled)
 *   c11u c13u c33u c15u c35u c55ipjpu c15ipjpu c35ipjpu    (viscoelastic VTI/TTI)
 *   absorb                    absorb_coeff of the damping frame (absorb.c)
 * Viscoelastic modulus defects: the reference stores one array per mechanism,
 * e.g. d[j][i][l] = pu * peta[l] * ptaus (prepare_update_s_visc.c:41-43). The
 * device stores the mechanism-independent factor once and multiplies by
 * peta[l] in the kernel, so L planes per defect cost one array of traffic:
 *   d_base = pu*taus   e_base = ppi*taup   dip_base = puipjp*tausipjp   (isotropic)
 *   c11d_base = c11*tau11, c13d_base, c33d_base, c55ipjpd_base              (VTI)
 *   + c15d_base c35d_base c15ipjpd_base c35ipjpd_base                       (TTI)
 * (relaxed moduli times tau; prepare_update_s_vti.c:40-43, _tti.c:40-55). */
int sofi_set_model_field(sofi_ctx *ctx, int model, const char *name, const float *host, long row_stride,
                         long col_stride);
/* 1-D arrays: CPML profiles K_x a_x b_x K_x_half a_x_half b_x_half and the _y
 * set (2*FW values, PML_pro.c), bip cip (L values, prepare_update_s_visc.c),
 * peta (L values, readmod_visco.c:59). */
int sofi_set_model_vector(sofi_ctx *ctx, const char *name, const float *host, int n);

/* ---- acquisition ------------------------------------------------------- */

/* Sources of one shot: srcpos is the reference's srcpos_loc rows 1..12 as a
 * row-major [12][nsrc] array (row 1 grid x index, 2 grid y index, 6 amplitude,
 * 7 azimuth/dip in degrees, 8 source type 1..5), signals is [nsrc][nt]
 * (acq->signals of wavelet.c). */
int sofi_set_sources(sofi_ctx *ctx, int shot, int nsrc, const float *srcpos, const float *signals);
/* Receivers of one shot: grid indices (acq->recpos_loc rows 1 and 2). */
int sofi_set_receivers(sofi_ctx *ctx, int shot, int ntr, const int *ix, const int *iy);

/* ---- time stepping ----------------------------------------------------- */

/* Zero the wavefield, CPML memory and sections of `shot` (-1: all shots) and
 * rewind the context to step 0 (zero_wavefield.c). */
int sofi_reset(sofi_ctx *ctx, int shot);
/* Advance every resident shot by `nsteps` time steps (time_loop.c:42-322).
 * Asynchronous with respect to the host except at snapshot steps; returns
 * SOFI_E_UNSTABLE (checked at the next synchronising call) if the probe cell
 * became NaN. */
int sofi_run(sofi_ctx *ctx, int nsteps);
/* Wait for the context's stream; reports a pending instability. */
int sofi_synchronize(sofi_ctx *ctx);
/* Number of sofi_run calls whose device work has not finished yet (never
 * blocks): a host loop keeps a few runs in flight per context with it. */
int sofi_pending_runs(sofi_ctx *ctx, int *pending);
int sofi_current_step(sofi_ctx *ctx, int *step);

/* ---- outputs ----------------------------------------------------------- */

/* Seismogram section of one component, [ntr][ns] floats, ns = NT / NDT
 * (gv->SECTION*; seismo_ssg.c). Synchronises the stream. */
int sofi_get_section(sofi_ctx *ctx, int shot, int comp, float *host);
int sofi_num_samples(sofi_ctx *ctx, int *ns);
/* Interior 1..NY x 1..NX of a wavefield array (vx vy sxx syy sxy, r<l> p<l> q<l>)
 * into host[(j-1)*NX + (i-1)]; set_field writes one (for restarts and tests). */
int sofi_get_field(sofi_ctx *ctx, int shot, const char *name, float *host);
int sofi_set_field(sofi_ctx *ctx, int shot, const char *name, const float *host);
/* Snapshots taken so far (snap_ssg.c): frame k of component comp in the
 * reference's file order (x outer, y inner, strides IDX/IDY). */
int sofi_num_snapshots(sofi_ctx *ctx, int *count, int *frame_size);
int sofi_get_snapshot(sofi_ctx *ctx, int shot, int k, int comp, float *host);

/* Device time (ms, CUDA events on the context's stream) of the last sofi_run. */
int sofi_last_run_ms(sofi_ctx *ctx, float *ms);

/* ---- instrumentation (no counterpart in the reference; replaces its
 * Perform timers, src/perform_struct.h) ---- */
/* Bracket the velocity and stress kernels of every `every`-th time step with
 * CUDA events on the context's stream (0 switches it off and clears totals). */
int sofi_set_kernel_timing(sofi_ctx *ctx, int every);
/* Mean device time per timed launch of kernel `name` ("update_v", "update_s")
 * and the number of timed launches since timing was switched on. */
int sofi_kernel_time(sofi_ctx *ctx, const char *name, double *avg_ms, long long *count);
/* Velocity-kernel variant in use: cells per thread along x (1, 2 or 4) and
 * rows per thread (1, 2 or 4). The first sofi_run after sofi_reset(ctx, -1)
 * times the variants on the zeroed arrays (where each leaves them zero) and
 * keeps the fastest for the grid shape; SOFI_VROWS=w4|w2|n4|1|2|4 fixes it
 * (n4: four cells on narrow blocks, see sofi_block_threads_x). 4th-order
 * time stepping is not timed: four cells per thread unless SOFI_VROWS asks
 * for rows. */
int sofi_velocity_variant(sofi_ctx *ctx, int *cells_per_thread, int *rows_per_thread);
/* ---- FWI gradient pass of one shot (MODE = FWI, ITERMAX 1, DTINV 1) ------
 * Replaces the gradient part of the reference's inversion()
 * (src/inversion.c:32-252 with snap_store.c, calc_conv.c and the sw = 1
 * branches of time_loop.c:288-303, update_v_interior.c:72-90 and
 * wavefield_update_v.c:31-44) for WEQ = EL_ISO, one shot per context,
 * NDT = 1, SEISMO 1 or 4.
 * sofi_fwi_begin: the model as read (vp, vs, rho; [NY][NX] row-major) and the
 *   pass's VELOCITY (1: velocities, 0: displacements) and ADJOINT_TYPE (1:
 *   x and y residuals, 2: y, 3: x); allocates the forward store (NT x 5 x
 *   NX x NY floats; SOFI_E_NOMEM if it does not fit) and zeroes the sums. The
 *   next sofi_reset(ctx, -1) + sofi_run of NT steps is the forward run; it
 *   keeps every step's gradient quantities.
 * sofi_fwi_backward: the adjoint signals ([ntr][NT] each, time-reversed
 *   residuals as calc_res.c forms them, sofih_fwi_residual) after a complete
 *   forward run: zeroes the wavefield and runs NT steps with them injected at
 *   the receivers, no other source, correlating every step with forward step
 *   NT - nt + 1. Synchronous. The sections then hold the backward run's.
 * sofi_fwi_gradients: gradLam_shot, gradMu_shot, gradRhos_shot ([NY][NX]);
 *   sofih_fwi_model_gradients turns them into the vp / vs / rho' gradients.
 * When NT steps of forward quantities do not fit the device, sofi_fwi_begin
 * plans checkpoints instead (SOFI_FWI_CHECKPOINT=K forces an interval): the
 * forward run keeps the wavefield and CPML memory after steps K, 2K, ...
 * (about sqrt(NT) states), and sofi_fwi_backward recomputes each segment's
 * forward steps from its checkpoint before the backward steps that read
 * them -- one extra forward run, the same gradients bit for bit; the
 * recomputed steps record no seismograms, so the sections after the pass
 * hold the backward run's samples as after a whole-store pass.
 * sofi_fwi_checkpoints reports the interval (0: the whole run is stored) and
 * the number of segments. */
int sofi_fwi_begin(sofi_ctx *ctx, int velocity, int adjoint_type, const float *vp, const float *vs,
                   const float *rho);
int sofi_fwi_backward(sofi_ctx *ctx, const float *adj_x, const float *adj_y);
int sofi_fwi_gradients(sofi_ctx *ctx, float *grad_lam, float *grad_mu, float *grad_rhos);
int sofi_fwi_checkpoints(sofi_ctx *ctx, int *interval, int *segments);

/* Programmatic dependent launch of the step kernels: each may be scheduled
 * while the previous kernel on the context's stream finishes, and waits in
 * hardware for that kernel's completion before it touches memory, so a
 * kernel's launch overlaps the tail of the one before. On by default
 * (SOFI_PDL=0 turns it off for every new context). The request loop of
 * sofiserve.h turns it off for its contexts: with many solves sharing the
 * GPU, waiting blocks hold SM slots that other solves' kernels could use.
 * Results are the same either way. */
int sofi_pdl(sofi_ctx *ctx, int *on);
int sofi_set_pdl(sofi_ctx *ctx, int on);
/* Stress-kernel variant in use: cells per thread along x (1, 2 or 4; TTI: 1),
 * chosen by the same autotuning run; SOFI_SW=0|2|4|n4 fixes it (4th-order time
 * stepping: four unless SOFI_SW=0). */
int sofi_stress_variant(sofi_ctx *ctx, int *cells_per_thread);
/* Threads per block along x of the four-cell velocity and stress kernels in
 * use: 32 (blocks of 32 x 8 threads, 128 columns by 8 rows) or 8 (8 x 32
 * threads, 32 columns by 32 rows, which leave less of a block idle at the
 * edge of a narrow grid); chosen by the same autotuning run, SOFI_VROWS=n4 /
 * SOFI_SW=n4 fix the narrow form. */
int sofi_block_threads_x(sofi_ctx *ctx, int *velocity, int *stress);
/* 1 when the steps of a sofi_run on the current settings launch no separate
 * post-stress kernel: the one-cell stress kernel (sofi_stress_variant 1)
 * injects the explosive sources, samples the seismograms and probes for NaN
 * itself. It applies to ISO and VTI media with 2nd-order time, no free
 * surface, no moment-tensor source and at most 8 sources per shot, on grids
 * of at most 2^22 cells over all shots, outside FWI runs; SOFI_POSTF=0 turns
 * it off. Results are bit-identical either way for ISO media; for VTI media
 * the two stress kernels agree to float32 rounding. */
int sofi_post_fused(sofi_ctx *ctx, int *on);
/* Kernels launched by sofi_run since the context was created. */
int sofi_launch_count(sofi_ctx *ctx, long long *launches);
/* The context's CUDA stream (a cudaStream_t), for callers that order their own
 * work or events with the time loop. */
int sofi_get_stream(sofi_ctx *ctx, void **stream);

/* ---- allocation-free TTI stress update ------------------------------- */

/* Maximum padded cells (pitch * (NY + 16)) sofi_tti_stress_noalloc accepts. */
#define SOFI_NOALLOC_MAX_CELLS (1L << 20)

/* Device buffers of one shot for sofi_tti_stress_noalloc. Every 2-D field uses
 * this library's padded layout: float[(NY + 16) * pitch] with
 * pitch = ((NX + 16 + 31) / 32) * 32 and cell (j, i) at
 * (j - 1 + 8) * pitch + (i - 1 + 8); ghost cells zero. */
typedef struct {
    const float *vx, *vy;               /* in: velocities after this step's velocity update */
    float *sxx, *syy, *sxy;             /* in/out: stresses */
    float *r, *p, *q;                   /* in/out, VEL_TTI only: L fields each, one after another */
    float *psi_vxx, *psi_vyx;           /* in/out, CPML only: [NY][2FW] */
    float *psi_vyy, *psi_vxy;           /* in/out, CPML only: [2FW][NX] */
    /* in: the stress update's moduli (EL_TTI: DT-scaled c*, VEL_TTI: unrelaxed c*u) */
    const float *c11, *c13, *c33, *c15, *c35, *c55ipjp, *c15ipjp, *c35ipjp;
    /* in, VEL_TTI only: relaxed modulus * tau of each defect (see sofi_set_model_field) */
    const float *c11d_base, *c13d_base, *c33d_base, *c15d_base, *c35d_base, *c55ipjpd_base, *c15ipjpd_base,
        *c35ipjpd_base;
    const float *absorb;                /* in, damping frame only */
    /* in, CPML only: the 2*FW-value profiles of PML_pro.c, on the device */
    const float *K_x, *a_x, *b_x, *K_x_half, *a_x_half, *b_x_half;
    const float *K_y, *a_y, *b_y, *K_y_half, *a_y_half, *b_y_half;
    float bip[8], cip[8], peta[8];      /* VEL_TTI: L values each (host values) */
    float hc[7];                        /* FD coefficients (holbergcoeff.c) */
} sofi_tti_stress_args;

/* The stress half of one TTI time step -- the velocity derivatives, their
 * CPML stretch and the stress / memory-variable update of
 * update_s_{elastic,visc}_TTI_{interior,PML,abs}.c -- on buffers the caller
 * owns, allocating nothing. It has no counterpart in the reference: it exists
 * for callers that cannot allocate device memory (a host process that runs
 * under a fixed memory budget set at start-up, or code already inside a
 * stream capture where a cudaMalloc would break the capture). It runs the
 * two-kernel form of the TTI stress update (derivative fields between the
 * kernels; sofi_run uses it with SOFI_TTI=split, and by default a one-pass
 * kernel with the same results).
 *
 * The eight derivative fields this update needs between its two kernels live
 * in one array of the library, SOFI_NOALLOC_MAX_CELLS * 8 floats (32 MiB),
 * which every GPU that loads the library holds until the process exits;
 * grids whose padded size exceeds SOFI_NOALLOC_MAX_CELLS are rejected with
 * SOFI_E_ARG. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before
 * any stream capture. All calls share the array: calls whose work overlaps on
 * the GPU (other streams, other host threads) race, so order them on one
 * stream. Every value read from the array is written earlier in the same call,
 * so nothing has to be cleared between calls.
 *
 * The free-surface correction (surface_elastic.c / surface.c, which
 * time_loop.c applies after the stress update) and the source injection are
 * not part of this update: a caller with FREE_SURF applies them after the
 * call, as time_loop() does; FREE_SURF here only sets the CPML region order
 * (no top frame, GY[2] = 0). With periodic x (BOUNDARY 1) the caller fills
 * the ghost columns of vx and vy (the opposite edge's columns) first, as
 * exchange_v does in the reference.
 *
 * cfg: WEQ must be SOFI_EL_TTI or SOFI_VEL_TTI; nshots and the acquisition
 * fields are ignored. stream: a cudaStream_t (NULL = legacy default stream).
 * Returns after the work is queued; errors of the launch are reported. */
int sofi_tti_stress_noalloc(const sofi_config *cfg, const sofi_tti_stress_args *args, void *stream);

#ifdef __cplusplus
}
#endif
#endif
