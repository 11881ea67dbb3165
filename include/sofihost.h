/*
 * sofihost.h -- C host around the GPU time loop (libsofihost.so).
 *
 * Everything the reference does on the host before and after time_loop() for
 * one forward-modelling run, kept file-compatible:
 *   - the parameter file (reference src/json_parser.c, src/read_par_json.c),
 *   - binary model files, NX traces of NY float32 samples (readmod_*.c),
 *   - model preparation: media conversion (readmod_elastic/visco/_vti/_tti.c),
 *     averaging and DT scaling (prepmod.c, av_*.c, prepare_update_s_*.c),
 *     CPML profiles (PML_pro.c) and the damping frame (absorb.c),
 *   - source and receiver files (sources.c, receiver.c), wavelets (wavelet.c),
 *   - SU seismograms (outseis_glob.c, write_su.c) and binary snapshots (snap_ssg.c),
 *   - the host side of an FWI gradient pass: observed data, residuals, the
 *     vp / vs / rho' gradients and their files (inseis.c, calc_res.c,
 *     inversion.c, output_gradient.c).
 * Pure C; no CUDA types. Errors return non-zero with sofih_last_error().
 */
#ifndef SOFIHOST_H
#define SOFIHOST_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SOFIH_MAX_L 8

/* Parameters of one run (the GlobVar fields read_par_json.c fills). */
typedef struct {
    int weq;                   /* 2..7 (EL_ISO .. VEL_TTI) */
    int nx, ny;
    float dh, dt, time;
    int nt;                    /* iround(TIME/DT) */
    int fdorder, maxrelerror, L;
    float f_ref, fl[SOFIH_MAX_L];
    int fw, abs_type, free_surf, boundary;
    float npower, k_max_cpml, vppml, fpml, damping;
    int source_shape, source_type, run_multiple_shots;
    char source_file[256];
    int seismo, ndt, readrec, seis_format;
    char rec_file[256], seis_file[256];
    float refrec[2], xrec1, yrec1, xrec2, yrec2;
    int ngeoph;
    int snap, snap_format;
    float tsnap1, tsnap2, tsnapinc;
    int idx, idy;
    char snap_file[256], mfile[256];
    int sigout, sigout_format;  /* source wavelet output (initsrc.c:64-93): 1 SU, 2 ASCII, 3 binary */
    char sigout_file[256];
    int fdorder_time;           /* 2 leapfrog, 4 Adams-Bashforth (gv->FDORDER_TIME) */
    /* MODE = FWI (read_par_json_fwi.c): one gradient pass per shot */
    int mode_fwi;
    int fwi_itermax, fwi_velocity, fwi_adjoint, fwi_lnorm, fwi_dtinv;
    char data_dir[256], gradient[256];
    /* the model: 1 from MFILE files, 0 the reference's built-in half space of
     * hh_elastic.c / hh_visco.c / hh_*_VTI.c / hh_*_TTI.c (READMOD); TAU: the
     * built-in anisotropic viscoelastic models' tau (read_par_json.c:447-449) */
    int readmod;
    float tau;
    char signal_file[256];      /* SOURCE_SHAPE 3: the signal (read_srcsig.c), ASCII or SU */
    /* receiver planes without a receiver file (REC_ARRAY > 0, receiver.c:101-116):
     * REC_ARRAY rows at depths REC_ARRAY_DEPTH + n REC_ARRAY_DIST, every DRX-th
     * column from FW to NX - FW */
    int rec_array, drx;
    float rec_array_depth, rec_array_dist;
    /* receivers (REC_TOPO) / sources (SOURCE_TOPO) placed below the topography
     * that sofih_scan_topo finds in MFILE.vp (acq_read.c:31-60); neither
     * combines with FREE_SURF (read_par_json.c:425-427) */
    int rec_topo, source_topo;
    /* SRCREC 1: sources from SOURCE_FILE; 2: a plane wave, one source per
     * column at PLANE_WAVE_DEPTH + x tan(PLANE_WAVE_ANGLE), centre frequency
     * 1 / TS (sources.c:337-371) */
    int srcrec;
    float plane_wave_depth, plane_wave_angle, ts;
    /* the shots that write snapshots (SNAPSHOT_START / _END / _INCR, read_par_json.c:320-330) */
    int snapshot_start, snapshot_end, snapshot_incr;
} sofih_par;

const char *sofih_last_error(void);

/* Read a SOFI2D parameter file; `base_dir` (may be NULL) prefixes relative
 * file names inside it. */
int sofih_read_par(const char *path, sofih_par *p);

/* Model-file suffixes the wave equation needs (vp vs rho [qp qs] [epsilon delta [theta]]). */
int sofih_model_suffixes(int weq, const char **names, int max);
/* Read MFILE.<suffix> for each needed suffix into out[k] (caller frees with free()).
 * When MFILE.vp.su exists every model is read from MFILE.<suffix>.su instead
 * (readmod_*.c): one SU trace per x column; traces past NX and samples past NY
 * are ignored, fewer is an error. */
int sofih_read_model(const sofih_par *p, const char *mfile, float **out, int max);

/* ---- model preparation ---- */
typedef struct sofih_prep sofih_prep;

/* Prepare the arrays the time loop reads from the raw material of one model
 * (arrays in model-file order [NX][NY], y fastest; unused ones may be NULL).
 * nthreads <= 0 uses every core. */
int sofih_prepare(const sofih_par *p, const float *vp, const float *vs, const float *rho, const float *qp,
                  const float *qs, const float *eps, const float *del, const float *theta, int nthreads,
                  sofih_prep **out);
void sofih_prep_free(sofih_prep *m);
/* Prepared 2-D arrays, each [NY][NX] (x fastest), named as sofi_set_model_field expects. */
int sofih_prep_num_fields(const sofih_prep *m);
const char *sofih_prep_field_name(const sofih_prep *m, int k);
const float *sofih_prep_field(const sofih_prep *m, int k);
/* 1-D arrays (CPML profiles, bip cip peta): returns the length, 0 if absent. */
int sofih_prep_vector(const sofih_prep *m, const char *name, const float **data);
/* Smallest / largest P velocity the model holds (for the CFL check). */
void sofih_prep_vrange(const sofih_prep *m, float *vpmin, float *vpmax, float *vsmin, float *vsmax);
/* FD coefficients hc[0..6] of holbergcoeff.c for (FDORDER, MAXRELERROR). */
int sofih_holberg(int fdorder, int maxrelerror, float *hc);
/* Stability bound of checkfd.c:41-52: DT <= DH / (sqrt(2) * sum|hc| * VMAX). */
int sofih_check_cfl(const sofih_par *p, const sofih_prep *m, float *dt_max);

/* ---- acquisition ---- */
/* Topography (scan_topo.c:27-76): for each column i = 1..NX the first row
 * j >= 2 whose P velocity differs from row 1's, 1 when none does, from
 * MFILE.vp.su when that file exists, else MFILE.vp. topo holds NX ints. */
int sofih_scan_topo(const sofih_par *p, const char *mfile, int *topo);
/* Sources: srcpos [12][nsrc] row-major in grid indices (reference srcpos_loc
 * layout after splitsrc.c); xy [2][nsrc] physical coordinates. SRCREC 2
 * ignores path and builds the plane wave; SOURCE_TOPO 1 counts a file
 * source's depth from the topography below its x (sources.c:122-127). */
int sofih_read_sources(const sofih_par *p, const char *path, float **srcpos, float **xy, int *nsrc);
/* Source signals [nsrc][nt] (wavelet.c): SOURCE_SHAPE 1 Ricker, 2 Fuchs-Mueller,
 * 4 sin^3, 5 Berlage, 6 Klauder (5 and 6 normalised to the amplitude; their
 * parameters in srcpos rows 8..11 as sofih_read_sources fills them).
 * SOURCE_SHAPE 3 takes the samples of SIGNAL_FILE: sofih_wavelet_file. */
int sofih_wavelet(int shape, int nt, float dt, int nsrc, const float *srcpos, float *signals);
/* The samples of a signal file (read_srcsig.c:38-184): SU (a name holding
 * ".su", first trace) or ASCII (one value per line, '#' comments, a comment
 * "DT = <s>" gives the interval); a stated interval must equal dt. The
 * caller frees *samples with free(). */
int sofih_read_signal(const char *path, float dt, float **samples, int *ns);
/* SOURCE_SHAPE 3: every source's signal is the file's samples (zero past
 * them) times its amplitude. */
int sofih_wavelet_file(const char *signal_file, int nt, float dt, int nsrc, const float *srcpos, float *signals);
/* Receivers (grid indices, reference receiver.c:41-173): from the receiver
 * file (READREC 1; co-located receivers after the first dropped; REC_TOPO 1:
 * the depth counted from the column's topography), as receiver planes
 * (REC_ARRAY > 0) or on the line XREC1..XREC2 every NGEOPH grid points; an
 * index 0 becomes 1. */
int sofih_read_receivers(const sofih_par *p, const char *path, int **ix, int **iy, int *ntr);
/* The same with each receiver's trace number (recpos[3]: its place in the
 * receiver file, which keeps the gaps of dropped co-located receivers; 1..ntr
 * otherwise); the caller frees all three arrays. */
int sofih_read_receiver_traces(const sofih_par *p, const char *path, int **ix, int **iy, int **trace, int *ntr);

/* ---- output ---- */
/* The shots (1-based, in order) whose snapshots the snapshot files hold
 * after a run of nshots shots; returns their count (shots holds nshots ints).
 * initsrc.c:96-98 lets shot s write snapshots when SNAP is set,
 * (s - SNAPSHOT_START) is a multiple of SNAPSHOT_INCR and s <= SNAPSHOT_START;
 * time_loop.c:36 numbers snapshots across shots, so only the very first
 * truncates the files (snap_ssg.c:78-83) and each such shot's frames follow
 * the previous shot's. */
int sofih_snapshot_shots(const sofih_par *p, int nshots, int *shots);
/* One SU file of a component; ep = energy source point (comp for the trace
 * header's 'ep' as outseis_glob.c writes it). xs, ys: source position [m]. */
int sofih_write_su(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                   float xs, float ys, const sofih_par *p, int ishot, int comp);
/* The same with the traces numbered as sofih_read_receiver_traces gives them
 * (tracl, tracr and cdp, outseis_glob.c:53-75; NULL: 1..ntr). */
int sofih_write_su_traces(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                          const int *trace, float xs, float ys, const sofih_par *p, int ishot, int comp);
/* The source wavelet file of initsrc.c:64-93: <SIGOUT_FILE>.shot<ishot>.<su|txt|bin>
 * holding signal[0..nt-1] as one trace (format 1 SU, 2 one value per line
 * "%e", 3 float32). (ix, iy): the source's grid position, (xs, ys) its
 * coordinates [m]. Writes the file name used into path_out (may be NULL). */
int sofih_write_signal(const sofih_par *p, int ishot, const float *signal, int nt, int ix, int iy, float xs,
                       float ys, char *path_out, int path_len);
/* Append frames to a binary snapshot file (float32, x outer, y inner). */
int sofih_write_snap(const char *path, const float *frame, int n, int append);
/* The same in SNAP_FORMAT (writedsk.c:36-52): 3 float32, 2 one value per
 * line "%e"; 1 (SU) is an error, as in the reference. */
int sofih_write_snap_format(const char *path, const float *frame, int n, int append, int format);
/* File-name extension of SEIS_FORMAT (saveseis_glob.c:39-57): 1 "su",
 * 2 "txt", 3 "bin", 0 / 4 / 5 "sgy"; NULL for any other value. */
const char *sofih_seis_ext(int format);
/* One seismogram file in p->seis_format (outseis_glob.c:39-100): 1 SU as
 * sofih_write_su_traces, 2 one value per line "%e" trace after trace, 3
 * float32 trace after trace; 0, 4 and 5 leave the file empty (the reference
 * creates it and writes nothing); returns 1 on an I/O error. */
int sofih_write_seis(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                     const int *trace, float xs, float ys, const sofih_par *p, int ishot, int comp);

/* ---- FWI gradient pass (MODE = FWI; with sofi_fwi_* of sofigpu.h) ------
 * sofih_fwi_read_data: the first ntr traces of ns samples of an observed SU
 *   file (inseis.c; "<DATA_DIR>_vx.su.shot<n>") into out [ntr][ns].
 * sofih_fwi_residual: calc_res.c for LNORM = 2 -- with velocity = 0 both
 *   sections are integrated (running float sum times DT) -- synthetic minus
 *   observed, reversed in time: diff [ntr][ns] drives the backward run; l2 =
 *   sum of its squares.
 * sofih_fwi_model_gradients: inversion.c:225-240 per cell (n cells, any
 *   common layout): the vp / vs / rho' gradients from the Lame / density sums
 *   and the model.
 * sofih_write_gradient: a [ny][nx] gradient as the reference writes it
 *   (writemod.c format 3: x outer, y inner, every idx-th / idy-th cell). */
int sofih_fwi_read_data(const char *path, int ntr, int ns, float *out);
int sofih_fwi_residual(const float *calc, const float *data, int ntr, int ns, int velocity, float dt, float *diff,
                       double *l2);
void sofih_fwi_model_gradients(size_t n, const float *lam, const float *mu, const float *rhos, const float *vp,
                               const float *vs, const float *rho, float *gvp, float *gvs, float *grho);
int sofih_write_gradient(const char *path, const float *g, int nx, int ny, int idx, int idy);

#ifdef __cplusplus
}
#endif
#endif
