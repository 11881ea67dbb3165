/*
 * fd.h -- stand-in for the reference's src/fd.h, for running the drop-in
 * time_loop() (gpi_project_gb300/csrc/shim/time_loop_gb300.c) without the
 * reference tree. It declares the reference's interface types with only the
 * members the shim reads or writes, under the reference's names, and the
 * enum values of src/enums.h:22-37 (the WEQ codes equal sofigpu.h's). It is
 * test infrastructure: tests/test_gpu_shim.py builds the shim against it with
 * harness.c as the caller. Linking the shim into the reference itself uses
 * the reference's own headers (tests/test_shim_link.py).
 */
#ifndef SHIM_HARNESS_FD_H
#define SHIM_HARNESS_FD_H

#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#define STRING_SIZE 256
#define iround(x) ((int)(floor)((x) + 0.5))

typedef enum { AC_ISO = 0, VAC_ISO, EL_ISO, VEL_ISO, EL_VTI, VEL_VTI, EL_TTI, VEL_TTI } WEQTYPE;
typedef enum { FWI = 0, FW, RTM } RUNMODE;

/* src/globvar_struct.h: the run's settings and the seismogram sections */
typedef struct {
    int NX, NY, ND, NT, FDORDER, FDORDER_TIME, MAXRELERROR, L, FW, ABS_TYPE, FREE_SURF, BOUNDARY;
    int SEISMO, NDT, NTR, SNAP, SNAP_FORMAT, IDX, IDY, WEQ, MODE, NPROCX, NPROCY, OUTNTIMESTEPINFO;
    int POS[3];
    float DT, DH, TSNAP1, TSNAP2, TSNAPINC;
    char SNAP_FILE[STRING_SIZE];
    float **SECTIONVX, **SECTIONVY, **SECTIONP, **SECTIONDIV, **SECTIONCURL;
} GlobVar;

/* src/globvar_struct_fwi.h */
typedef struct {
    int ADJOINT_TYPE, DTINV, LNORM, VELOCITY;
} GlobVarInv;

/* src/memm_struct.h: prepared model arrays [-ND+1..NY+ND][-ND+1..NX+ND],
 * absorb_coeff [1..NY][1..NX], profile vectors [1..2FW], bip cip peta [1..L] */
typedef struct {
    float **prip, **prjp, **ppi, **pu, **g, **f, **fipjp, **ptaus, **ptaup, **puipjp, **ptausipjp;
    float **pc11, **pc13, **pc33, **pc15, **pc35, **pc55ipjp, **pc15ipjp, **pc35ipjp;
    float **pc11u, **pc13u, **pc33u, **pc15u, **pc35u, **pc55ipjpu, **pc15ipjpu, **pc35ipjpu;
    float **ptau11, **ptau13, **ptau33, **ptau15, **ptau35, **ptau55ipjp, **ptau15ipjp, **ptau35ipjp;
    float **absorb_coeff;
    float *K_x, *a_x, *b_x, *K_x_half, *a_x_half, *b_x_half;
    float *K_y, *a_y, *b_y, *K_y_half, *a_y_half, *b_y_half;
    float *bip, *cip, *peta;
} MemModel;

/* src/memw_struct.h */
typedef struct {
    float **pvx, **pvy, **psxx, **psyy, **psxy;
} MemWavefield;

/* src/memfwi_struct.h */
typedef struct {
    float **Vp0, **Vs0, **Rho0;
    float **gradLam_shot, **gradMu_shot, **gradRhos_shot;
} MemInv;

/* src/acq_struct.h: receiver grid positions [1..2][1..NTR] */
typedef struct {
    int **recpos_loc;
} AcqVar;

/* src/perform_struct.h */
typedef struct {
    int infocounter;
    double time_av_v_update;
    double time_av_s_update;
    double time_av_v_exchange;
    double time_av_s_exchange;
    double time_av_timestep;
} Perform;

void time_loop(int iter, int ishot, int snapcheck, float *hc, float **srcpos_loc, float **signalx,
               float **signaly, int nsrc, int sw, AcqVar *acq, MemModel *mpm, MemWavefield *mpw,
               MemInv *minv, GlobVar *gv, GlobVarInv *vinv, Perform *perf);

#endif
