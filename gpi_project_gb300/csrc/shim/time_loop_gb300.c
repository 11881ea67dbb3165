/*
 * time_loop_gb300.c -- drop-in replacement of SOFI2D's time_loop() that runs
 * the loop on one GPU through libsofigpu.so.
 *
 * Build it with the reference's own headers and link it instead of
 * src/time_loop.c:
 *     cc -c -I<sofi2d>/src -I<repo>/include time_loop_gb300.c
 *     ... link the reference's objects minus time_loop.o, plus -lsofigpu
 *
 * Signature and meaning are those of the reference (src/fd.h:335-337,
 * src/time_loop.c:27-326): the model arrays of *mpm after prepmod(), the
 * shot's sources srcpos_loc[1..12][1..nsrc] with signals signalx[1..nsrc][1..NT],
 * the receivers acq->recpos_loc[1..2][1..NTR]; outputs gv->SECTION*[1..NTR][1..NS],
 * the final wavefield in *mpw and the snapshot files of snap().
 * Supported: MODE=FW (sw = 0), FDORDER_TIME = 2 (and 4 for EL_ISO / VEL_ISO without
 * free surface; the moduli are uploaded as prepmod() left them), one domain (NPROCX = NPROCY = 1),
 * WEQ AC_ISO and EL_ISO..VEL_TTI; and MODE=FWI for EL_ISO with NDT 1, DTINV 1,
 * LNORM 2, ADJOINT_TYPE 1..3: the forward call (sw = 0) keeps the gradient
 * quantities of every step on the GPU (snap_store.c's store stays in device
 * memory), the backward call (sw = 1, the residuals of calc_res.c as signals
 * at the receivers, inversion.c:222) runs the adjoint steps with the
 * correlation of calc_conv.c and adds the shot's gradients to
 * minv->gradLam_shot / gradMu_shot / gradRhos_shot. Anything else stops the
 * run through log_fatal like the reference's own checks. The GPU context
 * (device 0, or $SOFI_GPU_DEVICE) is created on the first call and reused
 * while the configuration holds; the model is uploaded once per iteration
 * `iter` (prepmod runs per iteration). *perf accumulates as time_loop.c:94-116,
 * 264-279,312-314 does: the reference samples steps 1, 1 + OUTNTIMESTEPINFO,
 * ...; here each sampled step counts the GPU's mean velocity- and
 * stress-kernel times and the run's mean step time (no exchanges on one
 * domain).
 */
#include "fd.h"
#include "logging.h"
#include "sofigpu.h"

#include <stdlib.h>
#include <string.h>

static sofi_ctx *g_ctx = NULL;
static sofi_config g_cfg;
static int g_model_iter = -1;
static int g_nsnap_files = 0; /* snapshot numbering runs across shots, as time_loop.c:36 */

#define GPU_CHECK(call)                                                 \
    do {                                                                \
        if ((call) != SOFI_OK)                                          \
            log_fatal("GPU time loop: %s\n", sofi_last_error());       \
    } while (0)

static void upload(const char *name, float **m, const GlobVar *gv)
{
    if (m)
        GPU_CHECK(sofi_set_model_field(g_ctx, 0, name, &m[1][1], gv->NX + 2 * gv->ND, 1));
}

/* modulus * tau of each viscoelastic defect, on the host */
static void upload_product(const char *name, float **a, float **b, const GlobVar *gv)
{
    float *tmp = (float *)malloc(sizeof(float) * (size_t)gv->NX * gv->NY);
    for (int j = 1; j <= gv->NY; j++)
        for (int i = 1; i <= gv->NX; i++)
            tmp[(size_t)(j - 1) * gv->NX + (i - 1)] = a[j][i] * b[j][i];
    GPU_CHECK(sofi_set_model_field(g_ctx, 0, name, tmp, gv->NX, 1));
    free(tmp);
}

static void upload_model(MemModel *mpm, GlobVar *gv, float *hc)
{
    int weq = gv->WEQ;
    GPU_CHECK(sofi_set_hc(g_ctx, hc));
    upload("prip", mpm->prip, gv);
    upload("prjp", mpm->prjp, gv);
    if (weq == AC_ISO) {
        /* initmem_model.c:33-39: no mu; g = ppi * DT (prepare_update_s_ac.c) */
        upload("g", mpm->g, gv);
    } else {
        upload("ppi", mpm->ppi, gv);
        upload("pu", mpm->pu, gv);
    }
    if (weq == EL_ISO || weq == VEL_ISO) {
        upload("g", mpm->g, gv);
        upload("f", mpm->f, gv);
        upload("fipjp", mpm->fipjp, gv);
        if (weq == VEL_ISO) {
            upload_product("d_base", mpm->pu, mpm->ptaus, gv);
            upload_product("e_base", mpm->ppi, mpm->ptaup, gv);
            upload_product("dip_base", mpm->puipjp, mpm->ptausipjp, gv);
            if (gv->FREE_SURF) {
                upload("taus", mpm->ptaus, gv);
                upload("taup", mpm->ptaup, gv);
            }
        }
    } else if (weq != AC_ISO) {
        int tti = (weq == EL_TTI || weq == VEL_TTI), visco = (weq == VEL_VTI || weq == VEL_TTI);
        if (!visco) {
            upload("c11", mpm->pc11, gv);
            upload("c13", mpm->pc13, gv);
            upload("c33", mpm->pc33, gv);
            upload("c55ipjp", mpm->pc55ipjp, gv);
            if (tti) {
                upload("c15", mpm->pc15, gv);
                upload("c35", mpm->pc35, gv);
                upload("c15ipjp", mpm->pc15ipjp, gv);
                upload("c35ipjp", mpm->pc35ipjp, gv);
            }
        } else {
            upload("c11u", mpm->pc11u, gv);
            upload("c13u", mpm->pc13u, gv);
            upload("c33u", mpm->pc33u, gv);
            upload("c55ipjpu", mpm->pc55ipjpu, gv);
            upload_product("c11d_base", mpm->pc11, mpm->ptau11, gv);
            upload_product("c13d_base", mpm->pc13, mpm->ptau13, gv);
            upload_product("c33d_base", mpm->pc33, mpm->ptau33, gv);
            upload_product("c55ipjpd_base", mpm->pc55ipjp, mpm->ptau55ipjp, gv);
            if (tti) {
                upload("c15u", mpm->pc15u, gv);
                upload("c35u", mpm->pc35u, gv);
                upload("c15ipjpu", mpm->pc15ipjpu, gv);
                upload("c35ipjpu", mpm->pc35ipjpu, gv);
                upload_product("c15d_base", mpm->pc15, mpm->ptau15, gv);
                upload_product("c35d_base", mpm->pc35, mpm->ptau35, gv);
                upload_product("c15ipjpd_base", mpm->pc15ipjp, mpm->ptau15ipjp, gv);
                upload_product("c35ipjpd_base", mpm->pc35ipjp, mpm->ptau35ipjp, gv);
            }
        }
    }
    if (gv->FW > 0 && gv->ABS_TYPE == 2)
        GPU_CHECK(sofi_set_model_field(g_ctx, 0, "absorb", &mpm->absorb_coeff[1][1], gv->NX, 1));
    if (gv->FW > 0 && gv->ABS_TYPE == 1) {
        int n = 2 * gv->FW;
        struct { const char *name; float *v; } prof[12] = {
            {"K_x", mpm->K_x}, {"a_x", mpm->a_x}, {"b_x", mpm->b_x}, {"K_x_half", mpm->K_x_half},
            {"a_x_half", mpm->a_x_half}, {"b_x_half", mpm->b_x_half}, {"K_y", mpm->K_y}, {"a_y", mpm->a_y},
            {"b_y", mpm->b_y}, {"K_y_half", mpm->K_y_half}, {"a_y_half", mpm->a_y_half},
            {"b_y_half", mpm->b_y_half}};
        for (int k = 0; k < 12; k++)
            GPU_CHECK(sofi_set_model_vector(g_ctx, prof[k].name, &prof[k].v[1], n));
    }
    if (gv->L > 0 && (weq == VEL_ISO || weq == VEL_VTI || weq == VEL_TTI)) {
        GPU_CHECK(sofi_set_model_vector(g_ctx, "bip", &mpm->bip[1], gv->L));
        GPU_CHECK(sofi_set_model_vector(g_ctx, "cip", &mpm->cip[1], gv->L));
        GPU_CHECK(sofi_set_model_vector(g_ctx, "peta", &mpm->peta[1], gv->L));
    }
}

static void write_snapshots(GlobVar *gv)
{
    int n = 0, fs = 0;
    sofi_num_snapshots(g_ctx, &n, &fs);
    if (!n)
        return;
    float *frame = (float *)malloc(sizeof(float) * (size_t)fs);
    const char *names[6] = {0, "vx", "vy", "p", "div", "curl"};
    for (int k = 0; k < n; k++) {
        g_nsnap_files++;
        for (int comp = 1; comp <= 5; comp++) {
            int want = gv->SNAP == 4 || (gv->SNAP == 1 && comp <= 2) || (gv->SNAP == 2 && comp == 3) ||
                       (gv->SNAP == 3 && comp >= 4);
            if (!want)
                continue;
            GPU_CHECK(sofi_get_snapshot(g_ctx, 0, k, comp, frame));
            char path[STRING_SIZE * 2];
            const int ascii = gv->SNAP_FORMAT == 2; /* snap_ssg.c:53-63, writedsk.c:36-52 */
            snprintf(path, sizeof path, "%s.%s.%s.%i.%i", gv->SNAP_FILE, ascii ? "asc" : "bin", names[comp],
                     gv->POS[1], gv->POS[2]);
            FILE *fp = fopen(path, g_nsnap_files == 1 ? "w" : "a");
            if (!fp)
                log_fatal("cannot open snapshot file %s\n", path);
            if (ascii)
                for (int q = 0; q < fs; q++)
                    fprintf(fp, "%e\n", frame[q]);
            else
                fwrite(frame, sizeof(float), (size_t)fs, fp);
            fclose(fp);
        }
    }
    free(frame);
}

/* One shot's time-loop statistics into *perf (time_loop.c:94-116,264-279,312-314). */
static void fill_perform(Perform *perf, const GlobVar *gv)
{
    const int every = gv->OUTNTIMESTEPINFO > 0 ? gv->OUTNTIMESTEPINFO : 1;
    const int k = (gv->NT - 1) / every + 1; /* steps nt with (nt - 1) % every == 0 */
    float ms = 0.f;
    double vms = 0, sms = 0;
    long long nv = 0, ns = 0;
    GPU_CHECK(sofi_last_run_ms(g_ctx, &ms));
    GPU_CHECK(sofi_kernel_time(g_ctx, "update_v", &vms, &nv));
    GPU_CHECK(sofi_kernel_time(g_ctx, "update_s", &sms, &ns));
    perf->infocounter += k;
    perf->time_av_v_update += k * vms * 1e-3;
    perf->time_av_s_update += k * sms * 1e-3;
    perf->time_av_timestep += k * (ms * 1e-3 / gv->NT);
}

/* A 1-based NR matrix m[1..NY][1..NX] into a contiguous [NY][NX] buffer. */
static float *dense(float **m, const GlobVar *gv)
{
    float *d = (float *)malloc(sizeof(float) * (size_t)gv->NX * gv->NY);
    for (int j = 1; j <= gv->NY; j++)
        memcpy(d + (size_t)(j - 1) * gv->NX, &m[j][1], sizeof(float) * gv->NX);
    return d;
}

void time_loop(int iter, int ishot, int snapcheck, float *hc, float **srcpos_loc, float **signalx,
               float **signaly, int nsrc, int sw, AcqVar *acq, MemModel *mpm, MemWavefield *mpw,
               MemInv *minv, GlobVar *gv, GlobVarInv *vinv, Perform *perf)
{
    (void)ishot;
    const int fwi = gv->MODE == FWI;
    if (gv->MODE != FW && !fwi)
        log_fatal("GPU time loop: MODE must be FW or FWI\n");
    if (sw != 0 && !fwi)
        log_fatal("GPU time loop: the backward pass (sw = 1) belongs to MODE=FWI\n");
    if (fwi && (gv->WEQ != EL_ISO || gv->NDT != 1 || (gv->SEISMO != 1 && gv->SEISMO != 4) || vinv->DTINV != 1 ||
                vinv->LNORM != 2 || vinv->ADJOINT_TYPE < 1 || vinv->ADJOINT_TYPE > 3 || gv->FDORDER_TIME != 2))
        log_fatal("GPU time loop: MODE=FWI needs WEQ=EL_ISO, NDT=1, SEISMO 1 or 4, DTINV=1, LNORM=2, "
                  "ADJOINT_TYPE 1..3 and FDORDER_TIME=2\n");
    if (gv->FDORDER_TIME != 2 && gv->FDORDER_TIME != 4)
        log_fatal("GPU time loop: FDORDER_TIME must be 2 or 4\n");
    if (gv->NPROCX != 1 || gv->NPROCY != 1)
        log_fatal("GPU time loop: run one domain (NPROCX = NPROCY = 1); the GPU holds the whole grid\n");
    if (gv->SNAP && snapcheck && gv->SNAP_FORMAT != 2 && gv->SNAP_FORMAT != 3)
        log_fatal("Sorry, SU format for snapshots not implemented.\n"); /* writedsk.c:40 */

    sofi_config c;
    memset(&c, 0, sizeof c);
    c.fdorder_time = gv->FDORDER_TIME;
    c.weq = gv->WEQ, c.nx = gv->NX, c.ny = gv->NY, c.fdorder = gv->FDORDER, c.maxrelerror = gv->MAXRELERROR;
    c.L = gv->L, c.dt = gv->DT, c.dh = gv->DH, c.nt = gv->NT, c.fw = gv->FW, c.abs_type = gv->ABS_TYPE;
    c.free_surf = gv->FREE_SURF, c.boundary = gv->BOUNDARY, c.seismo = gv->SEISMO, c.ndt = gv->NDT;
    c.snap = (gv->SNAP && snapcheck) ? gv->SNAP : 0;
    c.snap_first = iround(gv->TSNAP1 / gv->DT), c.snap_inc = iround(gv->TSNAPINC / gv->DT);
    c.snap_last = iround(gv->TSNAP2 / gv->DT), c.idx = gv->IDX, c.idy = gv->IDY;
    c.nshots = 1, c.shared_model = 1;

    if (!g_ctx || memcmp(&c, &g_cfg, sizeof c) != 0) {
        if (g_ctx)
            sofi_destroy(g_ctx);
        const char *dev = getenv("SOFI_GPU_DEVICE");
        GPU_CHECK(sofi_create(&c, dev ? atoi(dev) : 0, &g_ctx));
        g_cfg = c;
        g_model_iter = -1;
    }
    if (g_model_iter != iter) {
        upload_model(mpm, gv, hc);
        g_model_iter = iter;
    }
    const int every = gv->OUTNTIMESTEPINFO > 64 ? gv->OUTNTIMESTEPINFO : 64;
    GPU_CHECK(sofi_set_kernel_timing(g_ctx, 0)); /* clears the totals */
    GPU_CHECK(sofi_set_kernel_timing(g_ctx, every));
    if (sw == 1) {
        /* inversion.c:214-222: the adjoint signals at the receivers (srcpos_loc
         * holds their grid positions, nsrc = NTR, signals [1..NTR][1..NT]) */
        if (nsrc != gv->NTR)
            log_fatal("GPU time loop: the backward pass injects at the NTR receivers\n");
        float *ax = (float *)calloc((size_t)(nsrc > 0 ? nsrc : 1) * gv->NT, sizeof(float));
        float *ay = (float *)calloc((size_t)(nsrc > 0 ? nsrc : 1) * gv->NT, sizeof(float));
        for (int l = 1; l <= nsrc; l++) {
            memcpy(ax + (size_t)(l - 1) * gv->NT, &signalx[l][1], sizeof(float) * gv->NT);
            memcpy(ay + (size_t)(l - 1) * gv->NT, &signaly[l][1], sizeof(float) * gv->NT);
        }
        int rc = sofi_fwi_backward(g_ctx, ax, ay);
        free(ax), free(ay);
        if (rc == SOFI_E_UNSTABLE)
            log_fatal("Simulation is unstable! (%s)\n", sofi_last_error());
        GPU_CHECK(rc);
        /* calc_conv.c adds each step's correlation to the shot's gradients */
        float *g[3];
        for (int k = 0; k < 3; k++)
            g[k] = (float *)malloc(sizeof(float) * (size_t)gv->NX * gv->NY);
        GPU_CHECK(sofi_fwi_gradients(g_ctx, g[0], g[1], g[2]));
        float **dst[3] = {minv->gradLam_shot, minv->gradMu_shot, minv->gradRhos_shot};
        for (int k = 0; k < 3; k++) {
            for (int j = 1; j <= gv->NY; j++)
                for (int i = 1; i <= gv->NX; i++)
                    dst[k][j][i] += g[k][(size_t)(j - 1) * gv->NX + (i - 1)];
            free(g[k]);
        }
        goto outputs;
    }
    if (fwi) {
        /* the forward run of the gradient pass keeps its gradient quantities (snap_store.c) */
        float *vp = dense(minv->Vp0, gv), *vs = dense(minv->Vs0, gv), *rho = dense(minv->Rho0, gv);
        GPU_CHECK(sofi_fwi_begin(g_ctx, vinv->VELOCITY, vinv->ADJOINT_TYPE, vp, vs, rho));
        free(vp), free(vs), free(rho);
    }
    /* sources: srcpos_loc rows 1..12, columns 1..nsrc -> [12][nsrc] */
    float *sp = (float *)calloc((size_t)12 * (nsrc > 0 ? nsrc : 1), sizeof(float));
    float *sig = (float *)calloc((size_t)(nsrc > 0 ? nsrc : 1) * gv->NT, sizeof(float));
    for (int l = 1; l <= nsrc; l++) {
        for (int r = 1; r <= 12; r++)
            sp[(size_t)(r - 1) * nsrc + (l - 1)] = srcpos_loc[r][l];
        memcpy(sig + (size_t)(l - 1) * gv->NT, &signalx[l][1], sizeof(float) * gv->NT);
    }
    GPU_CHECK(sofi_set_sources(g_ctx, 0, nsrc, sp, sig));
    free(sp);
    free(sig);
    if (gv->SEISMO && gv->NTR > 0) {
        int *ix = (int *)malloc(sizeof(int) * gv->NTR), *iy = (int *)malloc(sizeof(int) * gv->NTR);
        for (int t = 1; t <= gv->NTR; t++)
            ix[t - 1] = acq->recpos_loc[1][t], iy[t - 1] = acq->recpos_loc[2][t];
        GPU_CHECK(sofi_set_receivers(g_ctx, 0, gv->NTR, ix, iy));
        free(ix);
        free(iy);
    }
    GPU_CHECK(sofi_reset(g_ctx, 0));
    log_infoc(0, "GPU time loop: %d time steps on a %d x %d grid.\n", gv->NT, gv->NX, gv->NY);
    int rc = sofi_run(g_ctx, gv->NT);
    if (rc == SOFI_OK)
        rc = sofi_synchronize(g_ctx);
    if (rc == SOFI_E_UNSTABLE)
        log_fatal("Simulation is unstable! (%s)\n", sofi_last_error());
    GPU_CHECK(rc);

outputs:
    fill_perform(perf, gv);
    /* sections: gv->SECTION*[1..NTR][1..NS] */
    if (gv->SEISMO && gv->NTR > 0) {
        int ns = 0;
        sofi_num_samples(g_ctx, &ns);
        float *buf = (float *)malloc(sizeof(float) * (size_t)gv->NTR * (ns > 0 ? ns : 1));
        float **dst[6] = {0, gv->SECTIONVX, gv->SECTIONVY, gv->SECTIONP, gv->SECTIONDIV, gv->SECTIONCURL};
        for (int comp = 1; comp <= 5; comp++) {
            if (!dst[comp])
                continue;
            GPU_CHECK(sofi_get_section(g_ctx, 0, comp, buf));
            for (int t = 1; t <= gv->NTR; t++)
                memcpy(&dst[comp][t][1], buf + (size_t)(t - 1) * ns, sizeof(float) * (size_t)ns);
        }
        free(buf);
    }
    /* final wavefield into MemWavefield (row pitch NX + 2*ND) */
    float *w = (float *)malloc(sizeof(float) * (size_t)gv->NX * gv->NY);
    struct { const char *name; float **a; } wf[5] = {{"vx", mpw->pvx}, {"vy", mpw->pvy}, {"sxx", mpw->psxx},
                                                     {"syy", mpw->psyy}, {"sxy", mpw->psxy}};
    for (int k = 0; k < 5; k++) {
        GPU_CHECK(sofi_get_field(g_ctx, 0, wf[k].name, w));
        for (int j = 1; j <= gv->NY; j++)
            memcpy(&wf[k].a[j][1], w + (size_t)(j - 1) * gv->NX, sizeof(float) * gv->NX);
    }
    free(w);
    if (c.snap)
        write_snapshots(gv);
    log_infoc(0, "Finished time stepping.\n");
}
