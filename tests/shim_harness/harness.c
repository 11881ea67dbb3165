/*
 * harness.c -- a caller of the drop-in time_loop() shaped like the
 * reference's own (sofi2D.c:369-370 for MODE = FW, inversion.c:130-222 for
 * the forward and backward calls of an FWI gradient pass), for the GPU test
 * tests/test_gpu_shim.py. It builds the reference's data structures (stand-in
 * fd.h here) from files the test writes into a directory, calls time_loop()
 * and writes back what the reference's caller would read afterwards.
 *
 *   harness <dir>
 *
 * <dir>/params.txt   "KEY value" lines: NX NY ND NT DT DH FDORDER MAXRELERROR
 *                    L FW ABS_TYPE FREE_SURF BOUNDARY SEISMO NDT WEQ MODE
 *                    OUTNTIMESTEPINFO NSRC NTR NS VELOCITY ADJOINT_TYPE
 * <dir>/f_<member>.bin  MemModel 2-D arrays, [NY][NX] float32 (absorb_coeff too)
 * <dir>/v_<member>.bin  MemModel 1-D arrays (CPML profiles, bip cip peta)
 * <dir>/hc.bin srcpos.bin ([12][NSRC]) signals.bin ([NSRC][NT]) rec.bin (int32 [2][NTR])
 * MODE = FWI: vp0.bin vs0.bin rho0.bin ([NY][NX]), adj_x.bin adj_y.bin ([NTR][NT])
 * Writes sec_<comp>.bin ([NTR][NS]) and fld_<vx..sxy>.bin ([NY][NX]) of the
 * forward call, perf.txt; MODE = FWI also bsec_vx/vy.bin (sections after the
 * backward call) and grad_lam/mu/rhos.bin ([NY][NX]).
 */
#include "fd.h"

#include <string.h>

static const char *g_dir;

static FILE *open_in(const char *name, const char *mode)
{
    char path[1024];
    snprintf(path, sizeof path, "%s/%s", g_dir, name);
    return fopen(path, mode);
}

/* NR-style matrix m[nrl..nrh][ncl..nch], rows contiguous (util.c:231-262) */
static float **matrix(int nrl, int nrh, int ncl, int nch)
{
    int nr = nrh - nrl + 1, nc = nch - ncl + 1;
    float **m = (float **)malloc(sizeof(float *) * (size_t)nr) - nrl;
    float *d = (float *)calloc((size_t)nr * nc, sizeof(float));
    for (int r = 0; r < nr; r++)
        m[nrl + r] = d + (size_t)r * nc - ncl;
    return m;
}

static int **imatrix(int nrl, int nrh, int ncl, int nch)
{
    int nr = nrh - nrl + 1, nc = nch - ncl + 1;
    int **m = (int **)malloc(sizeof(int *) * (size_t)nr) - nrl;
    int *d = (int *)calloc((size_t)nr * nc, sizeof(int));
    for (int r = 0; r < nr; r++)
        m[nrl + r] = d + (size_t)r * nc - ncl;
    return m;
}

/* [rows][cols] float32 file into m[r0..][c0..]; 0 if the file is absent */
static int read_block(const char *name, float **m, int r0, int rows, int c0, int cols)
{
    FILE *fp = open_in(name, "rb");
    if (!fp)
        return 0;
    for (int r = 0; r < rows; r++)
        if (fread(&m[r0 + r][c0], sizeof(float), (size_t)cols, fp) != (size_t)cols) {
            fprintf(stderr, "short read in %s\n", name);
            exit(2);
        }
    fclose(fp);
    return 1;
}

static void write_block(const char *name, float **m, int r0, int rows, int c0, int cols)
{
    FILE *fp = open_in(name, "wb");
    for (int r = 0; r < rows; r++)
        fwrite(&m[r0 + r][c0], sizeof(float), (size_t)cols, fp);
    fclose(fp);
}

/* a 1-based vector from a file, NULL if absent */
static float *read_vec(const char *name, int *n)
{
    FILE *fp = open_in(name, "rb");
    if (!fp)
        return NULL;
    fseek(fp, 0, SEEK_END);
    long bytes = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    *n = (int)(bytes / 4);
    float *v = (float *)calloc((size_t)*n + 1, sizeof(float));
    if (fread(v + 1, sizeof(float), (size_t)*n, fp) != (size_t)*n)
        exit(2);
    fclose(fp);
    return v;
}

static double param(const char *key)
{
    FILE *fp = open_in("params.txt", "r");
    char k[64];
    double v;
    while (fp && fscanf(fp, "%63s %lf", k, &v) == 2)
        if (!strcmp(k, key)) {
            fclose(fp);
            return v;
        }
    fprintf(stderr, "params.txt lacks %s\n", key);
    exit(2);
}

/* an optional setting of params.txt */
static double param_or(const char *key, double dflt)
{
    FILE *fp = open_in("params.txt", "r");
    char k[64];
    double v;
    while (fp && fscanf(fp, "%63s %lf", k, &v) == 2)
        if (!strcmp(k, key)) {
            fclose(fp);
            return v;
        }
    if (fp)
        fclose(fp);
    return dflt;
}

int main(int argc, char **argv)
{
    if (argc < 2)
        return 2;
    g_dir = argv[1];
    GlobVar gv;
    memset(&gv, 0, sizeof gv);
    gv.NX = (int)param("NX"), gv.NY = (int)param("NY"), gv.ND = (int)param("ND"), gv.NT = (int)param("NT");
    gv.DT = (float)param("DT"), gv.DH = (float)param("DH"), gv.FDORDER = (int)param("FDORDER");
    gv.FDORDER_TIME = 2, gv.MAXRELERROR = (int)param("MAXRELERROR"), gv.L = (int)param("L");
    gv.FW = (int)param("FW"), gv.ABS_TYPE = (int)param("ABS_TYPE"), gv.FREE_SURF = (int)param("FREE_SURF");
    gv.BOUNDARY = (int)param("BOUNDARY"), gv.SEISMO = (int)param("SEISMO"), gv.NDT = (int)param("NDT");
    gv.WEQ = (int)param("WEQ"), gv.MODE = (int)param("MODE"), gv.NPROCX = gv.NPROCY = 1;
    gv.OUTNTIMESTEPINFO = (int)param("OUTNTIMESTEPINFO");
    /* snapshots (optional): written by time_loop() under <dir>/snap, as snap_ssg.c names them */
    gv.SNAP = (int)param_or("SNAP", 0), gv.SNAP_FORMAT = (int)param_or("SNAP_FORMAT", 3);
    gv.TSNAP1 = (float)param_or("TSNAP1", 0), gv.TSNAP2 = (float)param_or("TSNAP2", 0);
    gv.TSNAPINC = (float)param_or("TSNAPINC", 1);
    snprintf(gv.SNAP_FILE, sizeof gv.SNAP_FILE, "%s/snap", g_dir);
    const int shots = (int)param_or("SHOTS", 1); /* forward calls, as sofi2D.c's loop over shots */
    gv.IDX = gv.IDY = 1;
    const int NX = gv.NX, NY = gv.NY, ND = gv.ND, NT = gv.NT;
    const int nsrc = (int)param("NSRC"), ntr = (int)param("NTR"), ns = (int)param("NS");
    gv.NTR = ntr;
    GlobVarInv vinv = {(int)param("ADJOINT_TYPE"), 1, 2, (int)param("VELOCITY")};

    MemModel mpm;
    memset(&mpm, 0, sizeof mpm);
    struct {
        const char *name;
        float ***m;
    } f2[] = {{"prip", &mpm.prip}, {"prjp", &mpm.prjp}, {"ppi", &mpm.ppi}, {"pu", &mpm.pu}, {"g", &mpm.g},
              {"f", &mpm.f}, {"fipjp", &mpm.fipjp}, {"ptaus", &mpm.ptaus}, {"ptaup", &mpm.ptaup},
              {"puipjp", &mpm.puipjp}, {"ptausipjp", &mpm.ptausipjp}};
    for (size_t k = 0; k < sizeof f2 / sizeof f2[0]; k++) {
        char name[64];
        snprintf(name, sizeof name, "f_%s.bin", f2[k].name);
        float **m = matrix(-ND + 1, NY + ND, -ND + 1, NX + ND);
        *f2[k].m = read_block(name, m, 1, NY, 1, NX) ? m : NULL;
    }
    float **ab = matrix(1, NY, 1, NX);
    mpm.absorb_coeff = read_block("f_absorb_coeff.bin", ab, 1, NY, 1, NX) ? ab : NULL;
    struct {
        const char *name;
        float **v;
    } v1[] = {{"K_x", &mpm.K_x}, {"a_x", &mpm.a_x}, {"b_x", &mpm.b_x}, {"K_x_half", &mpm.K_x_half},
              {"a_x_half", &mpm.a_x_half}, {"b_x_half", &mpm.b_x_half}, {"K_y", &mpm.K_y}, {"a_y", &mpm.a_y},
              {"b_y", &mpm.b_y}, {"K_y_half", &mpm.K_y_half}, {"a_y_half", &mpm.a_y_half},
              {"b_y_half", &mpm.b_y_half}, {"bip", &mpm.bip}, {"cip", &mpm.cip}, {"peta", &mpm.peta}};
    for (size_t k = 0; k < sizeof v1 / sizeof v1[0]; k++) {
        char name[64];
        int n = 0;
        snprintf(name, sizeof name, "v_%s.bin", v1[k].name);
        *v1[k].v = read_vec(name, &n);
    }
    int nhc = 0;
    float *hc1 = read_vec("hc.bin", &nhc);  /* hc[0..6] */
    float **srcpos = matrix(1, 12, 1, nsrc > 0 ? nsrc : 1);
    read_block("srcpos.bin", srcpos, 1, 12, 1, nsrc);
    float **sig = matrix(1, nsrc > 0 ? nsrc : 1, 1, NT);
    read_block("signals.bin", sig, 1, nsrc, 1, NT);
    AcqVar acq;
    acq.recpos_loc = imatrix(1, 3, 1, ntr > 0 ? ntr : 1);
    {
        FILE *fp = open_in("rec.bin", "rb");
        for (int r = 1; r <= 2; r++)
            if (fread(&acq.recpos_loc[r][1], sizeof(int), (size_t)ntr, fp) != (size_t)ntr)
                return 2;
        fclose(fp);
    }
    /* the sections SEISMO records (1 v, 2 p, 3 div / curl, 4 all), as initmem.c allocates them */
    float ***secs[5] = {&gv.SECTIONVX, &gv.SECTIONVY, &gv.SECTIONP, &gv.SECTIONDIV, &gv.SECTIONCURL};
    const int sm = gv.SEISMO, want[5] = {sm == 1 || sm == 4, sm == 1 || sm == 4, sm == 2 || sm == 4,
                                         sm == 3 || sm == 4, sm == 3 || sm == 4};
    for (int k = 0; k < 5; k++)
        *secs[k] = want[k] ? matrix(1, ntr, 1, ns) : NULL;
    MemWavefield mpw;
    float ***wf[5] = {&mpw.pvx, &mpw.pvy, &mpw.psxx, &mpw.psyy, &mpw.psxy};
    for (int k = 0; k < 5; k++)
        *wf[k] = matrix(-ND + 1, NY + ND, -ND + 1, NX + ND);
    MemInv minv;
    memset(&minv, 0, sizeof minv);
    float ***mi[6] = {&minv.Vp0, &minv.Vs0, &minv.Rho0, &minv.gradLam_shot, &minv.gradMu_shot, &minv.gradRhos_shot};
    for (int k = 0; k < 6; k++)
        *mi[k] = matrix(-ND + 1, NY + ND, -ND + 1, NX + ND);
    read_block("vp0.bin", minv.Vp0, 1, NY, 1, NX);
    read_block("vs0.bin", minv.Vs0, 1, NY, 1, NX);
    read_block("rho0.bin", minv.Rho0, 1, NY, 1, NX);
    Perform perf;
    memset(&perf, 0, sizeof perf);

    /* forward call: sofi2D.c:369-370 (MODE = FW) or inversion.c:130 (sw = 0) */
    for (int s = 1; s <= shots; s++)
        time_loop(1, s, gv.SNAP > 0, hc1 + 1, srcpos, sig, sig, nsrc, 0, &acq, &mpm, &mpw, &minv, &gv, &vinv,
                  &perf);
    const char *cn[5] = {"vx", "vy", "p", "div", "curl"};
    for (int k = 0; k < 5; k++) {
        char name[64];
        snprintf(name, sizeof name, "sec_%s.bin", cn[k]);
        if (*secs[k])
            write_block(name, *secs[k], 1, ntr, 1, ns);
    }
    const char *wn[5] = {"vx", "vy", "sxx", "syy", "sxy"};
    for (int k = 0; k < 5; k++) {
        char name[64];
        snprintf(name, sizeof name, "fld_%s.bin", wn[k]);
        write_block(name, *wf[k], 1, NY, 1, NX);
    }
    if (gv.MODE == FWI) {
        /* backward call: inversion.c:207-222, sources at the receivers */
        float **back = matrix(1, 6, 1, ntr);
        for (int t = 1; t <= ntr; t++)
            back[1][t] = acq.recpos_loc[1][t], back[2][t] = acq.recpos_loc[2][t];
        float **ax = matrix(1, ntr, 1, NT), **ay = matrix(1, ntr, 1, NT);
        read_block("adj_x.bin", ax, 1, ntr, 1, NT);
        read_block("adj_y.bin", ay, 1, ntr, 1, NT);
        time_loop(1, 1, 0, hc1 + 1, back, ax, ay, ntr, 1, &acq, &mpm, &mpw, &minv, &gv, &vinv, &perf);
        write_block("bsec_vx.bin", gv.SECTIONVX, 1, ntr, 1, ns);
        write_block("bsec_vy.bin", gv.SECTIONVY, 1, ntr, 1, ns);
        write_block("grad_lam.bin", minv.gradLam_shot, 1, NY, 1, NX);
        write_block("grad_mu.bin", minv.gradMu_shot, 1, NY, 1, NX);
        write_block("grad_rhos.bin", minv.gradRhos_shot, 1, NY, 1, NX);
    }
    FILE *fp = open_in("perf.txt", "w");
    fprintf(fp, "infocounter %d\ntime_av_v_update %.9e\ntime_av_s_update %.9e\ntime_av_timestep %.9e\n",
            perf.infocounter, perf.time_av_v_update, perf.time_av_s_update, perf.time_av_timestep);
    fclose(fp);
    return 0;
}
