/*
 * params.c -- SOFI2D parameter files.
 *
 * The reference's format (src/json_parser.c:52-140): one `"KEY" : "VALUE"`
 * pair per line, values always strings; a line holding "comment"/"Comment"
 * is skipped; comma-joined keys pair with comma-joined values
 * (`"XREC1,YREC1" : "50.0 , 1.0"`). read_par_json.c then derives
 * NT = iround(TIME/DT) (:505) and NS = NT/NDT (:516).
 */
#include "sofihost.h"

#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static __thread char g_err[512];

void sofih_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}

const char *sofih_last_error(void) { return g_err; }

#define MAXKV 256

typedef struct {
    int n;
    char key[MAXKV][96];
    char val[MAXKV][256];
} kvlist;

static void trim(char *s)
{
    size_t n = strlen(s);
    while (n && isspace((unsigned char)s[n - 1]))
        s[--n] = 0;
    size_t k = 0;
    while (s[k] && isspace((unsigned char)s[k]))
        k++;
    if (k)
        memmove(s, s + k, n - k + 1);
}

static int split_commas(char *s, char parts[][256], int max)
{
    int n = 0;
    char *tok = s;
    for (;;) {
        char *c = strchr(tok, ',');
        if (c)
            *c = 0;
        if (n < max) {
            snprintf(parts[n], 256, "%s", tok);
            trim(parts[n]);
            n++;
        }
        if (!c)
            break;
        tok = c + 1;
    }
    return n;
}

static int parse_file(const char *path, kvlist *kv)
{
    FILE *fp = fopen(path, "r");
    if (!fp) {
        sofih_set_error("cannot open parameter file %s", path);
        return 1;
    }
    char line[1024];
    int lineno = 0;
    kv->n = 0;
    while (fgets(line, sizeof line, fp)) {
        lineno++;
        if (!strchr(line, ':') || !strchr(line, '"') || strstr(line, "comment") || strstr(line, "Comment"))
            continue;
        char *q1 = strchr(line, '"'), *q2 = q1 ? strchr(q1 + 1, '"') : NULL;
        char *q3 = q2 ? strchr(q2 + 1, '"') : NULL, *q4 = q3 ? strchr(q3 + 1, '"') : NULL;
        if (!q4)
            continue;
        *q2 = 0, *q4 = 0;
        char keys[8][256], vals[8][256];
        int nk = split_commas(q1 + 1, keys, 8), nv = split_commas(q3 + 1, vals, 8);
        if (nk != nv) {
            fclose(fp);
            sofih_set_error("%s:%d: %d names but %d values", path, lineno, nk, nv);
            return 1;
        }
        for (int k = 0; k < nk && kv->n < MAXKV; k++) {
            snprintf(kv->key[kv->n], sizeof kv->key[0], "%s", keys[k]);
            snprintf(kv->val[kv->n], sizeof kv->val[0], "%s", vals[k]);
            kv->n++;
        }
    }
    fclose(fp);
    return 0;
}

static const char *get(const kvlist *kv, const char *key)
{
    for (int k = kv->n - 1; k >= 0; k--)
        if (!strcmp(kv->key[k], key))
            return kv->val[k];
    return NULL;
}

static int geti(const kvlist *kv, const char *key, int dflt)
{
    const char *v = get(kv, key);
    return v ? atoi(v) : dflt;
}

static float getf(const kvlist *kv, const char *key, float dflt)
{
    const char *v = get(kv, key);
    return v ? (float)atof(v) : dflt;
}

static void gets_(const kvlist *kv, const char *key, char *out, size_t n)
{
    const char *v = get(kv, key);
    snprintf(out, n, "%s", v ? v : "");
}

int sofih_read_par(const char *path, sofih_par *p)
{
    kvlist *kv = (kvlist *)calloc(1, sizeof(kvlist));
    if (!kv) {
        sofih_set_error("out of host memory reading %s", path);
        return 1;
    }
    if (parse_file(path, kv)) {
        free(kv);
        return 1;
    }
    memset(p, 0, sizeof *p);
    const char *w = get(kv, "WEQ");
    const char *names[] = {"AC_ISO", "VAC_ISO", "EL_ISO", "VEL_ISO", "EL_VTI", "VEL_VTI", "EL_TTI", "VEL_TTI"};
    p->weq = 2;
    if (w)
        for (int k = 0; k < 8; k++)
            if (!strcmp(w, names[k]))
                p->weq = k;
    if (p->weq == 1) {
        sofih_set_error("WEQ %s: viscoacoustic media are not supported (nor by the reference)", w);
        free(kv);
        return 1;
    }
    p->nx = geti(kv, "NX", 0), p->ny = geti(kv, "NY", 0);
    p->dh = getf(kv, "DH", 0.f), p->dt = getf(kv, "DT", 0.f), p->time = getf(kv, "TIME", 0.f);
    if (p->nx < 1 || p->ny < 1 || p->dh <= 0.f || p->dt <= 0.f) {
        sofih_set_error("%s: NX, NY, DH and DT must be positive", path);
        free(kv);
        return 1;
    }
    float ratio = p->time / p->dt;
    p->nt = (int)floor(ratio + 0.5);
    p->fdorder = geti(kv, "FDORDER", 4), p->maxrelerror = geti(kv, "MAXRELERROR", 0);
    if (geti(kv, "FDORDER_TIME", 2) != 2 && geti(kv, "FDORDER_TIME", 2) != 4) {
        sofih_set_error("FDORDER_TIME must be 2 or 4 (read_par_json.c)");
        free(kv);
        return 1;
    }
    p->L = (p->weq == 3 || p->weq == 5 || p->weq == 7) ? geti(kv, "L", 0) : 0;
    p->f_ref = getf(kv, "F_REF", 0.f);
    for (int l = 0; l < p->L && l < SOFIH_MAX_L; l++) {
        char k[16];
        snprintf(k, sizeof k, "FL%d", l + 1);
        p->fl[l] = getf(kv, k, 0.f);
    }
    p->free_surf = geti(kv, "FREE_SURF", 0), p->boundary = geti(kv, "BOUNDARY", 0);
    p->fw = geti(kv, "FW", 0), p->abs_type = geti(kv, "ABS_TYPE", 0);
    p->npower = getf(kv, "NPOWER", 2.f), p->k_max_cpml = getf(kv, "K_MAX_CPML", 1.f);
    p->vppml = getf(kv, "VPPML", 0.f), p->fpml = getf(kv, "FPML", 0.f), p->damping = getf(kv, "DAMPING", 8.f);
    p->source_shape = geti(kv, "SOURCE_SHAPE", 1), p->source_type = geti(kv, "SOURCE_TYPE", 1);
    p->run_multiple_shots = geti(kv, "RUN_MULTIPLE_SHOTS", 0);
    gets_(kv, "SOURCE_FILE", p->source_file, sizeof p->source_file);
    p->seismo = geti(kv, "SEISMO", 0), p->ndt = geti(kv, "NDT", 1), p->readrec = geti(kv, "READREC", 1);
    p->seis_format = geti(kv, "SEIS_FORMAT", 1);
    gets_(kv, "REC_FILE", p->rec_file, sizeof p->rec_file);
    gets_(kv, "SEIS_FILE", p->seis_file, sizeof p->seis_file);
    p->sigout = geti(kv, "SIGOUT", 0), p->sigout_format = geti(kv, "SIGOUT_FORMAT", 1);
    p->fdorder_time = geti(kv, "FDORDER_TIME", 2);
    gets_(kv, "SIGOUT_FILE", p->sigout_file, sizeof p->sigout_file);
    p->refrec[0] = getf(kv, "REFRECX", 0.f), p->refrec[1] = getf(kv, "REFRECY", 0.f);
    p->xrec1 = getf(kv, "XREC1", 0.f), p->yrec1 = getf(kv, "YREC1", 0.f);
    p->xrec2 = getf(kv, "XREC2", 0.f), p->yrec2 = getf(kv, "YREC2", 0.f);
    p->ngeoph = geti(kv, "NGEOPH", 1);
    p->snap = geti(kv, "SNAP", 0), p->snap_format = geti(kv, "SNAP_FORMAT", 3);
    p->tsnap1 = getf(kv, "TSNAP1", 0.f), p->tsnap2 = getf(kv, "TSNAP2", 0.f), p->tsnapinc = getf(kv, "TSNAPINC", 0.f);
    p->idx = geti(kv, "IDX", 1), p->idy = geti(kv, "IDY", 1);
    gets_(kv, "SNAP_FILE", p->snap_file, sizeof p->snap_file);
    gets_(kv, "MFILE", p->mfile, sizeof p->mfile);
    /* MODE = FWI (read_par_json_fwi.c): the keys one gradient pass reads */
    const char *mode = get(kv, "MODE");
    p->mode_fwi = mode && !strcmp(mode, "FWI");
    p->fwi_itermax = geti(kv, "ITERMAX", 1), p->fwi_velocity = geti(kv, "VELOCITY", 0);
    p->fwi_adjoint = geti(kv, "ADJOINT_TYPE", 1), p->fwi_lnorm = geti(kv, "LNORM", 2);
    p->fwi_dtinv = geti(kv, "DTINV", 1);
    gets_(kv, "DATA_DIR", p->data_dir, sizeof p->data_dir);
    gets_(kv, "GRADIENT", p->gradient, sizeof p->gradient);
    p->readmod = geti(kv, "READMOD", 1), p->tau = getf(kv, "TAU", 0.0001f);
    gets_(kv, "SIGNAL_FILE", p->signal_file, sizeof p->signal_file);
    /* receiver planes and topography (read_par_json.c:242-246, 347-403, 425-427) */
    p->rec_array = geti(kv, "REC_ARRAY", 0), p->drx = geti(kv, "DRX", 0);
    p->rec_array_depth = getf(kv, "REC_ARRAY_DEPTH", 0.f), p->rec_array_dist = getf(kv, "REC_ARRAY_DIST", 0.f);
    p->rec_topo = p->seismo > 0 ? geti(kv, "REC_TOPO", 0) : 0;
    p->srcrec = geti(kv, "SRCREC", 1);
    p->source_topo = p->srcrec == 1 ? geti(kv, "SOURCE_TOPO", 0) : 0;
    p->plane_wave_depth = getf(kv, "PLANE_WAVE_DEPTH", 0.f), p->plane_wave_angle = getf(kv, "PLANE_WAVE_ANGLE", 0.f);
    p->ts = getf(kv, "TS", 0.f);
    p->snapshot_start = geti(kv, "SNAPSHOT_START", 1), p->snapshot_end = geti(kv, "SNAPSHOT_END", -9999);
    p->snapshot_incr = geti(kv, "SNAPSHOT_INCR", 1);
    const char *bad = NULL;
    if (p->rec_topo < 0 || p->rec_topo > 1)
        bad = "REC_TOPO needs to be 0 or 1";
    else if (p->source_topo < 0 || p->source_topo > 1)
        bad = "SOURCE_TOPO needs to be 0 or 1";
    else if ((p->rec_topo || p->source_topo) && p->free_surf)
        bad = "source or receiver topography cannot be combined with FREE_SURF";
    else if (p->seismo > 0 && !p->readrec && p->rec_array > 0 && p->drx < 1)
        bad = "REC_ARRAY > 0 needs DRX >= 1";
    else if (p->srcrec != 1 && p->srcrec != 2)
        bad = "SRCREC must be 1 (source file) or 2 (plane wave)";
    else if (p->srcrec == 2 && p->plane_wave_depth <= 0.f)
        bad = "SRCREC 2 (plane wave) needs PLANE_WAVE_DEPTH > 0";
    else if (p->srcrec == 2 && p->source_shape > 4)
        bad = "a plane wave takes SOURCE_SHAPE 1-4 only";
    else if (p->srcrec == 2 && p->ts <= 0.f)
        bad = "a plane wave needs TS > 0";
    else if (p->snap > 0 && p->snapshot_incr < 1)
        bad = "SNAPSHOT_INCR must be at least 1";
    else if (p->snap > 0 && p->snap_format != 2 && p->snap_format != 3)
        bad = p->snap_format == 1 ? "SNAP_FORMAT 1: the SU format for snapshots is not implemented (nor by the "
                                    "reference); SNAP_FORMAT 2 (ASCII) or 3 (binary)"
                                  : "SNAP_FORMAT must be 2 (ASCII) or 3 (binary)";
    else if (p->seismo > 0 && (p->seis_format < 0 || p->seis_format > 5))
        bad = "SEIS_FORMAT must be 0-5 (1 SU, 2 ASCII, 3 binary; 0, 4 and 5 write empty .sgy files)";
    free(kv);
    if (bad) {
        sofih_set_error("%s: %s", path, bad);
        return 1;
    }
    return 0;
}
