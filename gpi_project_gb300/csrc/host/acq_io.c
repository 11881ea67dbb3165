/*
 * acq_io.c -- model files, sources, receivers, wavelets and outputs.
 *
 *   model files      NX traces of NY float32 samples (readmod_elastic.c:103-111)
 *   source file      x y tshift fc amp [azimuth [type]] per line (Berlage and Klauder
 *                    wavelets: their parameters too), '#' comments (sources.c:60-316);
 *                    grid index floor(x/DH)+1 (splitsrc.c:34-36)
 *   receiver file    x y per line, '#'/'%' comments; duplicates dropped
 *                    (receiver.c:48-110); or a line XREC1..XREC2 every NGEOPH
 *   wavelets         Ricker, Fuchs-Mueller, file, sin^3, Berlage, Klauder (wavelet.c:33-149,
 *                    read_srcsig.c:38-184)
 *   SU traces        240-byte trace header + float32 samples (outseis_glob.c:40-81)
 *   snapshots        float32 stream per component (snap_ssg.c, SNAP_FORMAT=3)
 */
#include "sofihost.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define PI M_PI
#define IROUND(x) ((int)floor((x) + 0.5))

void sofih_set_error(const char *fmt, ...);

static const char *SUFFIX[8][8] = {
    {"vp", "rho"}, {0}, {"vp", "vs", "rho"}, {"vp", "vs", "rho", "qp", "qs"}, {"vp", "vs", "rho", "epsilon", "delta"},
    {"vp", "vs", "rho", "epsilon", "delta", "qp", "qs"}, {"vp", "vs", "rho", "epsilon", "delta", "theta"},
    {"vp", "vs", "rho", "epsilon", "delta", "theta", "qp", "qs"}};

int sofih_model_suffixes(int weq, const char **names, int max)
{
    if (weq < 0 || weq == 1 || weq > 7)
        return 0;
    int n = 0;
    while (n < 8 && SUFFIX[weq][n])
        n++;
    for (int k = 0; k < n && k < max; k++)
        names[k] = SUFFIX[weq][k];
    return n;
}

/* One model in SU format (readmod_elastic.c:62-96 with read_su.c): NX traces
 * of at least NY samples, 240-byte headers, native endian; ns from the first
 * header. out: [NX][NY], y fastest. */
static int read_su_model(const char *path, int nx, int ny, float *out)
{
    FILE *fp = fopen(path, "rb");
    if (!fp) {
        sofih_set_error("cannot open model file %s", path);
        return 1;
    }
    unsigned char h[240];
    unsigned short ns = 0;
    if (fread(h, 1, 240, fp) != 240) {
        fclose(fp);
        sofih_set_error("short read in SU file %s", path);
        return 1;
    }
    memcpy(&ns, h + 114, 2);
    fseek(fp, 0, SEEK_END);
    long size = ftell(fp);
    long tracelen = 240 + 4L * ns;
    long ntr = ns ? size / tracelen : 0;
    if (ns < 1 || ntr < nx || ns < ny) {
        fclose(fp);
        sofih_set_error("%s: %ld traces of %u samples, NX=%d traces of NY=%d samples needed", path, ntr,
                        (unsigned)ns, nx, ny);
        return 1;
    }
    float *tr = (float *)malloc(sizeof(float) * ns);
    int bad = !tr;
    for (int i = 0; i < nx && !bad; i++) {
        bad = fseek(fp, (long)i * tracelen + 240, SEEK_SET) != 0 || fread(tr, sizeof(float), ns, fp) != ns;
        if (!bad)
            memcpy(out + (size_t)i * ny, tr, sizeof(float) * (size_t)ny);
    }
    free(tr);
    fclose(fp);
    if (bad) {
        sofih_set_error("short read in SU file %s", path);
        return 1;
    }
    return 0;
}

int sofih_read_model(const sofih_par *p, const char *mfile, float **out, int max)
{
    const char *names[8];
    int n = sofih_model_suffixes(p->weq, names, 8);
    size_t cnt = (size_t)p->nx * (size_t)p->ny;
    char probe[600];
    snprintf(probe, sizeof probe, "%s.vp.su", mfile);
    FILE *pf = fopen(probe, "rb");
    const int su = pf != NULL; /* readmod_elastic.c:50-58: vp.su decides for all models */
    if (pf)
        fclose(pf);
    for (int k = 0; k < n && k < max; k++) {
        if (su) {
            char path[600];
            snprintf(path, sizeof path, "%s.%s.su", mfile, names[k]);
            out[k] = (float *)malloc(cnt * sizeof(float));
            if (!out[k] || read_su_model(path, p->nx, p->ny, out[k]))
                return 1;
            continue;
        }
        char path[600];
        snprintf(path, sizeof path, "%s.%s", mfile, names[k]);
        FILE *fp = fopen(path, "rb");
        if (!fp) {
            sofih_set_error("cannot open model file %s", path);
            return 1;
        }
        out[k] = (float *)malloc(cnt * sizeof(float));
        size_t got = fread(out[k], sizeof(float), cnt, fp);
        fclose(fp);
        if (got != cnt) {
            sofih_set_error("%s holds %zu values, NX*NY = %zu needed", path, got, cnt);
            return 1;
        }
    }
    return 0;
}

int sofih_scan_topo(const sofih_par *p, const char *mfile, int *topo)
{
    const size_t cnt = (size_t)p->nx * (size_t)p->ny;
    float *vp = (float *)malloc(cnt * sizeof(float));
    if (!vp) {
        sofih_set_error("out of host memory scanning the topography");
        return 1;
    }
    char path[600];
    snprintf(path, sizeof path, "%s.vp.su", mfile);
    FILE *fp = fopen(path, "rb");
    int rc = 0;
    if (fp) { /* scan_topo.c:35-45: the SU model when it is readable */
        fclose(fp);
        rc = read_su_model(path, p->nx, p->ny, vp);
    } else {
        snprintf(path, sizeof path, "%s.vp", mfile);
        fp = fopen(path, "rb");
        if (!fp) {
            free(vp);
            sofih_set_error("could not open the P-wave velocity model %s to scan the topography", path);
            return 1;
        }
        const size_t got = fread(vp, sizeof(float), cnt, fp);
        fclose(fp);
        if (got != cnt) {
            sofih_set_error("%s holds %zu values, NX*NY = %zu needed", path, got, cnt);
            rc = 1;
        }
    }
    for (int i = 0; i < p->nx && !rc; i++) { /* scan_topo.c:58-68 */
        const float *tr = vp + (size_t)i * p->ny;
        int t = 1;
        for (int j = 2; j <= p->ny; j++)
            if (tr[j - 1] != tr[0]) {
                t = j;
                break;
            }
        topo[i] = t;
    }
    free(vp);
    return rc;
}

static int is_data_line(const char *s, int allow_percent)
{
    if (strchr(s, '#') || (allow_percent && strchr(s, '%')))
        return 0;
    char tok[64];
    return sscanf(s, "%63s", tok) == 1;
}

/* SRCREC 2 (sources.c:337-371): one source per column at the plane wave's
 * depth, no time shift, centre frequency 1 / TS, unit amplitude, the run's
 * SOURCE_TYPE; the operand types follow the reference's. */
static int plane_wave_sources(const sofih_par *p, float **srcpos, float **xy, int *nsrc)
{
    const float tan_phi = (float)tan(p->plane_wave_angle * PI / 180.0);
    const float dz = (float)(p->nx - 1) * p->dh * tan_phi;
    if (p->plane_wave_depth + dz > (p->ny - 1) * p->dh) {
        sofih_set_error("the plane wave's maximum depth %g m exceeds the model depth", p->plane_wave_depth + dz);
        return 1;
    }
    const int n = p->nx;
    float *sp = (float *)calloc((size_t)12 * n, sizeof(float));
    float *pos = (float *)calloc((size_t)2 * n, sizeof(float));
    if (!sp || !pos) {
        free(sp), free(pos);
        sofih_set_error("out of host memory");
        return 1;
    }
    for (int i = 1; i <= n; i++) {
        const int l = i - 1;
        const float x = (i - 1) * p->dh;
        const float y = p->plane_wave_depth + (tan_phi * x);
        const float fc = 1.0 / p->ts;
        sp[0 * n + l] = (float)((int)floor(x / p->dh) + 1);
        sp[1 * n + l] = (float)((int)floor(y / p->dh) + 1);
        sp[3 * n + l] = 0.0f, sp[4 * n + l] = fc, sp[5 * n + l] = 1.0f;
        sp[6 * n + l] = 0.0f, sp[7 * n + l] = (float)p->source_type;
        pos[l] = x, pos[n + l] = y;
    }
    *srcpos = sp, *xy = pos, *nsrc = n;
    return 0;
}

int sofih_read_sources(const sofih_par *p, const char *path, float **srcpos, float **xy, int *nsrc)
{
    if (p->srcrec == 2)
        return plane_wave_sources(p, srcpos, xy, nsrc);
    int *topo = NULL;
    if (p->source_topo) {
        topo = (int *)malloc(sizeof(int) * (size_t)p->nx);
        if (!topo || sofih_scan_topo(p, p->mfile, topo)) {
            free(topo);
            return 1;
        }
    }
    FILE *fp = fopen(path, "r");
    if (!fp) {
        free(topo);
        sofih_set_error("cannot open source file %s", path);
        return 1;
    }
    char line[512];
    int n = 0;
    while (fgets(line, sizeof line, fp))
        n += is_data_line(line, 0);
    rewind(fp);
    float *sp = (float *)calloc((size_t)12 * (n ? n : 1), sizeof(float));
    float *pos = (float *)calloc((size_t)2 * (n ? n : 1), sizeof(float));
    int l = 0;
    while (fgets(line, sizeof line, fp)) {
        if (!is_data_line(line, 0))
            continue;
        /* columns (sources.c:60-316): x y tshift, then
         *   SOURCE_SHAPE <= 4  fc amp [azimuth [type]]
         *   5 (Berlage)        fc amp exponent decay phase [azimuth [type]]
         *   6 (Klauder)        fmin fmax amp sweep-length width [azimuth [type]]  (fc = (fmin + fmax) / 2) */
        float v[10] = {0};
        const int k = sscanf(line, "%f%f%f%f%f%f%f%f%f%f", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &v[7],
                             &v[8], &v[9]);
        const int shape = p->source_shape, need = shape == 5 || shape == 6 ? 8 : 5;
        if (k < need) {
            fclose(fp);
            free(sp), free(pos), free(topo);
            sofih_set_error("%s: source %d lacks %s", path, l + 1,
                            shape == 5   ? "time shift, frequency, amplitude, exponent, decay or phase"
                            : shape == 6 ? "time shift, frequencies, amplitude, sweep length or width"
                                         : "time shift, frequency or amplitude");
            return 1;
        }
        float az = k > need ? v[need] : 0.0f, type = k > need + 1 ? v[need + 1] : (float)p->source_type;
        if (topo) { /* sources.c:122-127: the depth below the topography at the source's column */
            const int xidx = (int)floor(v[0] / p->dh) + 1;
            if (xidx < 1 || xidx > p->nx) {
                fclose(fp);
                free(sp), free(pos), free(topo);
                sofih_set_error("%s: source %d lies outside the model's columns", path, l + 1);
                return 1;
            }
            v[1] = (topo[xidx - 1] - 1) * p->dh + v[1];
        }
        sp[0 * n + l] = (float)((int)floor(v[0] / p->dh) + 1);
        sp[1 * n + l] = (float)((int)floor(v[1] / p->dh) + 1);
        sp[3 * n + l] = v[2];
        if (shape == 6) {
            sp[8 * n + l] = v[3], sp[9 * n + l] = v[4], sp[5 * n + l] = v[5], sp[10 * n + l] = v[6];
            sp[11 * n + l] = v[7];
            sp[4 * n + l] = (v[3] + v[4]) / 2;
        } else {
            sp[4 * n + l] = v[3], sp[5 * n + l] = v[4];
            if (shape == 5)
                sp[8 * n + l] = v[5], sp[9 * n + l] = v[6], sp[10 * n + l] = v[7];
        }
        sp[6 * n + l] = az, sp[7 * n + l] = type;
        pos[l] = v[0], pos[n + l] = v[1];
        l++;
    }
    fclose(fp);
    free(topo);
    *srcpos = sp, *xy = pos, *nsrc = n;
    return 0;
}

/* One source's signal (wavelet.c:48-142). The operand types follow the
 * reference's (float variables, double constants and libm calls), so the
 * samples equal its own bit for bit: srcpos row 3 time shift, 4 centre
 * frequency, 5 amplitude, rows 8..11 the Berlage (time exponent, decay,
 * initial phase [deg]) or Klauder (lowest / highest frequency, sweep length,
 * half width in centre periods) parameters; `file` the samples of a
 * SOURCE_SHAPE 3 signal file. */
static int one_wavelet(int shape, int nt, float dt, int nsrc, int k, const float *srcpos, const float *file,
                       int nfile, float *sig)
{
    const float tshift = srcpos[3 * nsrc + k], fc = srcpos[4 * nsrc + k], a = srcpos[5 * nsrc + k];
    const float ts = 1.0 / fc;
    float sigmax = 0.0;
    for (int n = 1; n <= nt; n++) {
        const float t = (float)n * dt;
        float amp = 0.0, tau;
        switch (shape) {
          case 1: /* Ricker */
              tau = PI * (t - 1.5 * ts - tshift) / (ts);
              amp = (((1.0 - 2.0 * tau * tau) * exp(-tau * tau)));
              break;
          case 2: /* Fuchs-Mueller */
              amp = ((t < tshift) || (t > (tshift + ts)))
                        ? 0.0
                        : (sin(2.0 * PI * (t - tshift) * fc) - 0.5 * sin(4.0 * PI * (t - tshift) * fc));
              break;
          case 3: /* samples of SIGNAL_FILE */
              amp = n <= nfile ? file[n - 1] : 0.0f;
              break;
          case 4: /* sin^3 */
              amp = ((t < tshift) || (t > (tshift + ts))) ? 0.0 : pow(sin(PI * (t - tshift) / ts), 3.0);
              break;
          case 5: { /* Berlage (Aldridge 1990), wavelet.c:82-96 */
              const float ex = srcpos[8 * nsrc + k], alpha = srcpos[9 * nsrc + k];
              const float phi0 = srcpos[10 * nsrc + k] * PI / 180;
              if (ex <= 0) {
                  sofih_set_error("source %d: the Berlage wavelet needs a time exponent > 0", k + 1);
                  return 1;
              }
              amp = (t < tshift) ? 0.0
                                 : a * pow((t - tshift), ex) * exp(-alpha * (t - tshift)) *
                                       cos(2 * PI * fc * (t - tshift) + phi0);
              break;
          }
          case 6: { /* Klauder, wavelet.c:97-125. The reference's exp() of the complex
                     * carrier sees only its real part (no <tgmath.h>): exp(0) = 1, so
                     * the wavelet is the sweep's envelope without the carrier */
              const float fmin = srcpos[8 * nsrc + k], fmax = srcpos[9 * nsrc + k];
              const float T = srcpos[10 * nsrc + k], width = srcpos[11 * nsrc + k];
              const float f2 = (fmax - fmin) / T;
              tau = (width / fc);
              if ((t < tshift) || (t > (tau * 2) + tshift)) {
                  amp = 0.0;
              } else {
                  const float tp = t - tau - tshift;
                  amp = sin(PI * f2 * tp * (T - tp)) / (PI * f2 * tp) * 1.0;
                  if (t < (tau * 0.2) + tshift) {
                      const float taper = (1 - cos(((t - tshift) / tau / 0.2) * PI)) / 2;
                      amp = amp * taper;
                  } else if (t > (tau * 1.8) + tshift) {
                      const float taper = (1 - cos(((2 * tau + tshift - t) / 0.2 / tau) * PI)) / 2;
                      amp = amp * taper;
                  }
              }
              break;
          }
          default:
              sofih_set_error("SOURCE_SHAPE %d is not supported (1 Ricker, 2 Fuchs-Mueller, 3 file, 4 sin^3, "
                              "5 Berlage, 6 Klauder)", shape);
              return 1;
        }
        if (fabs(amp) > sigmax)
            sigmax = fabs(amp);
        sig[n - 1] = amp * a;
    }
    if (0.0 == sigmax) {
        sofih_set_error("source %d: the source signal contains only zeros", k + 1);
        return 1;
    }
    if (shape == 5 || shape == 6) /* normalised to the amplitude */
        for (int n = 0; n < nt; n++)
            sig[n] = sig[n] / sigmax;
    return 0;
}

int sofih_wavelet(int shape, int nt, float dt, int nsrc, const float *srcpos, float *signals)
{
    if (shape == 3) {
        sofih_set_error("SOURCE_SHAPE 3 reads SIGNAL_FILE: use sofih_wavelet_file");
        return 1;
    }
    for (int k = 0; k < nsrc; k++)
        if (one_wavelet(shape, nt, dt, nsrc, k, srcpos, NULL, 0, signals + (size_t)k * nt))
            return 1;
    return 0;
}

int sofih_read_signal(const char *path, float dt, float **samples, int *ns)
{
    *samples = NULL, *ns = 0;
    float sdt = 0.f;
    int dt_found = 0;
    float *sig = NULL;
    FILE *fp = NULL;
    /* the file type from the name: ".su" anywhere (case-insensitive) is SU,
     * anything else is ASCII (read_srcsig.c:55-62) */
    char low[1024];
    size_t L = strlen(path);
    if (L >= sizeof low)
        L = sizeof low - 1;
    for (size_t c = 0; c < L; c++)
        low[c] = (char)((path[c] >= 'A' && path[c] <= 'Z') ? path[c] - 'A' + 'a' : path[c]);
    low[L] = 0;
    if (strstr(low, ".su")) {
        fp = fopen(path, "rb");
        if (!fp) {
            sofih_set_error("cannot open signal file %s", path);
            return 1;
        }
        unsigned char h[240];
        if (fread(h, 1, 240, fp) != 240) {
            fclose(fp);
            sofih_set_error("short read in SU file %s", path);
            return 1;
        }
        unsigned short suns, sudt;
        short delrt;
        memcpy(&delrt, h + 108, 2), memcpy(&suns, h + 114, 2), memcpy(&sudt, h + 116, 2);
        if (suns < 1 || delrt != 0) {
            fclose(fp);
            sofih_set_error("SU signal file %s: no samples, or a delay recording time (unsupported)", path);
            return 1;
        }
        sig = (float *)calloc(suns, sizeof(float));
        if (fread(sig, sizeof(float), suns, fp) != suns) {
            fclose(fp), free(sig);
            sofih_set_error("short read in SU file %s", path);
            return 1;
        }
        fclose(fp);
        *ns = suns;
        if (sudt > 0)
            sdt = sudt * 1e-6, dt_found = 1;
    } else {
        fp = fopen(path, "r");
        if (!fp) {
            sofih_set_error("cannot open signal file %s", path);
            return 1;
        }
        char line[256];
        int n = 0;
        /* first pass: count samples; a comment line "# ... DT ... = <value>" gives the interval */
        while (fgets(line, sizeof line, fp)) {
            char *q = line;
            while (*q == ' ' || *q == '\t' || *q == '\n' || *q == '\r' || *q == '\v' || *q == '\f')
                q++;
            if (!*q)
                continue;
            if (*q == '#') {
                char lc[256];
                size_t m = strlen(q + 1);
                for (size_t c = 0; c <= m; c++)
                    lc[c] = (char)((q[1 + c] >= 'A' && q[1 + c] <= 'Z') ? q[1 + c] - 'A' + 'a' : q[1 + c]);
                if (!strstr(lc, "dt") || !strchr(q + 1, '='))
                    continue;
                char *v = strchr(q + 1, '=') + 1;
                while (*v == ' ' || *v == '\t')
                    v++;
                if (sscanf(v, "%e", &sdt) == 1)
                    dt_found = 1;
                continue;
            }
            n++;
        }
        if (!n) {
            fclose(fp);
            sofih_set_error("signal file %s holds no samples", path);
            return 1;
        }
        sig = (float *)calloc((size_t)n, sizeof(float));
        rewind(fp);
        int i = 0;
        while (fgets(line, sizeof line, fp) && i < n) {
            char *q = line;
            while (*q == ' ' || *q == '\t' || *q == '\n' || *q == '\r' || *q == '\v' || *q == '\f')
                q++;
            if (!*q || *q == '#')
                continue;
            if (sscanf(q, "%e", &sig[i]) != 1)
                sig[i] = 0.0f;
            i++;
        }
        fclose(fp);
        *ns = n;
    }
    if (dt_found && sdt != dt) {
        free(sig);
        sofih_set_error("signal file %s: sampling interval %g s differs from DT %g s", path, sdt, dt);
        return 1;
    }
    *samples = sig;
    return 0;
}

int sofih_wavelet_file(const char *signal_file, int nt, float dt, int nsrc, const float *srcpos, float *signals)
{
    float *f = NULL;
    int nf = 0;
    if (sofih_read_signal(signal_file, dt, &f, &nf))
        return 1;
    int rc = 0;
    for (int k = 0; k < nsrc && !rc; k++)
        rc = one_wavelet(3, nt, dt, nsrc, k, srcpos, f, nf, signals + (size_t)k * nt);
    free(f);
    return rc;
}

typedef struct {
    int *x, *y, *t;
    int n, cap;
} reclist;

static int rec_push(reclist *r, int x, int y, int t)
{
    if (r->n == r->cap) {
        const int cap = r->cap ? 2 * r->cap : 64;
        int *nx = (int *)realloc(r->x, sizeof(int) * cap), *ny = (int *)realloc(r->y, sizeof(int) * cap),
            *nt = (int *)realloc(r->t, sizeof(int) * cap);
        if (nx)
            r->x = nx;
        if (ny)
            r->y = ny;
        if (nt)
            r->t = nt;
        if (!nx || !ny || !nt) {
            sofih_set_error("out of host memory");
            return 1;
        }
        r->cap = cap;
    }
    r->x[r->n] = x, r->y[r->n] = y, r->t[r->n] = t;
    r->n++;
    return 0;
}

int sofih_read_receiver_traces(const sofih_par *p, const char *path, int **ix, int **iy, int **trace, int *ntr)
{
    reclist r = {0};
    int rc = 0;
    if (p->readrec) { /* receiver.c:41-99 */
        int *topo = NULL;
        if (p->rec_topo) {
            topo = (int *)malloc(sizeof(int) * (size_t)p->nx);
            if (!topo || sofih_scan_topo(p, p->mfile, topo)) {
                free(topo);
                return 1;
            }
        }
        FILE *fp = fopen(path, "r");
        if (!fp) {
            free(topo);
            sofih_set_error("cannot open receiver file %s", path);
            return 1;
        }
        char line[512];
        int itr = 0;
        while (!rc && fgets(line, sizeof line, fp)) {
            if (!is_data_line(line, 1))
                continue;
            float xr, yr;
            if (sscanf(line, "%f%f", &xr, &yr) != 2)
                continue;
            itr++;
            const int x = (int)floor((xr + p->refrec[0]) / p->dh) + 1;
            int y;
            if (topo) { /* receiver.c:68-70: the depth counted from the column's topography */
                if (x < 1 || x > p->nx) {
                    sofih_set_error("%s: receiver %d lies outside the model's columns", path, itr);
                    rc = 1;
                    break;
                }
                y = topo[x - 1] + (int)floor(yr / p->dh);
            } else {
                y = (int)floor((yr + p->refrec[1]) / p->dh) + 1;
            }
            rc = rec_push(&r, x, y, itr);
        }
        fclose(fp);
        free(topo);
        /* co-located receivers: the first keeps the grid point, its trace number stays */
        int m = 0;
        for (int k = 0; k < r.n && !rc; k++) {
            int dup = 0;
            for (int q = 0; q < m && !dup; q++)
                dup = (r.x[q] == r.x[k] && r.y[q] == r.y[k]);
            if (!dup)
                r.x[m] = r.x[k], r.y[m] = r.y[k], r.t[m] = r.t[k], m++;
        }
        r.n = m;
    } else if (p->rec_array > 0) { /* receiver.c:101-116: receiver planes */
        int itr = 0;
        for (int n = 0; n <= p->rec_array - 1 && !rc; n++) {
            const float depth = p->rec_array_depth + p->rec_array_dist * (float)n;
            const int j = IROUND(depth / p->dh);
            for (int i = p->fw; i <= p->nx - p->fw && !rc; i += p->drx)
                rc = rec_push(&r, i, j, ++itr);
        }
    } else { /* receiver.c:117-164: one point, or a horizontal or vertical line */
        const int x1 = (int)floor(p->xrec1 / p->dh) + 1, y1 = (int)floor(p->yrec1 / p->dh) + 1;
        const int x2 = (int)floor(p->xrec2 / p->dh) + 1, y2 = (int)floor(p->yrec2 / p->dh) + 1;
        const int step = p->ngeoph > 0 ? p->ngeoph : 1;
        if (y1 != y2 && x1 != x2) {
            sofih_set_error("no horizontal or vertical receiver line: an oblique one needs a receiver file (READREC 1)");
            return 1;
        }
        const int len = (y1 == y2) ? x2 - x1 : y2 - y1;
        for (int k = 0, itr = 1; k <= len && !rc; k += step, itr++)
            rc = rec_push(&r, (y1 == y2) ? x1 + k : x1, (y1 == y2) ? y1 : y1 + k, itr);
    }
    if (rc) {
        free(r.x), free(r.y), free(r.t);
        return 1;
    }
    for (int k = 0; k < r.n; k++) { /* receiver.c:166-171 */
        if (r.x[k] == 0)
            r.x[k] = 1;
        if (r.y[k] == 0)
            r.y[k] = 1;
    }
    if (!r.n) /* callers free what they get */
        rc = rec_push(&r, 0, 0, 0), r.n = 0;
    *ix = r.x, *iy = r.y, *trace = r.t, *ntr = r.n;
    return rc;
}

int sofih_read_receivers(const sofih_par *p, const char *path, int **ix, int **iy, int *ntr)
{
    int *trace = NULL;
    const int rc = sofih_read_receiver_traces(p, path, ix, iy, &trace, ntr);
    free(trace);
    return rc;
}

/* SEG-Y trace header fields written by outseis_glob.c:46-81 (byte offsets of
 * the standard 240-byte header). */
static void put_i32(unsigned char *h, int off, int v) { memcpy(h + off, &v, 4); }
static void put_i16(unsigned char *h, int off, short v) { memcpy(h + off, &v, 2); }
static void put_u16(unsigned char *h, int off, unsigned short v) { memcpy(h + off, &v, 2); }
static void put_f32(unsigned char *h, int off, float v) { memcpy(h + off, &v, 4); }

/* SU traces as outseis_glob.c:40-82 writes them; tracl_of[t] is the trace
 * number field (recpos[3]), NULL for 1..ntr. */
static int write_su_traces(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                           const int *tracl_of, float xs, float ys, const sofih_par *p, int ishot)
{
    if (ns > 65535) { /* checkfd.c:119-122: the SU header holds ns in 16 bits */
        sofih_set_error("%s: %d samples per trace, at most 65535 in SU format (SEIS_FORMAT 2 or 3 have no limit)",
                        path, ns);
        return 1;
    }
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        sofih_set_error("cannot write %s", path);
        return 1;
    }
    const float xshift = 800.0, yshift = 800.0;
    for (int t = 0; t < ntr; t++) {
        unsigned char h[240];
        memset(h, 0, sizeof h);
        float xr = (ix[t] - 1) * p->dh, yr = (iy[t] - 1) * p->dh;
        float x = xr - p->refrec[0], y = yr - p->refrec[1];
        int tracl = tracl_of ? tracl_of[t] : t + 1;
        put_i32(h, 0, tracl);                                                   /* tracl */
        put_i32(h, 4, tracl);                                                   /* tracr */
        put_i32(h, 8, ishot);                                                   /* fldr */
        put_i32(h, 12, t + 1);                                                  /* tracf */
        put_i32(h, 16, ishot);                                                  /* ep */
        put_i32(h, 20, tracl);                                                  /* cdp */
        put_i16(h, 28, 1);                                                      /* trid */
        put_i32(h, 36, IROUND(sqrt((xs - xr) * (xs - xr) + (ys - yr) * (ys - yr)))); /* offset */
        put_i32(h, 40, IROUND(yr * 1000.0));                                    /* gelev */
        put_i32(h, 48, IROUND(ys * 1000.0));                                    /* sdepth */
        put_i32(h, 60, IROUND(((360.0 / (2.0 * PI)) * atan2(x - xshift, y - yshift)) * 1000.0)); /* swdep */
        put_i16(h, 68, -1000);                                                  /* scalel */
        put_i16(h, 70, -1000);                                                  /* scalco */
        put_i32(h, 72, IROUND(xs * 1000.0));                                    /* sx */
        put_i32(h, 80, IROUND(xr * 1000.0));                                    /* gx */
        put_u16(h, 114, (unsigned short)ns);                                    /* ns */
        unsigned short dt_us = (unsigned short)IROUND((float)p->ndt * p->dt * 1.0e6);
        put_u16(h, 116, dt_us);                                                 /* dt */
        put_f32(h, 180, (float)dt_us * 1.0e-6);                                 /* d1 */
        if (fwrite(h, 1, 240, fp) != 240 || fwrite(section + (size_t)t * ns, sizeof(float), ns, fp) != (size_t)ns) {
            fclose(fp);
            sofih_set_error("short write on %s", path);
            return 1;
        }
    }
    fclose(fp);
    return 0;
}

int sofih_write_su(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                   float xs, float ys, const sofih_par *p, int ishot, int comp)
{
    (void)comp; /* outseis_glob.c:55,79: ep is set to comp, then to ishot */
    return write_su_traces(path, section, ntr, ns, ix, iy, NULL, xs, ys, p, ishot);
}

int sofih_snapshot_shots(const sofih_par *p, int nshots, int *shots)
{
    int n = 0;
    for (int s = 1; s <= nshots && p->snap > 0 && p->snapshot_incr > 0; s++)
        if ((s - p->snapshot_start) % p->snapshot_incr == 0 && s <= p->snapshot_start)
            shots[n++] = s;
    return n;
}

int sofih_write_su_traces(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                          const int *trace, float xs, float ys, const sofih_par *p, int ishot, int comp)
{
    (void)comp;
    return write_su_traces(path, section, ntr, ns, ix, iy, trace, xs, ys, p, ishot);
}

int sofih_write_signal(const sofih_par *p, int ishot, const float *signal, int nt, int ix, int iy, float xs,
                       float ys, char *path_out, int path_len)
{
    static const char *ext[4] = {"", "su", "txt", "bin"};
    int fmt = p->sigout_format;
    if (fmt < 1 || fmt > 3) {
        sofih_set_error("Unknown SIGOUT_FORMAT %d", fmt);
        return 1;
    }
    char path[600];
    snprintf(path, sizeof path, "%s.shot%d.%s", p->sigout_file, ishot, ext[fmt]);
    if (path_out && path_len > 0)
        snprintf(path_out, (size_t)path_len, "%s", path);
    if (fmt == 1) {
        const int zero = 0; /* initsrc.c:82: the dummy receiver's trace number */
        return write_su_traces(path, signal, 1, nt, &ix, &iy, &zero, xs, ys, p, ishot);
    }
    FILE *fp = fopen(path, fmt == 2 ? "w" : "wb");
    if (!fp) {
        sofih_set_error("cannot write %s", path);
        return 1;
    }
    int bad = 0;
    for (int k = 0; k < nt && !bad; k++)
        bad = fmt == 2 ? fprintf(fp, "%e\n", signal[k]) < 0 : fwrite(signal + k, sizeof(float), 1, fp) != 1;
    if (fclose(fp) || bad) {
        sofih_set_error("short write on %s", path);
        return 1;
    }
    return 0;
}

int sofih_write_snap_format(const char *path, const float *frame, int n, int append, int format)
{
    if (format == 3)
        return sofih_write_snap(path, frame, n, append);
    if (format != 2) {
        sofih_set_error(format == 1 ? "SNAP_FORMAT 1: the SU format for snapshots is not implemented (nor by "
                                      "the reference)"
                                    : "unknown SNAP_FORMAT %d",
                        format);
        return 1;
    }
    FILE *fp = fopen(path, append ? "a" : "w");
    if (!fp) {
        sofih_set_error("cannot write %s", path);
        return 1;
    }
    int bad = 0;
    for (int k = 0; k < n && !bad; k++)
        bad = fprintf(fp, "%e\n", frame[k]) < 0;
    bad |= fclose(fp) != 0;
    if (bad)
        sofih_set_error("short write on %s", path);
    return bad;
}

const char *sofih_seis_ext(int format)
{
    switch (format) {
      case 1:
          return "su";
      case 2:
          return "txt";
      case 3:
          return "bin";
      case 0:
      case 4:
      case 5:
          return "sgy";
    }
    return NULL;
}

int sofih_write_seis(const char *path, const float *section, int ntr, int ns, const int *ix, const int *iy,
                     const int *trace, float xs, float ys, const sofih_par *p, int ishot, int comp)
{
    if (p->seis_format == 1)
        return sofih_write_su_traces(path, section, ntr, ns, ix, iy, trace, xs, ys, p, ishot, comp);
    FILE *fp = fopen(path, p->seis_format == 2 ? "w" : "wb");
    if (!fp) {
        sofih_set_error("cannot write %s", path);
        return 1;
    }
    int bad = 0;
    const size_t n = (size_t)ntr * (size_t)ns;
    if (p->seis_format == 2)
        for (size_t k = 0; k < n && !bad; k++)
            bad = fprintf(fp, "%e\n", section[k]) < 0;
    else if (p->seis_format == 3)
        bad = fwrite(section, sizeof(float), n, fp) != n;
    bad |= fclose(fp) != 0;
    if (bad)
        sofih_set_error("short write on %s", path);
    return bad;
}

int sofih_write_snap(const char *path, const float *frame, int n, int append)
{
    FILE *fp = fopen(path, append ? "ab" : "wb");
    if (!fp) {
        sofih_set_error("cannot write %s", path);
        return 1;
    }
    size_t w = fwrite(frame, sizeof(float), (size_t)n, fp);
    fclose(fp);
    if (w != (size_t)n) {
        sofih_set_error("short write on %s", path);
        return 1;
    }
    return 0;
}

/* Holberg / Taylor operator coefficients (published tables; reference
 * holbergcoeff.c:40-82): row MAXRELERROR, FDORDER/2 - 1; hc[0] is the
 * operator's points-per-wavelength figure, hc[1..6] the coefficients. */
static const double HOLBERG[5][6][7] = {
    {{23.0, 1.0, 0, 0, 0, 0, 0}, {8.0, 9.0 / 8.0, -1.0 / 24.0, 0, 0, 0, 0},
     {6.0, 75.0 / 64.0, -25.0 / 384.0, 3.0 / 640.0, 0, 0, 0},
     {5.0, 1225.0 / 1024.0, -245.0 / 3072.0, 49.0 / 5120.0, -5.0 / 7168.0, 0, 0},
     {5.0, 19845.0 / 16384.0, -735.0 / 8192.0, 567.0 / 40960.0, -405.0 / 229376.0, 35.0 / 294912.0, 0},
     {4.0, 160083.0 / 131072.0, -12705.0 / 131072.0, 22869.0 / 1310720.0, -5445.0 / 1835008.0,
      847.0 / 2359296.0, -63.0 / 2883584.0}},
    {{49.7, 1.0010, 0, 0, 0, 0, 0}, {8.32, 1.1382, -0.046414, 0, 0, 0, 0},
     {4.77, 1.1965, -0.078804, 0.0081781, 0, 0, 0}, {3.69, 1.2257, -0.099537, 0.018063, -0.0026274, 0, 0},
     {3.19, 1.2415, -0.11231, 0.026191, -0.0064682, 0.001191, 0},
     {2.91, 1.2508, -0.12034, 0.032131, -0.010142, 0.0029857, -0.00066667}},
    {{22.2, 1.0050, 0, 0, 0, 0, 0}, {5.65, 1.1534, -0.052806, 0, 0, 0, 0},
     {3.74, 1.2111, -0.088313, 0.011768, 0, 0, 0}, {3.11, 1.2367, -0.10815, 0.023113, -0.0046905, 0, 0},
     {2.80, 1.2496, -0.11921, 0.031130, -0.0093272, 0.0025161, 0},
     {2.62, 1.2568, -0.12573, 0.036423, -0.013132, 0.0047484, -0.0015979}},
    {{15.8, 1.0100, 0, 0, 0, 0, 0}, {4.80, 1.1640, -0.057991, 0, 0, 0, 0},
     {3.39, 1.2192, -0.094070, 0.014608, 0, 0, 0}, {2.90, 1.2422, -0.11269, 0.026140, -0.0064054, 0, 0},
     {2.65, 1.2534, -0.12257, 0.033755, -0.011081, 0.0036784, 0},
     {2.51, 1.2596, -0.12825, 0.038550, -0.014763, 0.0058619, -0.0024538}},
    {{9.16, 1.0300, 0, 0, 0, 0, 0}, {3.47, 1.1876, -0.072518, 0, 0, 0, 0},
     {2.91, 1.2341, -0.10569, 0.022589, 0, 0, 0}, {2.61, 1.2516, -0.12085, 0.032236, -0.011459, 0, 0},
     {2.45, 1.2596, -0.12829, 0.038533, -0.014681, 0.0072580, 0},
     {2.36, 1.2640, -0.13239, 0.042217, -0.017803, 0.0081959, -0.0051848}},
};

int sofih_holberg(int fdorder, int maxrelerror, float *hc)
{
    if (fdorder < 2 || fdorder > 12 || (fdorder & 1) || maxrelerror < 0 || maxrelerror > 4) {
        sofih_set_error("no FD coefficients for FDORDER %d, MAXRELERROR %d", fdorder, maxrelerror);
        return 1;
    }
    for (int k = 0; k < 7; k++)
        hc[k] = (float)HOLBERG[maxrelerror][fdorder / 2 - 1][k];
    return 0;
}

/* checkfd.c:41-52: DT must not exceed DH / (sqrt(2) * gamma * cmax) with
 * gamma = sum |hc[1..6]| and cmax the largest velocity of the model. */
int sofih_check_cfl(const sofih_par *p, const sofih_prep *m, float *dt_max)
{
    float hc[7];
    if (sofih_holberg(p->fdorder, p->maxrelerror, hc))
        return 1;
    float vpmin, vpmax, vsmin, vsmax;
    sofih_prep_vrange(m, &vpmin, &vpmax, &vsmin, &vsmax);
    float cmax = vsmax > vpmax ? vsmax : vpmax;
    double gamma = 0;
    for (int k = 1; k <= 6; k++)
        gamma += fabs(hc[k]);
    double lim = p->dh / (sqrt(2) * gamma * cmax);
    *dt_max = (float)lim;
    if (p->dt > lim) {
        sofih_set_error("unstable: DT=%g exceeds the stability limit %g (VMAX=%g)", p->dt, lim, cmax);
        return 1;
    }
    return 0;
}
