/*
 * sofiserve.c -- continuous-batching request loop over libsofigpu (one GPU).
 *
 * Threads: the caller's thread drives the loop (sofi_server_poll/_drain) and
 * is the only one that touches GPU contexts; `prep_threads` workers turn
 * arrived requests into prepared models (sofih_prepare: readmod_*.c, prepmod.c,
 * PML_pro.c of the reference) and wavelets (wavelet.c). All request state is
 * guarded by one mutex; GPU calls run outside it.
 */
#include "sofiserve.h"
#include "sofigpu.h"

#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>

static __thread char g_err[512];

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
    return code;
}

const char *sofi_server_last_error(void) { return g_err; }

typedef struct {
    sofi_request r;
    int id, state, status;
    char error[256];
    double arrival, ready, admitted, finished;
    sofih_prep *prep;
    float *signals;         /* [nsrc][NT] */
    sofi_config cfg;
    long long bytes;
    int priority;
    sofi_ctx *ctx;
    int issued;             /* time steps queued on the GPU */
    long long launches;
    int ns, ncomp, comps[5];
    float *sec[6];          /* host sections by component, [ntr][ns] */
} req_t;

struct sofi_server {
    sofi_server_options o;
    struct timespec t0;
    pthread_mutex_t mu;
    pthread_cond_t cv;      /* workers wait here for arrivals */
    req_t **reqs;
    int n, cap;
    pthread_t *workers;
    int nworkers, stop;
    long long in_use, peak_bytes;
    int resident, peak_resident;
    int prio_least, prio_greatest;
};

double sofi_server_clock(const sofi_server *s)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)(t.tv_sec - s->t0.tv_sec) + 1e-9 * (double)(t.tv_nsec - s->t0.tv_nsec);
}

/* ---- policy ------------------------------------------------------------ */

int sofi_server_plan(const long long *bytes, int n, long long in_use, long long budget, int resident,
                     int max_resident, int *admit)
{
    int k, m = 0;
    for (k = 0; k < n; k++) {
        admit[k] = 0;
        if (resident + m >= max_resident)
            continue;
        if (in_use + bytes[k] <= budget) {
            admit[k] = 1;
            in_use += bytes[k];
            m++;
        }
    }
    return m;
}

int sofi_server_priority(double cell_updates, int least, int greatest)
{
    /* greatest <= least (CUDA: lower is more urgent) */
    double w = cell_updates > 1.0 ? log2(cell_updates) : 0.0;
    int level = w <= 30.0 ? 0 : (int)((w - 30.0) / 2.0);
    int p = greatest + level;
    return p > least ? least : p;
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

double sofi_server_percentile(const double *x, int n, double q)
{
    if (n <= 0)
        return 0.0;
    double *t = (double *)malloc(sizeof(double) * (size_t)n);
    if (!t)
        return 0.0;
    memcpy(t, x, sizeof(double) * (size_t)n);
    qsort(t, (size_t)n, sizeof(double), cmp_double);
    if (q < 0.0)
        q = 0.0;
    if (q > 1.0)
        q = 1.0;
    int rank = (int)ceil(q * n); /* nearest rank, 1-based */
    if (rank < 1)
        rank = 1;
    double v = t[rank - 1];
    free(t);
    return v;
}

/* ---- preparation (worker threads) ---------------------------------------- */

static void components(int seismo, int *comps, int *nc)
{
    *nc = 0;
    if (seismo == 1)
        comps[(*nc)++] = SOFI_COMP_VX, comps[(*nc)++] = SOFI_COMP_VY;
    if (seismo == 2)
        comps[(*nc)++] = SOFI_COMP_P;
    if (seismo == 3)
        comps[(*nc)++] = SOFI_COMP_DIV, comps[(*nc)++] = SOFI_COMP_CURL;
    if (seismo == 4)
        for (int k = 1; k <= 5; k++)
            comps[(*nc)++] = k;
}

/* Everything the GPU needs of one request, built on a worker thread. */
static int prepare_request(const sofi_server *s, req_t *q)
{
    const sofih_par *p = &q->r.par;
    int rc = sofih_prepare(p, q->r.vp, q->r.vs, q->r.rho, q->r.qp, q->r.qs, q->r.eps, q->r.del, q->r.theta,
                           s->o.prep_omp_threads, &q->prep);
    if (rc)
        return fail(SOFI_E_ARG, "preparation: %s", sofih_last_error());
    float dt_max = 0.f;
    if (sofih_check_cfl(p, q->prep, &dt_max))
        return fail(SOFI_E_ARG, "DT=%g exceeds the stability bound %g (checkfd.c)", p->dt, dt_max);
    if (q->r.nsrc > 0) {
        q->signals = (float *)malloc(sizeof(float) * (size_t)q->r.nsrc * (size_t)p->nt);
        if (!q->signals)
            return fail(SOFI_E_NOMEM, "host memory for %d wavelets", q->r.nsrc);
        if (p->source_shape == 3 ? sofih_wavelet_file(p->signal_file, p->nt, p->dt, q->r.nsrc, q->r.srcpos, q->signals)
                                 : sofih_wavelet(p->source_shape, p->nt, p->dt, q->r.nsrc, q->r.srcpos, q->signals))
            return fail(SOFI_E_ARG, "wavelet: %s", sofih_last_error());
    }
    sofi_config *c = &q->cfg;
    memset(c, 0, sizeof *c);
    c->weq = p->weq, c->nx = p->nx, c->ny = p->ny, c->fdorder = p->fdorder, c->maxrelerror = p->maxrelerror;
    c->L = p->L, c->dt = p->dt, c->dh = p->dh, c->nt = p->nt, c->fw = p->fw, c->abs_type = p->abs_type;
    c->free_surf = p->free_surf, c->boundary = p->boundary, c->seismo = q->r.ntr > 0 ? p->seismo : 0;
    c->ndt = p->ndt > 0 ? p->ndt : 1;
    c->idx = c->idy = 1, c->nshots = 1, c->shared_model = 1;
    c->fdorder_time = p->fdorder_time;
    if ((rc = sofi_device_bytes(c, &q->bytes)))
        return fail(rc, "%s", sofi_last_error());
    components(c->seismo, q->comps, &q->ncomp);
    q->ns = c->seismo ? c->nt / c->ndt : 0;
    return 0;
}

static void release_prep(req_t *q)
{
    if (q->prep)
        sofih_prep_free(q->prep);
    q->prep = NULL;
    free(q->signals);
    q->signals = NULL;
}

static void *worker_main(void *arg)
{
    sofi_server *s = (sofi_server *)arg;
    pthread_mutex_lock(&s->mu);
    while (!s->stop) {
        double now = sofi_server_clock(s), next = -1.0;
        req_t *pick = NULL;
        double most = -1.0;
        for (int k = 0; k < s->n; k++) {
            req_t *q = s->reqs[k];
            if (q->state != SOFI_REQ_WAITING)
                continue;
            if (q->arrival <= now) {
                if (!s->o.largest_first) {
                    pick = q;
                    break;
                }
                const double work = (double)q->r.par.nx * (double)q->r.par.ny * (double)q->r.par.nt;
                if (work > most)
                    most = work, pick = q;
                continue;
            }
            if (next < 0.0 || q->arrival < next)
                next = q->arrival;
        }
        if (!pick) {
            if (next < 0.0) {
                pthread_cond_wait(&s->cv, &s->mu);
            } else {
                struct timespec ts;
                clock_gettime(CLOCK_MONOTONIC, &ts);
                double dt = next - now;
                ts.tv_sec += (time_t)dt;
                ts.tv_nsec += (long)((dt - floor(dt)) * 1e9);
                if (ts.tv_nsec >= 1000000000L)
                    ts.tv_sec++, ts.tv_nsec -= 1000000000L;
                pthread_cond_timedwait(&s->cv, &s->mu, &ts);
            }
            continue;
        }
        pick->state = SOFI_REQ_PREPARING;
        pthread_mutex_unlock(&s->mu);
        int rc = prepare_request(s, pick);
        char msg[256];
        if (rc) {
            snprintf(msg, sizeof msg, "%.250s", g_err);
            release_prep(pick);
        }
        pthread_mutex_lock(&s->mu);
        pick->ready = sofi_server_clock(s);
        if (rc) {
            pick->state = SOFI_REQ_FAILED, pick->status = rc, pick->finished = pick->ready;
            snprintf(pick->error, sizeof pick->error, "%s", msg);
        } else {
            pick->state = SOFI_REQ_READY;
        }
    }
    pthread_mutex_unlock(&s->mu);
    return NULL;
}

/* ---- lifecycle ----------------------------------------------------------- */

void sofi_server_default_options(sofi_server_options *o)
{
    memset(o, 0, sizeof *o);
    o->device = 0;
    o->max_resident = 64;
    o->chunk_steps = 32;
    o->depth = 2;
    o->prep_threads = 2;
    o->use_priorities = 1;
}

int sofi_server_create(const sofi_server_options *opt, sofi_server **out)
{
    if (!out)
        return fail(SOFI_E_ARG, "null output pointer");
    *out = NULL;
    sofi_server_options o;
    if (opt)
        o = *opt;
    else
        sofi_server_default_options(&o);
    if (o.max_resident <= 0)
        o.max_resident = 64;
    if (o.chunk_steps <= 0)
        o.chunk_steps = 32;
    if (o.depth <= 0)
        o.depth = 2;
    if (o.prep_threads <= 0)
        o.prep_threads = 2;
    if (o.prep_omp_threads <= 0) {
        long nc = sysconf(_SC_NPROCESSORS_ONLN);
        o.prep_omp_threads = nc > o.prep_threads ? (int)(nc / o.prep_threads) : 1;
    }
    long long fr = 0, tot = 0;
    int rc = sofi_device_memory(o.device, &fr, &tot);
    if (rc)
        return fail(rc, "%s", sofi_last_error());
    if (o.hbm_budget <= 0)
        o.hbm_budget = (long long)(0.9 * (double)fr);
    sofi_server *s = (sofi_server *)calloc(1, sizeof *s);
    if (!s)
        return fail(SOFI_E_NOMEM, "host memory");
    s->o = o;
    if ((rc = sofi_stream_priority_range(o.device, &s->prio_least, &s->prio_greatest))) {
        free(s);
        return fail(rc, "%s", sofi_last_error());
    }
    clock_gettime(CLOCK_MONOTONIC, &s->t0);
    pthread_mutex_init(&s->mu, NULL);
    pthread_condattr_t ca;
    pthread_condattr_init(&ca);
    pthread_condattr_setclock(&ca, CLOCK_MONOTONIC);
    pthread_cond_init(&s->cv, &ca);
    pthread_condattr_destroy(&ca);
    s->workers = (pthread_t *)calloc((size_t)o.prep_threads, sizeof(pthread_t));
    for (int k = 0; k < o.prep_threads; k++)
        if (pthread_create(&s->workers[k], NULL, worker_main, s) == 0)
            s->nworkers++;
    if (!s->nworkers) {
        sofi_server_destroy(s);
        return fail(SOFI_E_STATE, "no preparation thread could be started");
    }
    *out = s;
    return 0;
}

static void free_request(req_t *q)
{
    if (q->ctx)
        sofi_destroy(q->ctx);
    release_prep(q);
    for (int k = 0; k < 6; k++)
        free(q->sec[k]);
    free(q);
}

int sofi_server_destroy(sofi_server *s)
{
    if (!s)
        return 0;
    pthread_mutex_lock(&s->mu);
    s->stop = 1;
    pthread_cond_broadcast(&s->cv);
    pthread_mutex_unlock(&s->mu);
    for (int k = 0; k < s->nworkers; k++)
        pthread_join(s->workers[k], NULL);
    for (int k = 0; k < s->n; k++)
        free_request(s->reqs[k]);
    free(s->reqs);
    free(s->workers);
    pthread_cond_destroy(&s->cv);
    pthread_mutex_destroy(&s->mu);
    free(s);
    return 0;
}

int sofi_server_submit(sofi_server *s, const sofi_request *r, int *id)
{
    if (!s || !r || !id)
        return fail(SOFI_E_ARG, "null argument");
    const sofih_par *p = &r->par;
    if (p->nx <= 0 || p->ny <= 0 || p->nt <= 0 || !r->vp || !r->vs || !r->rho)
        return fail(SOFI_E_ARG, "request needs NX, NY, NT > 0 and vp, vs, rho");
    if ((r->nsrc > 0 && !r->srcpos) || (r->ntr > 0 && (!r->rec_ix || !r->rec_iy)))
        return fail(SOFI_E_ARG, "sources or receivers missing");
    if (p->snap)
        return fail(SOFI_E_ARG, "snapshots are not served");
    req_t *q = (req_t *)calloc(1, sizeof *q);
    if (!q)
        return fail(SOFI_E_NOMEM, "host memory");
    q->r = *r;
    pthread_mutex_lock(&s->mu);
    if (s->n == s->cap) {
        int cap = s->cap ? 2 * s->cap : 64;
        req_t **t = (req_t **)realloc(s->reqs, sizeof(req_t *) * (size_t)cap);
        if (!t) {
            pthread_mutex_unlock(&s->mu);
            free(q);
            return fail(SOFI_E_NOMEM, "host memory");
        }
        s->reqs = t, s->cap = cap;
    }
    double now = sofi_server_clock(s);
    q->arrival = r->arrival < 0.0 ? now : r->arrival;
    q->id = s->n;
    q->state = SOFI_REQ_WAITING;
    s->reqs[s->n++] = q;
    *id = q->id;
    pthread_cond_broadcast(&s->cv);
    pthread_mutex_unlock(&s->mu);
    return 0;
}

/* ---- the loop (caller's thread) ------------------------------------------ */

static const char *kVectors[] = {"K_x", "a_x", "b_x", "K_x_half", "a_x_half", "b_x_half", "K_y", "a_y", "b_y",
                                 "K_y_half", "a_y_half", "b_y_half", "bip", "cip", "peta"};

/* Create the context of a prepared request and upload its model and
 * acquisition; on failure the context is destroyed again. */
static int make_resident(sofi_server *s, req_t *q)
{
    int rc;
    double work = (double)q->cfg.nx * (double)q->cfg.ny * (double)q->cfg.nt;
    q->priority = s->o.use_priorities ? sofi_server_priority(work, s->prio_least, s->prio_greatest) : 0;
    if ((rc = sofi_create_with_priority(&q->cfg, s->o.device, q->priority, &q->ctx)))
        return rc;
    /* solves share the GPU: no blocks parked waiting for their predecessor */
    rc = sofi_set_pdl(q->ctx, 0);
    for (int k = 0; k < sofih_prep_num_fields(q->prep) && !rc; k++)
        rc = sofi_set_model_field(q->ctx, 0, sofih_prep_field_name(q->prep, k), sofih_prep_field(q->prep, k),
                                  q->cfg.nx, 1);
    for (size_t k = 0; k < sizeof kVectors / sizeof kVectors[0] && !rc; k++) {
        const float *d;
        int n = sofih_prep_vector(q->prep, kVectors[k], &d);
        if (n)
            rc = sofi_set_model_vector(q->ctx, kVectors[k], d, n);
    }
    if (!rc)
        rc = sofi_set_sources(q->ctx, 0, q->r.nsrc, q->r.srcpos, q->signals);
    if (!rc && q->cfg.seismo)
        rc = sofi_set_receivers(q->ctx, 0, q->r.ntr, q->r.rec_ix, q->r.rec_iy);
    if (!rc)
        rc = sofi_reset(q->ctx, -1);
    if (rc) {
        sofi_destroy(q->ctx);
        q->ctx = NULL;
    }
    return rc;
}

/* Copy the sections of a finished request to the host and free its context. */
static int retire(req_t *q)
{
    int rc = sofi_synchronize(q->ctx);
    if (!rc)
        rc = sofi_launch_count(q->ctx, &q->launches);
    for (int k = 0; k < q->ncomp && !rc; k++) {
        int c = q->comps[k];
        q->sec[c] = (float *)malloc(sizeof(float) * (size_t)q->r.ntr * (size_t)(q->ns > 0 ? q->ns : 1));
        if (!q->sec[c])
            rc = fail(SOFI_E_NOMEM, "host memory for a section");
        else
            rc = sofi_get_section(q->ctx, 0, c, q->sec[c]);
    }
    sofi_destroy(q->ctx);
    q->ctx = NULL;
    return rc;
}

int sofi_server_poll(sofi_server *s, int *active)
{
    if (!s)
        return fail(SOFI_E_ARG, "null server");
    int rc = 0, n;
    /* the request list may grow (and move) under concurrent submissions:
     * work on a snapshot of its pointers; only this thread retires or admits */
    pthread_mutex_lock(&s->mu);
    n = s->n;
    req_t **all = (req_t **)malloc(sizeof(req_t *) * (size_t)(n + 1));
    if (!all) {
        pthread_mutex_unlock(&s->mu);
        return fail(SOFI_E_NOMEM, "host memory");
    }
    memcpy(all, s->reqs, sizeof(req_t *) * (size_t)n);
    pthread_mutex_unlock(&s->mu);
    /* 1. retire solves whose last chunk has finished */
    for (int k = 0; k < n; k++) {
        req_t *q = all[k];
        if (q->state != SOFI_REQ_RESIDENT || q->issued < q->cfg.nt)
            continue;
        int pending = 0;
        if ((rc = sofi_pending_runs(q->ctx, &pending))) {
            free(all);
            return fail(rc, "%s", sofi_last_error());
        }
        if (pending)
            continue;
        double t = sofi_server_clock(s);
        int st = retire(q);
        char msg[256];
        if (st)
            snprintf(msg, sizeof msg, "%.250s", sofi_last_error());
        pthread_mutex_lock(&s->mu);
        s->in_use -= q->bytes;
        s->resident--;
        q->finished = t;
        q->status = st;
        q->state = st ? SOFI_REQ_FAILED : SOFI_REQ_DONE;
        if (st)
            snprintf(q->error, sizeof q->error, "%s", msg);
        pthread_mutex_unlock(&s->mu);
    }
    /* 2. admit ready requests, first fit in arrival order */
    pthread_mutex_lock(&s->mu);
    int nready = 0;
    req_t **ready = (req_t **)malloc(sizeof(req_t *) * (size_t)(n + 1));
    long long *bytes = (long long *)malloc(sizeof(long long) * (size_t)(n + 1));
    int *admit = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    if (!ready || !bytes || !admit) {
        pthread_mutex_unlock(&s->mu);
        free(ready), free(bytes), free(admit), free(all);
        return fail(SOFI_E_NOMEM, "host memory");
    }
    for (int k = 0; k < n; k++)
        if (all[k]->state == SOFI_REQ_READY)
            ready[nready] = all[k], bytes[nready++] = all[k]->bytes;
    /* arrival order (submission order breaks ties) */
    for (int a = 1; a < nready; a++)
        for (int b = a; b > 0 && ready[b]->arrival < ready[b - 1]->arrival; b--) {
            req_t *t = ready[b];
            ready[b] = ready[b - 1], ready[b - 1] = t;
            long long u = bytes[b];
            bytes[b] = bytes[b - 1], bytes[b - 1] = u;
        }
    long long in_use = s->in_use;
    int resident = s->resident;
    pthread_mutex_unlock(&s->mu);
    sofi_server_plan(bytes, nready, in_use, s->o.hbm_budget, resident, s->o.max_resident, admit);
    for (int k = 0; k < nready; k++) {
        if (!admit[k])
            continue;
        req_t *q = ready[k];
        /* a solve larger than the whole budget can never be admitted */
        int st = make_resident(s, q);
        double t = sofi_server_clock(s);
        pthread_mutex_lock(&s->mu);
        if (st == SOFI_E_NOMEM && s->resident > 0) {
            /* the device is fuller than the budget says: retry after a retirement */
            pthread_mutex_unlock(&s->mu);
            break;
        }
        if (st) {
            q->state = SOFI_REQ_FAILED, q->status = st, q->finished = t;
            snprintf(q->error, sizeof q->error, "%.250s", sofi_last_error());
        } else {
            q->state = SOFI_REQ_RESIDENT, q->admitted = t;
            s->in_use += q->bytes;
            s->resident++;
            if (s->in_use > s->peak_bytes)
                s->peak_bytes = s->in_use;
            if (s->resident > s->peak_resident)
                s->peak_resident = s->resident;
        }
        pthread_mutex_unlock(&s->mu);
        release_prep(q);
    }
    /* requests that can never fit fail instead of waiting forever */
    pthread_mutex_lock(&s->mu);
    for (int k = 0; k < nready; k++)
        if (ready[k]->state == SOFI_REQ_READY && ready[k]->bytes > s->o.hbm_budget) {
            req_t *q = ready[k];
            q->state = SOFI_REQ_FAILED, q->status = SOFI_E_NOMEM, q->finished = sofi_server_clock(s);
            snprintf(q->error, sizeof q->error, "needs %lld device bytes, budget %lld", q->bytes,
                     s->o.hbm_budget);
            release_prep(q);
        }
    pthread_mutex_unlock(&s->mu);
    free(ready), free(bytes), free(admit);
    /* 3. issue: one chunk per resident solve per pass, up to `depth` in flight */
    for (int pass = 0; pass < s->o.depth; pass++) {
        for (int k = 0; k < n && !rc; k++) {
            req_t *q = all[k];
            if (q->state != SOFI_REQ_RESIDENT || q->issued >= q->cfg.nt)
                continue;
            int pending = 0;
            if ((rc = sofi_pending_runs(q->ctx, &pending)))
                break;
            if (pending >= s->o.depth)
                continue;
            int m = q->cfg.nt - q->issued;
            if (m > s->o.chunk_steps)
                m = s->o.chunk_steps;
            if ((rc = sofi_run(q->ctx, m)))
                break;
            q->issued += m;
        }
    }
    free(all);
    if (rc)
        return fail(rc, "%s", sofi_last_error());
    if (active) {
        int a = 0;
        pthread_mutex_lock(&s->mu);
        for (int k = 0; k < s->n; k++)
            a += s->reqs[k]->state < SOFI_REQ_DONE;
        pthread_mutex_unlock(&s->mu);
        *active = a;
    }
    return 0;
}

int sofi_server_drain(sofi_server *s)
{
    for (;;) {
        int active = 0;
        int rc = sofi_server_poll(s, &active);
        if (rc)
            return rc;
        if (!active)
            return 0;
        struct timespec ts = {0, 20000};
        nanosleep(&ts, NULL);
    }
}

int sofi_server_info(sofi_server *s, int id, sofi_request_info *info)
{
    if (!s || !info)
        return fail(SOFI_E_ARG, "null argument");
    pthread_mutex_lock(&s->mu);
    if (id < 0 || id >= s->n) {
        pthread_mutex_unlock(&s->mu);
        return fail(SOFI_E_ARG, "no request %d", id);
    }
    req_t *q = s->reqs[id];
    memset(info, 0, sizeof *info);
    info->state = q->state, info->status = q->status;
    snprintf(info->error, sizeof info->error, "%s", q->error);
    info->arrival = q->arrival, info->ready = q->ready, info->admitted = q->admitted, info->finished = q->finished;
    info->device_bytes = q->bytes, info->priority = q->priority;
    info->ntr = q->cfg.seismo ? q->r.ntr : 0, info->ns = q->ns;
    info->cell_updates = (double)q->r.par.nx * (double)q->r.par.ny * (double)q->r.par.nt;
    info->launches = q->launches;
    pthread_mutex_unlock(&s->mu);
    return 0;
}

int sofi_server_section(sofi_server *s, int id, int comp, float *out)
{
    if (!s || !out || comp < 1 || comp > 5)
        return fail(SOFI_E_ARG, "invalid section arguments");
    pthread_mutex_lock(&s->mu);
    if (id < 0 || id >= s->n) {
        pthread_mutex_unlock(&s->mu);
        return fail(SOFI_E_ARG, "no request %d", id);
    }
    req_t *q = s->reqs[id];
    int rc = 0;
    if (q->state != SOFI_REQ_DONE)
        rc = fail(SOFI_E_STATE, "request %d has not finished", id);
    else if (!q->sec[comp])
        rc = fail(SOFI_E_ARG, "component %d was not recorded (SEISMO=%d)", comp, q->cfg.seismo);
    else
        memcpy(out, q->sec[comp], sizeof(float) * (size_t)q->r.ntr * (size_t)q->ns);
    pthread_mutex_unlock(&s->mu);
    return rc;
}

int sofi_server_stats_get(sofi_server *s, sofi_server_stats *st)
{
    if (!s || !st)
        return fail(SOFI_E_ARG, "null argument");
    memset(st, 0, sizeof *st);
    pthread_mutex_lock(&s->mu);
    double *lat = (double *)malloc(sizeof(double) * (size_t)(s->n + 1));
    if (!lat) {
        pthread_mutex_unlock(&s->mu);
        return fail(SOFI_E_NOMEM, "host memory");
    }
    double cells = 0.0, sum = 0.0;
    st->submitted = s->n;
    st->first_arrival = -1.0;
    for (int k = 0; k < s->n; k++) {
        req_t *q = s->reqs[k];
        if (st->first_arrival < 0.0 || q->arrival < st->first_arrival)
            st->first_arrival = q->arrival;
        if (q->state == SOFI_REQ_FAILED)
            st->failed++;
        if (q->state != SOFI_REQ_DONE)
            continue;
        double l = q->finished - q->arrival;
        lat[st->completed++] = l;
        sum += l;
        if (l > st->max_s)
            st->max_s = l;
        if (q->finished > st->last_finish)
            st->last_finish = q->finished;
        cells += (double)q->r.par.nx * (double)q->r.par.ny * (double)q->r.par.nt;
        st->launches += q->launches;
    }
    st->peak_bytes = s->peak_bytes, st->peak_resident = s->peak_resident;
    pthread_mutex_unlock(&s->mu);
    if (st->completed) {
        st->p50_s = sofi_server_percentile(lat, st->completed, 0.50);
        st->p99_s = sofi_server_percentile(lat, st->completed, 0.99);
        st->mean_s = sum / st->completed;
        double span = st->last_finish - st->first_arrival;
        if (span > 0.0) {
            st->shots_per_s = st->completed / span;
            st->gcell_per_s = cells / span / 1e9;
        }
    }
    free(lat);
    return 0;
}
