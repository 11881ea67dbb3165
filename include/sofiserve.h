/*
 * sofiserve.h -- continuous-batching request loop for forward-modelling solves
 * on one GPU (libsofiserve.so).
 *
 * The reference has no counterpart: sofi2D.c:369-370 runs its shots one after
 * another, each through time_loop(). This loop accepts a stream of independent
 * solves of uneven grid sizes and orders, and keeps as many of them resident on
 * the GPU as the HBM budget and the slot count allow:
 *
 *   arrival -> preparation (host worker threads: sofih_prepare, wavelets)
 *           -> admission   (first fit in arrival order against the budget,
 *                           sofi_device_bytes of each solve)
 *           -> resident    (one sofi_ctx per solve on its own priority stream;
 *                           the loop issues every resident solve one chunk of
 *                           time steps per pass, a CUDA-graph replay, so the
 *                           chunks of all solves interleave on the device)
 *           -> retired     (sections copied to the host, device memory freed,
 *                           the freed budget admits the next arrivals).
 *
 * Each solve is bit-identical to the same solve run alone through libsofigpu:
 * the kernels of one context read and write only that context's arrays.
 * Latency of a request = retirement time - arrival time on the server clock.
 * All calls are thread-safe; one thread at a time drives the loop
 * (sofi_server_poll / sofi_server_drain).
 */
#ifndef SOFISERVE_H
#define SOFISERVE_H

#include "sofihost.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sofi_server sofi_server;

/* One forward-modelling solve. Arrays are borrowed: they must stay valid and
 * unchanged until the request reaches SOFI_REQ_DONE or SOFI_REQ_FAILED. */
typedef struct {
    sofih_par par;          /* WEQ NX NY DH DT NT FDORDER MAXRELERROR L F_REF FL FW ABS_TYPE
                               FREE_SURF BOUNDARY NPOWER K_MAX_CPML VPPML FPML DAMPING
                               SOURCE_SHAPE SEISMO NDT (snapshots are not served) */
    const float *vp, *vs, *rho, *qp, *qs, *eps, *del, *theta; /* raw material [NX][NY], y fastest */
    int nsrc;
    const float *srcpos;    /* [12][nsrc], grid indices (sofigpu.h, sofi_set_sources) */
    int ntr;
    const int *rec_ix, *rec_iy; /* receiver grid indices */
    double arrival;         /* seconds on sofi_server_clock(); work starts no earlier */
} sofi_request;

/* request states */
#define SOFI_REQ_WAITING 0   /* submitted, arrival time not reached */
#define SOFI_REQ_PREPARING 1 /* on a host worker */
#define SOFI_REQ_READY 2     /* prepared, waiting for budget or a slot */
#define SOFI_REQ_RESIDENT 3  /* wavefields on the GPU, time steps in flight */
#define SOFI_REQ_DONE 4
#define SOFI_REQ_FAILED 5

typedef struct {
    int state;
    int status;             /* SOFI_OK or the SOFI_E_* code that failed the request */
    char error[256];
    double arrival, ready, admitted, finished; /* server clock, seconds */
    long long device_bytes; /* sofi_device_bytes of the solve */
    int priority;           /* stream priority it ran with */
    int ntr, ns;            /* section shape [ntr][ns] */
    double cell_updates;    /* NX * NY * NT */
    long long launches;     /* kernels the solve launched (sofi_launch_count) */
} sofi_request_info;

typedef struct {
    int submitted, completed, failed;
    double p50_s, p99_s, mean_s, max_s; /* latency of completed requests */
    double first_arrival, last_finish;  /* server clock */
    double shots_per_s;                 /* completed / (last_finish - first_arrival) */
    double gcell_per_s;                 /* completed cell updates / same span / 1e9 */
    long long peak_bytes;               /* largest sum of resident device bytes */
    int peak_resident;                  /* largest number of resident solves */
    long long launches;                 /* kernels launched by completed solves */
} sofi_server_stats;

typedef struct {
    int device;
    long long hbm_budget;   /* bytes the resident solves may hold; <= 0: 90 % of free memory */
    int max_resident;       /* slots; <= 0: 64 */
    int chunk_steps;        /* time steps issued per solve per pass; <= 0: 32 */
    int depth;              /* chunks in flight per solve; <= 0: 2 */
    int prep_threads;       /* host workers; <= 0: 2 */
    int prep_omp_threads;   /* OpenMP threads per worker; <= 0: cores / workers */
    int use_priorities;     /* 1: smaller solves get more urgent streams */
    int largest_first;      /* 1: of the requests that have arrived, the workers prepare
                               the one with the most cell updates (NX NY NT) first, so
                               the longest solves start early; 0: arrival order */
} sofi_server_options;

const char *sofi_server_last_error(void);

/* Fill `o` with the defaults listed above (device 0, priorities on). */
void sofi_server_default_options(sofi_server_options *o);
int sofi_server_create(const sofi_server_options *o, sofi_server **out);
/* Waits for resident work, frees everything. */
int sofi_server_destroy(sofi_server *s);
/* Seconds since the server was created (CLOCK_MONOTONIC). */
double sofi_server_clock(const sofi_server *s);

/* Queue a request; *id is its handle. A negative arrival means "now". */
int sofi_server_submit(sofi_server *s, const sofi_request *r, int *id);
/* One pass of the loop: retire finished solves, admit ready ones, issue
 * chunks. Never blocks on the GPU. *active = requests not yet finished. */
int sofi_server_poll(sofi_server *s, int *active);
/* Run the loop until every submitted request is done or failed. */
int sofi_server_drain(sofi_server *s);

int sofi_server_info(sofi_server *s, int id, sofi_request_info *info);
/* Seismogram section of a finished request, [ntr][ns] (SOFI_COMP_*). */
int sofi_server_section(sofi_server *s, int id, int comp, float *out);
int sofi_server_stats_get(sofi_server *s, sofi_server_stats *st);

/* ---- pure policy functions (no GPU), exported for tests ---- */
/* First fit in order: admit[k] = 1 for each of the n ready requests (in
 * arrival order) that fits next to `in_use` bytes under `budget` while fewer
 * than max_resident solves are resident. Returns the number admitted. */
int sofi_server_plan(const long long *bytes, int n, long long in_use, long long budget, int resident,
                     int max_resident, int *admit);
/* Stream priority of a solve of `cell_updates` work within [greatest, least]:
 * one level per factor 4 of work above 2^30, the smallest the most urgent. */
int sofi_server_priority(double cell_updates, int least, int greatest);
/* Nearest-rank percentile (q in [0, 1]) of n values (not modified). */
double sofi_server_percentile(const double *x, int n, double q);

#ifdef __cplusplus
}
#endif
#endif
