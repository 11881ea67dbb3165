/*
 * Single-rank stand-in for the subset of MPI that the SOFI2D reference calls.
 *
 * Test infrastructure only: it lets the unmodified reference sources (read in
 * place from the reference tree) build as one process with NPROCX = NPROCY = 1,
 * so the compiled reference can serve as the oracle's own reference.
 *
 * Semantics with one rank (every neighbour index the reference computes in
 * initproc.c:41-68 resolves to rank 0 itself):
 *   - MPI_Sendrecv_replace: a message sent to self and received back into the
 *     same buffer leaves it unchanged -> no-op (exchange_v.c:64-67, exchange_s.c).
 *   - MPI_Bsend / MPI_Recv: every pair in matcopy*.c uses one buffer for both
 *     calls, so the received data equals the sent data -> no-op.
 *   - MPI_Allreduce(SUM) over one rank copies sendbuf to recvbuf (catseis.c:45).
 *   - MPI_Bcast, MPI_Barrier, buffer attach/detach: no-ops.
 */
#ifndef SOFI_ORACLE_MPI_STUB_H
#define SOFI_ORACLE_MPI_STUB_H

#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_FLOAT 4
#define MPI_INT 5
#define MPI_CHAR 1
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_IN_PLACE ((void *)1)

static inline size_t sofi_stub_type_size(MPI_Datatype t)
{
    switch (t) {
      case MPI_FLOAT: return sizeof(float);
      case MPI_INT: return sizeof(int);
      case MPI_DOUBLE: return sizeof(double);
      default: return 1;
    }
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code ? code : 1); return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static inline int MPI_Sendrecv_replace(void *b, int n, MPI_Datatype t, int dst, int stag, int src, int rtag,
                                       MPI_Comm c, MPI_Status *s)
{ (void)b; (void)n; (void)t; (void)dst; (void)stag; (void)src; (void)rtag; (void)c; (void)s; return 0; }
static inline int MPI_Bsend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)dst; (void)tag; (void)c; return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s)
{ (void)b; (void)n; (void)t; (void)src; (void)tag; (void)c; (void)s; return 0; }
static inline int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    if (sb != MPI_IN_PLACE && sb != rb)
        memmove(rb, sb, (size_t)n * sofi_stub_type_size(t));
    return 0;
}
static inline int MPI_Buffer_attach(void *b, int n) { (void)b; (void)n; return 0; }
static inline int MPI_Buffer_detach(void *b, int *n) { (void)b; (void)n; return 0; }

#endif
