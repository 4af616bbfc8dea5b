/*
 * Single-rank MPI stand-in used to build the miniAMR reference (and the
 * drop-in hybrid) in a container with no MPI installed.
 *
 * Test infrastructure only: this header is part of the oracle build recipe
 * (oracle/Makefile) and never of the GPU library.
 *
 * Semantics on one rank (MPI_COMM_WORLD has size 1):
 *   - collectives (Allreduce, Bcast, Scan, Alltoall) are identities: the
 *     send buffer is copied to the receive buffer;
 *   - MPI_Comm_split returns the parent communicator;
 *   - MPI_Wtime reads CLOCK_MONOTONIC;
 *   - point-to-point calls have no partner on one rank; every one of them
 *     prints a message and aborts, so a run that ever reaches one fails
 *     loudly instead of returning made-up data.
 * The symbol list follows what the reference uses (MPI_Init .. MPI_Wtime in
 * ref/main.c, ref/comm.c, ref/refine.c, ref/rcb.c, ref/sfc.c, ref/plot.c).
 */
#ifndef MAMR_MPI_STUB_H
#define MAMR_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Errhandler;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_REQUEST_NULL (-1)
#define MPI_ERRORS_ARE_FATAL 0

#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_LONG_LONG_INT 3

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline size_t mamr_stub_type_size(MPI_Datatype t)
{
   switch (t) {
      case MPI_INT: return sizeof(int);
      case MPI_DOUBLE: return sizeof(double);
      case MPI_LONG_LONG_INT: return sizeof(long long);
   }
   fprintf(stderr, "mpi stub: unknown datatype %d\n", t);
   abort();
}

static inline void mamr_stub_copy(const void *s, void *r, int count,
                                  MPI_Datatype t)
{
   if (count > 0 && s != r)
      memmove(r, s, (size_t) count * mamr_stub_type_size(t));
}

static inline void mamr_stub_no_partner(const char *what)
{
   fprintf(stderr, "mpi stub: %s has no partner on a single rank\n", what);
   abort();
}

static inline int MPI_Init(int *argc, char ***argv)
{ (void) argc; (void) argv; return MPI_SUCCESS; }
static inline int MPI_Finalize(void) { return MPI_SUCCESS; }
static inline int MPI_Comm_set_errhandler(MPI_Comm c, MPI_Errhandler e)
{ (void) c; (void) e; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void) c; *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void) c; *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *out)
{ (void) color; (void) key; *out = c; return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm c) { (void) c; return MPI_SUCCESS; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void) c; exit(code); }
static inline double MPI_Wtime(void)
{
   struct timespec ts;
   clock_gettime(CLOCK_MONOTONIC, &ts);
   return (double) ts.tv_sec + 1.0e-9 * (double) ts.tv_nsec;
}
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void) b; (void) n; (void) t; (void) root; (void) c; return MPI_SUCCESS; }
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t,
                                MPI_Op op, MPI_Comm c)
{ (void) op; (void) c; mamr_stub_copy(s, r, n, t); return MPI_SUCCESS; }
static inline int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t,
                           MPI_Op op, MPI_Comm c)
{ (void) op; (void) c; mamr_stub_copy(s, r, n, t); return MPI_SUCCESS; }
static inline int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r,
                               int rn, MPI_Datatype rt, MPI_Comm c)
{ (void) rn; (void) rt; (void) c; mamr_stub_copy(s, r, sn, st); return MPI_SUCCESS; }

static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag,
                            MPI_Comm c, MPI_Request *rq)
{ (void) b; (void) n; (void) t; (void) src; (void) tag; (void) c; (void) rq;
  mamr_stub_no_partner("MPI_Irecv"); return 1; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst,
                            int tag, MPI_Comm c, MPI_Request *rq)
{ (void) b; (void) n; (void) t; (void) dst; (void) tag; (void) c; (void) rq;
  mamr_stub_no_partner("MPI_Isend"); return 1; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int dst,
                           int tag, MPI_Comm c)
{ (void) b; (void) n; (void) t; (void) dst; (void) tag; (void) c;
  mamr_stub_no_partner("MPI_Send"); return 1; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag,
                           MPI_Comm c, MPI_Status *st)
{ (void) b; (void) n; (void) t; (void) src; (void) tag; (void) c; (void) st;
  mamr_stub_no_partner("MPI_Recv"); return 1; }
static inline int MPI_Wait(MPI_Request *rq, MPI_Status *st)
{
   (void) st;
   if (*rq == MPI_REQUEST_NULL) return MPI_SUCCESS;
   mamr_stub_no_partner("MPI_Wait");
   return 1;
}
static inline int MPI_Waitany(int n, MPI_Request *rq, int *idx, MPI_Status *st)
{ (void) n; (void) rq; (void) idx; (void) st;
  mamr_stub_no_partner("MPI_Waitany"); return 1; }

#endif
