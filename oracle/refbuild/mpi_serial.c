/* Single-rank implementation of the MPI calls made by the Tramonto C sources.
 * Part of the oracle build only (oracle/_ref): it lets the reference's own
 * physics code run in one process without an MPI installation.
 * Collectives copy the send buffer; point-to-point calls are never reached
 * with one rank and report an error if they are. */
#include "mpi.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static size_t tsize(MPI_Datatype t)
{
  switch (t) {
    case MPI_CHAR: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_FLOAT: return sizeof(float);
    case MPI_DOUBLE: return sizeof(double);
    case MPI_LONG: return sizeof(long);
    default:
      if (t >= 1000) return (size_t)(t - 1000); /* contiguous derived type: byte size */
      return 1;
  }
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *o) { (void)color; (void)key; *o = c; return 0; }
int MPI_Comm_dup(MPI_Comm c, MPI_Comm *o) { *o = c; return 0; }
int MPI_Comm_free(MPI_Comm *c) { (void)c; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
double MPI_Wtime(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
static void copyn(const void *s, void *r, int n, MPI_Datatype t)
{
  if (s != r && n > 0) memmove(r, s, (size_t)n * tsize(t));
}
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; copyn(s, r, n, t); return 0; }
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) { (void)op; (void)root; (void)c; copyn(s, r, n, t); return 0; }
int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; copyn(s, r, n, t); return 0; }
int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)rn; (void)rt; (void)root; (void)c; copyn(s, r, sn, st); return 0; }
int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rn, const int *disp, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)rn; (void)root; (void)c; copyn(s, (char *)r + (size_t)disp[0] * tsize(rt), sn, st); return 0; }
int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{ (void)rn; (void)rt; (void)c; copyn(s, r, sn, st); return 0; }
int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rn, const int *disp, MPI_Datatype rt, MPI_Comm c)
{ (void)rn; (void)c; copyn(s, (char *)r + (size_t)disp[0] * tsize(rt), sn, st); return 0; }
static int p2p(const char *what)
{
  fprintf(stderr, "oracle MPI shim: %s reached with a single rank\n", what);
  abort();
  return 1;
}
int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) { (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return p2p("MPI_Send"); }
int MPI_Rsend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) { (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return p2p("MPI_Rsend"); }
int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st) { (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return p2p("MPI_Recv"); }
int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *rq) { (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)rq; return p2p("MPI_Irecv"); }
int MPI_Wait(MPI_Request *rq, MPI_Status *st) { (void)rq; (void)st; return p2p("MPI_Wait"); }
int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *nt) { *nt = 1000 + n * (int)tsize(old); return 0; }
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
int MPI_Op_create(MPI_User_function *f, int commute, MPI_Op *op) { (void)f; (void)commute; *op = 100; return 0; }
int MPI_Op_free(MPI_Op *op) { (void)op; return 0; }
