/* Serial stand-in for the MPI interface used by the Tramonto C sources.
 * One process, one rank: reductions copy, broadcasts do nothing.
 * Used only to compile the reference's own C files into the oracle
 * library (oracle/_ref); nothing in the product links it. */
#ifndef TGPU_REF_SHIM_MPI_H
#define TGPU_REF_SHIM_MPI_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef void (MPI_User_function)(void *, void *, int *, MPI_Datatype *);
#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_FLOAT 5
#define MPI_LONG 9
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm c, int *r);
int MPI_Comm_size(MPI_Comm c, int *s);
int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm *out);
int MPI_Comm_dup(MPI_Comm c, MPI_Comm *out);
int MPI_Comm_free(MPI_Comm *c);
int MPI_Barrier(MPI_Comm c);
double MPI_Wtime(void);
int MPI_Bcast(void *buf, int n, MPI_Datatype t, int root, MPI_Comm c);
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Scan(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c);
int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rn, const int *disp, MPI_Datatype rt, int root, MPI_Comm c);
int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c);
int MPI_Allgatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rn, const int *disp, MPI_Datatype rt, MPI_Comm c);
int MPI_Send(const void *b, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c);
int MPI_Rsend(const void *b, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c);
int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st);
int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *rq);
int MPI_Wait(MPI_Request *rq, MPI_Status *st);
int MPI_Type_contiguous(int n, MPI_Datatype old, MPI_Datatype *nt);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);
int MPI_Op_create(MPI_User_function *f, int commute, MPI_Op *op);
int MPI_Op_free(MPI_Op *op);
#ifdef __cplusplus
}
#endif
#endif
