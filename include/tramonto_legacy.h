/*
 * tramonto_legacy.h - the reference's linear-problem-manager C ABI, served on one GB300.
 *
 * These are the entry points the reference's C fill, Newton driver and continuation code call
 * (declared extern "C" in src/dft_basic_lin_prob_mgr_wrapper.h:44-92 and
 * src/dft_hardsphere_lin_prob_mgr_wrapper.h:43-58, defined in the matching .cpp files).  With
 * libtramonto_gpu.so linked in place of the Trilinos managers, the reference's own CPU fill
 * inserts the residual and Jacobian scalar by scalar as before; finalizeproblemvalues turns
 * them into CSR blocks on the GPU and setupsolver/solve run the hard-sphere Schur-complement
 * GMRES there (the basic manager: GMRES on the whole matrix with a diagonal preconditioner).
 *
 * One process, one GPU: the row map (owned nodes) and column map (box nodes) must list the
 * same global ids; communicators and Teuchos parameter lists are accepted and ignored (the
 * solver's tolerance and iteration cap come from tgpu_legacy_set_solver, defaults 1e-10 and
 * 500).  Coarsened-node lists must be empty.  Every function returns 0 on success and a
 * negative status on failure (tgpu_legacy_last_error() has the message); nothing throws.
 *
 * Storage: x_box[junk][boxnode] and b_owned[iunk][ownednode] are the caller's arrays, as in
 * the reference (array_alloc, src/rf_allo.c:171).
 */
#ifndef TRAMONTO_LEGACY_H
#define TRAMONTO_LEGACY_H

/* The communicator argument of the create calls: the caller's MPI_Comm wherever mpi.h is on the include path (the
 * reference's own declaration, so that its headers and this one agree in one translation unit), otherwise an
 * opaque word.  It is not read (one process, one GPU), and either type is passed in the third integer argument
 * register of the x86-64 and AArch64 C calling conventions; this library is built with TGPU_LEGACY_NO_MPI. */
#if !defined(TGPU_LEGACY_NO_MPI) && defined(__has_include)
#if __has_include(<mpi.h>)
#include <mpi.h>
#define TGPU_LEGACY_MPI_COMM 1
#endif
#endif
#ifdef TGPU_LEGACY_MPI_COMM
typedef MPI_Comm tgpu_legacy_comm;
#else
typedef void *tgpu_legacy_comm;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* dft_basic_lin_prob_mgr_create (src/dft_basic_lin_prob_mgr_wrapper.h:44) */
void *dft_basic_lin_prob_mgr_create(int numUnks, void *parameter_list, tgpu_legacy_comm comm);
/* dft_hardsphere_lin_prob_mgr_create / _create_debug (src/dft_hardsphere_lin_prob_mgr_wrapper.h:43,48) */
void *dft_hardsphere_lin_prob_mgr_create(int numUnks, void *parameter_list, tgpu_legacy_comm comm);
void *dft_hardsphere_lin_prob_mgr_create_debug(int numUnks, void *parameter_list, tgpu_legacy_comm comm);
/* dft_hardsphere_lin_prob_mgr_destruct (:52), dft_linprobmgr_destruct (basic :46) */
void dft_hardsphere_lin_prob_mgr_destruct(void *mgr);
void dft_linprobmgr_destruct(void *mgr);
/* equation (unknown) lists of the Schur split: linsolver_setup_HSTYPE, src/dft_linsolver_setup.c:182-241 (:54-58) */
int dft_hardsphere_lin_prob_mgr_setindnonlocalequationids(void *mgr, int numgids, int *gids);
int dft_hardsphere_lin_prob_mgr_setdepnonlocalequationids(void *mgr, int numgids, int *gids);
int dft_hardsphere_lin_prob_mgr_setdensityequationids(void *mgr, int numgids, int *gids);
/* the callers and the definition spell it ...diagonal; the reference's header declares ...diagona (:58): both exist */
int dft_hardsphere_lin_prob_mgr_seta22blockisdiagonal(void *mgr, int isa22diagonal);
int dft_hardsphere_lin_prob_mgr_seta22blockisdiagona(void *mgr, int isa22diagonal);
/* maps and block structure (basic :48-54); finalizeblockstructure returns 1 if already done, -1 if a map is missing */
int dft_linprobmgr_setnodalrowmap(void *mgr, int numgids, int *gids);
int dft_linprobmgr_setnodalcolmap(void *mgr, int numgids, int *gids);
int dft_linprobmgr_setcoarsenednodeslist(void *mgr, int numgids, int *gids);
int dft_linprobmgr_finalizeblockstructure(void *mgr);
/* per Newton step (basic :56-70): values are added (+=) to the rhs and the matrix */
int dft_linprobmgr_initializeproblemvalues(void *mgr);
int dft_linprobmgr_insertrhsvalue(void *mgr, int iunk, int inode, double value);
int dft_linprobmgr_insertonematrixvalue(void *mgr, int iunk, int ownednode, int junk, int boxnode, double value);
int dft_linprobmgr_insertmultinodematrixvalues(void *mgr, int iunk, int ownednode, int junk, int *boxnodeindices,
                                               double *values, int numentries);
int dft_linprobmgr_insertmultiphysicsmatrixvalues(void *mgr, int iunk, int ownednode, int *junkindices, int boxnode,
                                                  double *values, int numentries);
int dft_linprobmgr_finalizeproblemvalues(void *mgr);
double dft_linprobmgr_getmatrixvalue(void *mgr, int iunk, int ownednode, int junk, int boxnode);
/* vectors (basic :74-78) */
int dft_linprobmgr_setrhs(void *mgr, double **b);
int dft_linprobmgr_getlhs(void *mgr, double **x);
int dft_linprobmgr_getrhs(void *mgr, double **b);
/* MatrixMarket text of the assembled matrix (basic :80) */
int dft_linprobmgr_writeMatrix(void *mgr, char *filename, char *matrixName, char *matrixDescription);
/* solve (basic :82-84): setupsolver uploads the matrix; solve runs GMRES and keeps the solution for getlhs */
int dft_linprobmgr_setupsolver(void *mgr);
int dft_linprobmgr_solve(void *mgr);
/* b_owned = J x_box (basic :86) */
int dft_linprobmgr_applymatrix(void *mgr, double **x, double **b);
/* owned -> box copies (basic :88-92) */
int dft_linprobmgr_importr2c(void *mgr, double **x, double **b);
int dft_linprobmgr_importsingleunknownr2c(void *mgr, double *x, double *b);
int dft_linprobmgr_importnodalr2c(void *mgr, double *x, double *b);

/* Additions with no counterpart in the reference: solver settings that the reference reads from its
 * parameter list, the last solve's statistics, and the last error message. */
int tgpu_legacy_set_solver(void *mgr, double tol, int max_iter);
int tgpu_legacy_last_solve(void *mgr, int *iters, double *relres);
const char *tgpu_legacy_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
