/* tramonto_gpu.h — C ABI of the GB300 nonlocal-density path.
 *
 * One handle holds one hard-sphere (FMT) + WCA mean-field problem resident on
 * one GPU.  The entry points replace, one level above the per-scalar
 * dft_linprobmgr_* inserts, the reference calls on the Newton path:
 *
 *   tgpu_fill              fill_resid_and_matrix_control   src/dft_fill_control.c:39-63
 *                          (FMT1stDeriv_switch src/dft_switch_FMT.c:68, fill_resid_and_matrix
 *                           src/dft_fill_main.c:38-153 with load_euler_lagrange, load_rho_bar_s/v,
 *                           load_mean_field)
 *   tgpu_jv / tgpu_jtv     the assembled Jacobian of that fill applied matrix-free
 *                          (dft_linprobmgr_applymatrix src/dft_basic_lin_prob_mgr_wrapper.h:86;
 *                           the transpose has no reference counterpart: SetUseTranspose returns -1,
 *                           src/dft_HardSphereA11_Epetra_Operator.hpp:68)
 *   tgpu_schur_apply       dft_Schur_Epetra_Operator::Apply src/dft_Schur_Epetra_Operator.cpp:86-119
 *   tgpu_schur_rhs         dft_Schur_Epetra_Operator::ComputeRHS :121-133
 *   tgpu_schur_x1          dft_Schur_Epetra_Operator::ComputeX1 :135-147
 *   tgpu_solve             dft_linprobmgr_setupsolver + dft_linprobmgr_solve
 *                          (dft_HardSphereLinProbMgr::setupSolver/solve src/dft_HardSphereLinProbMgr.cpp:345-428)
 *   tgpu_newton            newton_solver + update_solution src/dft_newton.c:131-381
 *
 * Conventions
 *   - Fields are SoA [unknown][node], node = ix + nx*(iy + ny*iz): the layout
 *     of the reference's x[iunk][inode_box] for one process (src/rf_allo.c:171).
 *   - Unknown order as setup_nunk_per_node (src/dft_defs_unknowns.c:37-176):
 *     ncomp densities, 4+2*ndim weighted densities (n3, n2, n1, n0, V2[d], V1[d]),
 *     then ncomp mean-field unknowns when attractions are on.
 *   - Residuals R are returned with the reference's sign of "resid"; the
 *     reference's rhs vector is -R.
 *   - Functions without the _device suffix take HOST pointers and copy; the
 *     _device variants take device pointers on the handle's stream.
 *   - Every function returns a tgpu_status; no C++ exception crosses the ABI.
 *   - One handle is used from one host thread at a time.
 */
#ifndef TRAMONTO_GPU_H
#define TRAMONTO_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tgpu_ctx *tgpu_handle;

typedef enum {
  TGPU_OK = 0,
  TGPU_ERR_ARG = -1,          /* bad argument or size */
  TGPU_ERR_CUDA = -2,         /* a CUDA call failed; tgpu_last_error() has the text */
  TGPU_ERR_STATE = -3,        /* call out of order (e.g. apply before fill) */
  TGPU_ERR_UNSUPPORTED = -4,  /* option outside the implemented path */
  TGPU_ERR_NOCONV = -5,       /* iteration cap reached (GMRES or Newton) */
  TGPU_ERR_NONFINITE = -6,    /* NaN/Inf in inputs or iterates */
  TGPU_ERR_DOMAIN = -7        /* n3 >= 1 or density <= 0 where a log/1/(1-n3) is taken */
} tgpu_status;

/* boundary codes (reference Type_bc values, src/dft_globals_const.h) */
enum { TGPU_BC_IN_WALL = -1, TGPU_BC_IN_BULK = 0, TGPU_BC_PERIODIC = 1, TGPU_BC_REFLECT = 2 };
/* functionals (reference Type_func values, src/dft_globals_const.h:247-250): Rosenfeld (FMT1),
 * Rosenfeld with the zero-dimensional-crossover third term (FMT2), White-Bear (FMT3), White-Bear
 * with the FMT2 vector form (FMT4) */
enum { TGPU_FMT1 = 0, TGPU_FMT2 = 1, TGPU_FMT3 = 2, TGPU_FMT4 = 3 };
/* second derivatives of the FMT terms in J, J^T and Schur products (tgpu_set_jacobian_form) */
enum { TGPU_JAC_REFERENCE = 0, TGPU_JAC_EXACT = 1 };
/* stencil types (reference Stencil ids, src/dft_globals_const.h:152-161) */
enum { TGPU_STEN_DELTA = 0, TGPU_STEN_THETA = 1, TGPU_STEN_UATT = 2 };
/* arithmetic of the stencil convolutions */
enum { TGPU_FP64 = 0, TGPU_FP32 = 1, TGPU_BF16X3 = 2, TGPU_FP16TC = 3, TGPU_FP64_FFT = 4 };

#define TGPU_MAXC 4

typedef struct {
  int ndim;
  int nx[3];                 /* nodes per dimension (unused dims: 1) */
  double esize[3];           /* Esize_x */
  int bc[3][2];              /* Type_bc[idim][left/right] */
  int ncomp;
  int functional;            /* TGPU_FMT1 .. TGPU_FMT4 */
  int attraction;            /* 1: WCA mean field (Type_attr != NONE) */
  int att_in_a22;            /* ATTInA22Block: 0 mean field as its own unknown (MF_EQ rows); 1 summed into the
                                Euler-Lagrange rows: vectors then have ncomp + 4 + 2 ndim rows per node */
  int single_size;           /* n1, n0, V1 are local copies (src/dft_fill_FMT.c:215, :303) */
  int hard_surf;             /* Lhard_surf: hard-wall boundary weights */
  int nlists_hw;             /* Nlists_HW */
  double rho_b[TGPU_MAXC];
  double betamu_hs_ex[TGPU_MAXC];
  double betamu_att[TGPU_MAXC];
  double inv_rad[TGPU_MAXC];
  double inv_4pir[TGPU_MAXC];
  double inv_4pirsq[TGPU_MAXC];
  double fac_overlap[TGPU_MAXC];
  double dphi_bulk[4];       /* Dphi_Drhobar_b[0..3]: bulk dPhi/dn0..dn3 */
  double vext_max;           /* VEXT_MAX: nodes with V_ext == vext_max are zero-density rows */
  /* two-phase interface (Type_interface = PHASE_INTERFACE, no walls): beyond the low side of an IN_BULK
   * boundary the bulk state LBB, beyond the high side RTF (sentinels -3/-4 of offset_to_node_box,
   * src/dft_mesh_lib.c:213-265, with constant_boundary src/dft_utils.c:90-130), and the Euler-Lagrange rows
   * take the chemical potential betamu (the LBB/RTF mean, src/dft_thermo.c:326; src/dft_fill_EL.c:412-416) */
  int interface;             /* 0: uniform (the fields above); 2: phase interface (the fields below) */
  double rho_b_lbb[TGPU_MAXC], rho_b_rtf[TGPU_MAXC];
  double dphi_lbb[4], dphi_rtf[4];   /* Dphi_Drhobar_LBB / _RTF */
  double betamu[TGPU_MAXC];
  /* Lconstrain_interface: the first component's density at node pin_node held at pin_value
   * (fill_constant_density, src/dft_fill_EL.c:89-97) when pin is 1 */
  int pin;
  long pin_node;
  double pin_value;
} tgpu_geometry;

/* lifecycle: create -> set_stencil/set_vext/set_zero_density/set_hard_wall -> finalize */
int tgpu_create(const tgpu_geometry *geom, int device, tgpu_handle *out);
int tgpu_destroy(tgpu_handle h);
const char *tgpu_last_error(void);
/* Stencil table (Stencil[type][0][index], src/dft_globals_const.h:635-646):
 * offsets[length][ndim], weights[length], hw[length][2^ndim] or NULL. */
int tgpu_set_stencil(tgpu_handle h, int type, int index, int length, const short *offsets,
                     const double *weights, const double *hw);
int tgpu_set_vext(tgpu_handle h, const double *vext);                 /* [ncomp][N] */
int tgpu_set_zero_density(tgpu_handle h, const signed char *flags);   /* [ncomp][N] */
/* Hard-wall data: boundary_nodes[nlists][N] (Nodes_2_boundary_wall, -1 = none) and
 * fluid_masks[nlists][2^ndim][N]: bit l set when the element that has the node
 * as local corner l (for that reflection pattern) is fluid (src/dft_utils.c:41-62). */
int tgpu_set_hard_wall(tgpu_handle h, const int *boundary_nodes, const short *fluid_masks);
/* Mesh coarsening (Nzone quadrature zones with Mesh_coarsening on; replaces the Mesh_coarsen_flag and
 * Stencil[type][izone] reads of src/dft_fill_main.c:118-135, src/dft_fill_FMT.c:41-189 and
 * src/dft_fill_CLSmf.c:38-171, and dft_linprobmgr_setcoarsenednodeslist, src/dft_mesh.c:516).
 * flag[N] is Mesh_coarsen_flag: >= 0 the node's quadrature zone (< nzone, at most 5), -1/-2/-3 the
 * node's rows average its two neighbours along x/y/z (load_coarse_node_Ndim,
 * src/dft_fill_coarse.c:66-123), TGPU_FLAG_1DBC the node's rows copy the node with the same coordinate
 * along the tgpu_set_1d_boundary dimension and 0 along the others (L1D_bc: load_coarse_node_1dim,
 * src/dft_fill_coarse.c:37-64; set_mesh_coarsen_flag, src/dft_mesh.c:2835-2841), TGPU_FLAG_BULK /
 * TGPU_FLAG_PB the node's Euler-Lagrange rows hold the bulk density (BULK_ZONE: fill_bulk_density,
 * src/dft_fill_EL.c:265-284) / the ideal gas in the external field without hard-sphere or attraction
 * terms (PB_ZONE, src/dft_fill_EL.c:132-161, 405-410; no charges here), its other rows zone 0's
 * stencils (the reference indexes its stencil table with the negative flag there).  rb_bulk[4 + 2 ndim]
 * is Rhobar_b in solution order, the value of a weighted density beyond an IN_BULK boundary in averaged
 * rows; with a phase interface rb_bulk[2][4 + 2 ndim] holds Rhobar_b_LBB then Rhobar_b_RTF (the low and
 * the high side), the densities there Rho_b_LBB / _RTF.  Zone z >= 1 stencils come from
 * tgpu_set_zone_stencil (offsets in fine-node units, as calc_stencils scales them).  The Jacobian is the
 * residual's derivative (the Coarser_jac option, a cheaper approximate Jacobian for the assembled
 * matrix, has no use in the matrix-free products); the Newton step is solved on the nodes that are not
 * coarsened, the coarsened nodes following by interpolation (the adjoint solves that step's transpose).
 * With two zones the reference's averaged row next to a 1-D boundary, BULK_ZONE or PB_ZONE node reads past
 * its offset table; that pattern is TGPU_ERR_UNSUPPORTED. */
enum { TGPU_FLAG_PB = -777, TGPU_FLAG_BULK = -888, TGPU_FLAG_1DBC = -999 };
int tgpu_set_zones(tgpu_handle h, int nzone, const int *flag, const double *rb_bulk);
/* L1D_bc's dimension (Dim_1Dbc = Grad_dim, src/dft_input.c:1474-1477), 0 unless set; before finalize. */
int tgpu_set_1d_boundary(tgpu_handle h, int dim);
int tgpu_set_zone_stencil(tgpu_handle h, int zone, int type, int index, int length, const short *offsets,
                          const double *weights, const double *hw);
int tgpu_finalize(tgpu_handle h);
/* Move the bulk state (chemical potential) of a finalized problem: bulk densities, excess chemical
 * potentials (hard-sphere and attraction) per component and the bulk dPhi/dn0..dn3.  The Euler-Lagrange
 * rows then hold betamu = ln rho_b + betamu_hs_ex + betamu_att: the parameter the reference's continuation
 * in the chemical potential sets (assign_parameter_tramonto, CONT_BETAMU_I, src/dft_switch_continuation.c:
 * 123,170-180).  Stencils and V_ext stay; the next call must be a fill (the Jacobian state is dropped). */
int tgpu_set_bulk_state(tgpu_handle h, const double *rho_b, const double *betamu_hs_ex, const double *betamu_att,
                        const double *dphi_bulk);
/* Arithmetic of the Jacobian / Schur products: TGPU_FP64, TGPU_FP32 (stencil sums in FP32), or
 * TGPU_FP16TC (as TGPU_FP32, but the 3-D attraction sums on the tensor cores: FP16 inputs scaled by
 * powers of two, FP32 accumulation; TGPU_ERR_UNSUPPORTED when the problem has none), or TGPU_FP64_FFT
 * (FP64-accurate sums as TGPU_FILL_FFT forms them: in 3-D the long stencils as FP64 FFT convolutions, the
 * short ones in float-float arithmetic; 1-D and 2-D problems take the direct FP64 sums).  The residual
 * fill's arithmetic is set by tgpu_set_fill_arithmetic. */
int tgpu_set_precision(tgpu_handle h, int precision);
/* Arithmetic of the residual fill:
 *   TGPU_FILL_FP64     every stencil sum in FP64 (default; the reference's arithmetic)
 *   TGPU_FILL_FP32     FP32 stencil sums (an inexact residual)
 *   TGPU_FILL_REFINED  FP64 sums of a reference state plus FP32 sums of the change since then;
 *                      the reference is refreshed in FP64 when the change exceeds tau times the
 *                      field (max norms).  tgpu_newton uses FP32 sums while ||R|| > switch_norm.
 * tau / switch_norm <= 0 keep the current values (defaults 1e-2 and 1.0). */
enum { TGPU_FILL_FP64 = 0, TGPU_FILL_FP32 = 1, TGPU_FILL_REFINED = 2, TGPU_FILL_MIXED = 3, TGPU_FILL_FF = 4,
       TGPU_FILL_MIXED_FF = 5, TGPU_FILL_FFT = 6, TGPU_FILL_MIXED_FFT = 7 };
/* TGPU_FILL_FFT: as TGPU_FILL_FF, but in 3-D the long stencil sums (the attraction stencil; see
 * tgpu_set_fft_threshold) are FP64 FFT convolutions of the padded channel (forward transform, product with the stencil
 * coefficient's spectrum, inverse transform: the same sum to the FFT's rounding, ~eps log2 of the box, at a
 * cost independent of the stencil's length); the short ones stay float-float; 1-D and 2-D problems take
 * the direct FP64 sums.  TGPU_FILL_MIXED_FFT: FP32 sums while ||R||_2 > switch_norm, TGPU_FILL_FFT below. */
/* TGPU_FILL_FF: as TGPU_FILL_FP64, but the 3-D single-channel stencil sums (attraction, theta) run in
 * float-float arithmetic (FP32 high/low pairs, error-free products and two-sums: ~48-bit sums, within
 * ~1e-13 of FP64); TGPU_FILL_MIXED_FF: FP32 sums while ||R||_2 > switch_norm, TGPU_FILL_FF below. */
/* TGPU_FILL_MIXED: in tgpu_newton_solve, FP32 sums while ||R||_2 > switch_norm, FP64 below;
 * everywhere else it is the FP64 fill. */
int tgpu_set_fill_arithmetic(tgpu_handle h, int arith, double tau, double switch_norm);
/* Stencils of at least min_points points take the FFT in TGPU_FILL_FFT; min_points < 0 (default): a cost
 * model (direct float-float sum against the transforms) chooses. */
int tgpu_set_fft_threshold(tgpu_handle h, int min_points);
/* FP32 stencil sums (products, FP32 fills) as FP32 FFT convolutions: -1 (default) each sum's first use times
 * the FFT against its direct kernel and keeps the faster; 0 never; 1 always (3-D problems). */
int tgpu_set_fft32_policy(tgpu_handle h, int policy);
/* The choices of that policy so far, for stencil (type, index): choice[0] forward, choice[1] transposed sums
 * (1 FFT, -1 direct kernel, 0 not yet decided); ms[4] the timed direct and FFT sums behind them (forward direct,
 * forward FFT, transposed direct, transposed FFT; 0 where not timed).  For the attraction stencil the forward
 * choice is the one of the current product arithmetic (tensor-core products for TGPU_FP16TC, else the FP32 slab
 * kernel).  No reference counterpart (a benchmark and diagnostics hook). */
int tgpu_fft32_choice(tgpu_handle h, int type, int index, int *choice, double *ms);
/* Second derivatives of the FMT energy density in J, J^T and Schur products (and so in Newton):
 *   TGPU_JAC_REFERENCE  the reference's tables, entry for entry (default): d2phi_drb2_{delta,theta}_rb_FMT*
 *                       (src/dft_physics_FMT{1,2,3,4}.c, via FMT2ndDeriv*_switch, src/dft_switch_FMT.c:122-152)
 *   TGPU_JAC_EXACT      the Hessian of the energy density
 * The two agree for FMT1 and FMT3.  For FMT2 in 2-D and 3-D the reference's V2-V2 entry has |gamma|^2 v_d
 * where the Hessian has gamma_d (gamma . v); for FMT4 its n2-V2 entry has (fac^2 - 4 V2.V2 fac / n2) where
 * the Hessian has fac (1 + 3 V2.V2 / n2^2), fac = 1 - V2.V2/n2^2 (src/dft_physics_FMT2.c:178-184,
 * src/dft_physics_FMT4.c:175-182).  The sensitivities (tgpu_grad_*) always use the exact form. */
int tgpu_set_jacobian_form(tgpu_handle h, int form);
int tgpu_set_stream(tgpu_handle h, void *cuda_stream);
int tgpu_sizes(tgpu_handle h, long *nnodes, int *nunk, int *ncomp);

/* Residual of every unknown at state x ([nunk][N]).  mode 0 also keeps the
 * Jacobian state (the weighted densities and 1/rho of x) for the products below;
 * mode 1 is residual only (resid_only_flag CALC_RESID_ONLY). */
int tgpu_fill(tgpu_handle h, const double *x, double *resid, int mode);
int tgpu_fill_device(tgpu_handle h, const double *d_x, double *d_resid, int mode);
/* J v and J^T w with the Jacobian of the last mode-0 fill ([nunk][N] each) */
int tgpu_jv(tgpu_handle h, const double *v, double *out);
int tgpu_jv_device(tgpu_handle h, const double *d_v, double *d_out);
int tgpu_jtv(tgpu_handle h, const double *w, double *out);
int tgpu_jtv_device(tgpu_handle h, const double *d_w, double *d_out);
/* Adjoint solve J^T lambda = g ([nunk][N] each) with the Jacobian of the last mode-0 fill: GMRES on the
 * transposed Schur complement S^T = A22^T - A12^T A11^-T A21^T (A22 as left preconditioner, same stopping
 * test as tgpu_solve), then lambda1 = A11^-T (g1 - A21^T lambda2).  No reference counterpart (the
 * reference's operators refuse the transpose, src/dft_HardSphereA11_Epetra_Operator.hpp:68).  With g the
 * gradient of an objective F(x) at a converged state x*, the sensitivity of F(x*) to a parameter p that
 * enters the residual is dF/dp = dF/dp|_x - lambda^T dR/dp; for the external field the residual's
 * Euler-Lagrange rows hold +V_ext, so dF/dV_ext[ic][i] = dF/dV_ext|_x - lambda[ic][i] off zero-density rows.
 * Reflecting boundaries and hard-wall boundary weights are transposed exactly. */
int tgpu_adjoint_solve(tgpu_handle h, const double *g, double *lambda, double tol, int max_iter, int *iters,
                       double *relres);
int tgpu_adjoint_solve_device(tgpu_handle h, const double *d_g, double *d_lambda, double tol, int max_iter,
                              int *iters, double *relres);
/* ---- Objectives and their sensitivities ----------------------------------
 * Integration weights of integrateInSpace (src/dft_out_utils.c:38-62), per component and node ([ncomp][N]):
 *   w_fluid = Nel_hit2 * Vol_el / Nnodes_per_el_V * F,   w_bulk = Nel_hit * Vol_el / Nnodes_per_el_V * F,
 * with F = Fac_vol, or Fac_vol / (Fac_area * Area) for per-area results (Lper_area); Nel_hit / Nel_hit2 as
 * setup_integrals (src/dft_out_utils.c:179-270).  rhobar_b: the bulk weighted densities n3 n2 n1 n0
 * (Rhobar_b); betamu: the chemical potentials (Betamu). */
int tgpu_set_integration(tgpu_handle h, const double *w_fluid, const double *w_bulk, const double *rhobar_b,
                         const double *betamu);
/* omega_s: the surface excess grand free energy of calc_free_energy (src/dft_energy.c:31-168, ideal gas,
 * chemical potential, external field, FMT and mean-field terms minus their bulk terms); gamma_ex[ncomp]:
 * the excess adsorption of calc_adsorption (src/dft_out_ads.c:33-112).  Either pointer may be NULL. */
int tgpu_objectives(tgpu_handle h, const double *x, double *omega_s, double *gamma_ex);
int tgpu_objectives_device(tgpu_handle h, const double *d_x, double *omega_s, double *gamma_ex);
enum { TGPU_OBJ_OMEGA = 0, TGPU_OBJ_GAMMA = 1 };
/* Partial derivatives of omega_s (kind TGPU_OBJ_OMEGA) or gamma_ex[icomp] (TGPU_OBJ_GAMMA) at state d_x:
 * d_gx = dF/dx ([nunk][N]), d_gv = dF/dV_ext at fixed x ([ncomp][N]). */
int tgpu_objective_grad_device(tgpu_handle h, const double *d_x, int kind, int icomp, double *d_gx, double *d_gv);
/* Total sensitivity of an objective of the converged state x to the external field, dF/dV_ext ([ncomp][N]):
 * an FP64 mode-0 fill at x, the adjoint solve J^T lambda = dF/dx (tol, max_iter as tgpu_adjoint_solve) and
 * dF/dV_ext = dF/dV|_x - lambda on the Euler-Lagrange rows.  No reference counterpart. */
int tgpu_grad_vext_device(tgpu_handle h, const double *d_x, int kind, int icomp, double tol, int max_iter,
                          double *d_dF_dV, int *iters);
int tgpu_grad_omega_vext(tgpu_handle h, const double *x, double tol, int max_iter, double *dOmega_dV, int *iters);
int tgpu_grad_gamma_vext(tgpu_handle h, const double *x, int icomp, double tol, int max_iter, double *dGamma_dV,
                         int *iters);
/* Sensitivity to a wall parameter p (e.g. eps_w) that enters only through V_ext: dF/dp = sum dF/dV dV/dp,
 * with dvext_deps = dV_ext/dp ([ncomp][N]). */
int tgpu_grad_epsw(tgpu_handle h, const double *x, int kind, int icomp, const double *dvext_deps, double tol,
                   int max_iter, double *dF_deps, int *iters);
/* Schur complement on the density block ([ncomp][N] in and out) */
int tgpu_schur_apply(tgpu_handle h, const double *v2, double *y2);
int tgpu_schur_apply_device(tgpu_handle h, const double *d_v2, double *d_y2);
/* b2S = b2 - A21 A11^-1 b1 from a full right-hand side b ([nunk][N]) */
int tgpu_schur_rhs_device(tgpu_handle h, const double *d_b, double *d_b2s);
/* x1 = A11^-1 (b1 - A12 x2); writes the block-1 unknowns of d_x ([nunk][N]) and copies x2 in */
int tgpu_schur_x1_device(tgpu_handle h, const double *d_b, const double *d_x2, double *d_x);
/* Newton step: solve J dx = b (b = -R) by GMRES on the Schur complement with
 * A22 as left preconditioner; stops on ||M^-1 r|| / ||M^-1 r0|| < tol. */
int tgpu_solve(tgpu_handle h, const double *b, double *dx, double tol, int max_iter, int *iters, double *relres);
int tgpu_solve_device(tgpu_handle h, const double *d_b, double *d_dx, double tol, int max_iter, int *iters,
                      double *relres);
/* Damped Newton of src/dft_newton.c:131-381 on host-resident x ([nunk][N], updated in place).
 * Stops when the weighted update norm ||frac*dx/(rel_tol*x+abs_tol)|| <= 1. */
int tgpu_newton(tgpu_handle h, double *x, double rel_tol, double abs_tol, double update_floor, int max_iter,
                double lin_tol, int lin_max_iter, int *iters, double *final_resid_norm);
int tgpu_newton_device(tgpu_handle h, double *d_x, double rel_tol, double abs_tol, double update_floor,
                       int max_iter, double lin_tol, int lin_max_iter, int *iters, double *final_resid_norm);

/* Newton solve to a residual target: iterate until ||R||_2 <= resid_tol, R in
 * FP64-accurate arithmetic; inexact-Newton GMRES tolerances (Eisenstat-Walker,
 * floor lin_tol); damped update as update_solution (src/dft_newton.c:266-381).
 * Returns TGPU_ERR_NOCONV after max_iter iterations.  lin_iters_total: GMRES
 * iterations summed over the solve. */
int tgpu_newton_solve(tgpu_handle h, double *x, double resid_tol, int max_iter, double lin_tol, int lin_max_iter,
                      double update_floor, int *iters, double *final_resid, int *lin_iters_total);
int tgpu_newton_solve_device(tgpu_handle h, double *d_x, double resid_tol, int max_iter, double lin_tol,
                             int lin_max_iter, double update_floor, int *iters, double *final_resid,
                             int *lin_iters_total);

/* ---- set-up helpers ----------------------------------------------------------
 * Stencil tables built as calc_stencils (src/dft_stencil.c:40-287) builds
 * Stencil[type][0][index] for the delta shell (DELTA_FN_R), the theta ball
 * (THETA_FN_R) and the WCA attraction (THETA_PAIRPOT_RCUT, Type_attr 0 with the
 * cut-and-shifted LJ 12-6 tail, src/dft_stencil_theta_uattr.c:35-158).
 * Call with offsets == NULL to get the length; then with arrays of that
 * capacity.  hw (may be NULL) receives the per-corner weights [L][2^ndim].
 * Returns the length or a negative tgpu_status. */
int tgpu_make_stencil(int type, int ndim, const double *esize, double hs_diam, double sigma, double eps_over_kT,
                      double rcut, double rmin, int capacity, short *offsets, double *weights, double *hw,
                      double *volume);
/* The same tables built on the GPU (current device): one thread per element for the quadrature, one per
 * node for the corner sums, first-touch ordering by a radix sort and the renormalisation sum in table order.
 * The tables are bit-identical to tgpu_make_stencil's (both builders perform the same IEEE operations in
 * the same order).  Same arguments and return value; TGPU_ERR_CUDA without a usable device. */
int tgpu_make_stencil_device(int type, int ndim, const double *esize, double hs_diam, double sigma,
                             double eps_over_kT, double rcut, double rmin, int capacity, short *offsets,
                             double *weights, double *hw, double *volume);
/* External field of planar walls, generated on the GPU (the surfaces and wall-fluid potentials of
 * setup_external_field_n, src/dft_vext.c:38, for planar walls: Vext_LJ9_3_CS src/dft_vext_1D.c:42-56,
 * the 12-3 form, rough surfaces as in surface roughness patches, src/dft_surfacesAdjust_roughness.c:38-62).
 * Each wall faces +x (side 0: surface at x = position + h, d = x - position - h) or -x (side 1: surface at
 * x = position - h, d = position - h - x), x = ix esize[0]; h is the roughness height of the patch that
 * holds the node: heights[py][pz] (row-major) over patches[0] x patches[1] equal patches of the periodic
 * y (and z) extent, h = 0 without heights.  Per wall, with s = sigma/d:
 *   TGPU_WALL_LJ93_CS: eps (2 pi/3) sigma^3 [(2/15)(s^9 - (sigma/cut)^9) - (s^3 - (sigma/cut)^3)], 0 beyond cut
 *   TGPU_WALL_LJ123:   eps (s^12 - s^3)
 * eps is in kT and carries every prefactor; in 2-D and 3-D it is modulated along y as
 * eps (1 + pattern cos(2 pi y / L_y)), y = iy esize[1], L_y = nx[1] esize[1].  The field is the sum over
 * the walls; nodes with d <= 0 for some wall or a sum >= vext_max hold vext_max (zero-density rows).
 * Output [N] (node = ix + nx0 (iy + nx1 iz)).  No reference counterpart as a single call. */
enum { TGPU_WALL_LJ93_CS = 0, TGPU_WALL_LJ123 = 1 };
typedef struct {
  int form, side;
  double position, eps, sigma, cut, pattern;
  int patches[2];
  const double *heights;     /* host array [patches[0]][patches[1]] or NULL */
} tgpu_wall;
typedef struct {
  int ndim, nx[3];
  double esize[3];
  int nwalls;                /* 1 or 2 */
  tgpu_wall wall[2];
  double vext_max;
} tgpu_wall_field;
/* the field into device memory d_out [N] (current device, default stream, synchronised) */
int tgpu_wall_field_device(const tgpu_wall_field *f, double *d_out);
/* the same into host memory out [N] */
int tgpu_wall_field_host(const tgpu_wall_field *f, double *out);
/* Mean-field attraction stencils for the reference's other pair potentials and cores (THETA_PAIRPOT_RCUT
 * with Type_pairPot and the core that Type_attr selects, src/dft_defs_stencil.c:85-103):
 *   pot         TGPU_PAIR_LJ12_6_CS, TGPU_PAIR_YUKAWA_CS, TGPU_PAIR_EXP_CS, TGPU_PAIR_SW (Type_pairPot values)
 *   core_r      LJ only: TGPU_CORE_SIGMA, TGPU_CORE_UMIN, TGPU_CORE_UCSZERO, TGPU_CORE_SIGTOUMIN (Type_CoreATT_R)
 *   core_const  TGPU_CORECONST_UCONST (u held at its core value), TGPU_CORECONST_ZERO (Type_CoreATT_CONST)
 *   rmin, rzero LJ: the potential's minimum (tgpu_lj_rmin) and the zero of its cut-and-shifted form
 *   kappa       YukawaK_ff: K sigma for Yukawa, the decay length for the exponential
 * The Yukawa and exponential weights call exp(), whose last bit may differ between the host and the GPU: their
 * device tables agree with the host's to rounding; the LJ and square-well tables are bit-identical. */
enum { TGPU_PAIR_LJ12_6_CS = 0, TGPU_PAIR_YUKAWA_CS = 3, TGPU_PAIR_EXP_CS = 4, TGPU_PAIR_SW = 5 };
enum { TGPU_CORE_SIGMA = 0, TGPU_CORE_UMIN = 1, TGPU_CORE_UCSZERO = 2, TGPU_CORE_SIGTOUMIN = 3 };
enum { TGPU_CORECONST_UCONST = 0, TGPU_CORECONST_ZERO = 1 };
typedef struct {
  int pot, core_r, core_const;
  double sigma, eps_over_kT, rcut;
  double rmin, rzero, kappa;
} tgpu_pairpot;
int tgpu_make_attraction_stencil(const tgpu_pairpot *pp, int ndim, const double *esize, int device, int capacity,
                                 short *offsets, double *weights, double *hw, double *volume);
/* the attractive part u_att(r) in kT of the pair potential pp (pairPot_ATT_CS_switch, src/dft_switch_pairPot.c) */
double tgpu_pairpot_att(double r, const tgpu_pairpot *pp);
/* r of the minimum of the cut-and-shifted LJ 12-6 potential, located by the
 * search of pairPot_find_rmin (src/dft_pairPot.c:98-152) */
double tgpu_lj_rmin(double sigma, double eps_over_kT, double rcut, double esize0);

/* ---- Surfaces and their external fields (set-up; src/dft_surfaces.c setup_surface, src/dft_mesh.c
 * boundary flags, src/dft_vext.c setup_external_field_n and setup_integrated_LJ_walls) ----
 * The mesh is the reference's: Nodes_x = Size_x/Esize_x + 1 (Size_x/Esize_x when both ends are
 * periodic), Elements_x = Size_x/Esize_x, node i at -Size_x/2 + i Esize_x, node and element index
 * x fastest.  Each wall is a surface of one wall type placed at wall_pos (WallPos, dft_surfaces.dat).
 * An element belongs to a wall when the surface test of its type (Surf_type) holds at the element
 * centre (the reference's surface_*_inSurfaceTest), with the distance adjustment of the type's
 * linear and periodic overlays (surface_linear_offset, surface_periodic_offset).  A node has zero
 * density when no element around it is fluid for some wall (elements beyond an IN_WALL face count
 * for no wall, beyond an IN_BULK face as fluid) or one wall owns all of them (src/dft_mesh.c:1060-1145).
 * Walls of an integrated type (Ipot_wf_n = 5, Type_vext = VEXT_PAIR_POTENTIAL with the LJ 12-6 cut and
 * shifted pair potential) add, at every other node, the wall-fluid potential integrated over each of
 * their elements, their periodic and reflected images and, on IN_WALL / LAST_NODE faces, the element's
 * copies beyond the face (max cut / Esize of them), in the reference's order, each sum stopped at
 * vext_max once reached (setup_integrated_LJ_walls, src/dft_vext.c:671-865, integrate_potential and
 * get_wt_from_sten, src/dft_vext_integrated.c:42-200).  Zero-density nodes hold vext_max, and a node
 * whose field reaches vext_max has zero density (src/dft_vext.c:150-167).
 * Walls of Ipot_wf_n 2 and 3 add, at every other node, a potential of the distance X_wall from the node
 * to the wall's surface (or centre) as the surface test measures it with the overlay adjustment of the
 * node's element (src/dft_surfaces.c:400-430): a 1-D wall form (Type_vext 0) or the LJ 12-6 pair
 * potential (Type_vext 1), a node with X_wall <= 0.001 holding vext_max (setup_vext_XRSurf,
 * src/dft_vext.c:364-436); wall images add nothing (their X_wall is 1000, beyond every cut).
 * Roughness (Lrough_surf): the surface test's distance adjustment adds the height of the patch that
 * holds the element centre — patches of the planar, cylinder (2-D) and cylinder / pore (3-D) surfaces as
 * surface_*_roughness (src/dft_surfacesAdjust_roughness.c) — from the table Rough_precalc[type][100][100]
 * that the reference fills with the C library's rand() after srand(135649), for every wall type in
 * order (src/dft_setup_params.c:303-331); the library fills it with a restatement of glibc's rand()
 * (the additive feedback generator of random_r), so surfaces match a reference built on glibc.  A patch
 * index of 100 or more is TGPU_ERR_ARG (the reference exits there).
 * Angle cutouts (LangleCutout_surf; surface_angleCutout2D and surface_angleCutout3D_cyl,
 * src/dft_surfacesAdjust_angleCutout.c:40-139) restrict planar, cylinder, sphere and pore surfaces to a
 * wedge of angles about the wall centre (blocks have none); angle_start == angle_end is TGPU_ERR_ARG
 * (the reference leaves its test undefined there).
 * Not built (TGPU_ERR_UNSUPPORTED): Lhard_surf, semi-permeable walls, atomic and single-element
 * surfaces, 2-D slit pores of orientation 0, pair potentials other than LJ 12-6, the charged (LINEAR) and
 * Yukawa 1-D forms, Ipot_wf_n 4. */
#define TGPU_SURF_MAXWALLS 16
#define TGPU_SURF_MAXTYPES 16
#define TGPU_SURF_MAXFNC 4
/* Surf_type values (src/dft_globals_const.h surface ids): planar wall, finite block, cylinder (2-D) /
 * sphere (3-D), finite cylinder (3-D), cylindrical pore (2-D) / spherical cavity (3-D), slit pore (2-D) /
 * finite cylindrical pore (3-D) */
enum { TGPU_SURF_PLANAR = 0, TGPU_SURF_BLOCK = 1, TGPU_SURF_COLLOID = 2, TGPU_SURF_FINITE_CYL = 5,
       TGPU_SURF_PORE = 7, TGPU_SURF_FINITE_PORE = 8 };
/* Ipot_wf_n values: no wall-fluid term and hard walls (elements and zero density only), a potential of the
 * distance from the node to the surface or to the surface's centre, integrated LJ */
enum { TGPU_VEXT_NONE = 0, TGPU_VEXT_HARD = 1, TGPU_VEXT_DIST_TO_SURF = 2, TGPU_VEXT_DIST_TO_CENTER = 3,
       TGPU_VEXT_INTEGRATED = 5 };
/* Vext_PotentialID values of the 1-D wall forms (src/dft_vext_1D.c): 9-3 cut and shifted, its variant
 * without the 2 pi sigma^3 / 3 factor, 9-3 without the shift, the shifted-distance form, the 9 repulsion,
 * the attractive exponential */
enum { TGPU_WALL1D_LJ93_CS = 0, TGPU_WALL1D_LJ93_V2_CS = 1, TGPU_WALL1D_LJ93_NOCS = 2,
       TGPU_WALL1D_LJ93_SHIFTX_CS = 3, TGPU_WALL1D_REPULSIVE9 = 4, TGPU_WALL1D_EXP_ATT = 5 };
/* the reference's other boundary codes, read by the surface builder only */
enum { TGPU_BC_LAST_NODE = 3, TGPU_BC_LAST_NODE_RESTART = 4 };
typedef struct {
  int surf_type, orientation;          /* Surf_type, Orientation */
  double param[3];                     /* WallParam, WallParam_2, WallParam_3 */
  int nperiodic;                       /* periodic overlays: offset += amplitude cos(2 pi (x - origin)/wavelength) */
  int periodic_orient[TGPU_SURF_MAXFNC];
  double amplitude[TGPU_SURF_MAXFNC], wavelength[TGPU_SURF_MAXFNC], periodic_origin[TGPU_SURF_MAXFNC];
  int nlinear;                         /* linear overlays: offset += slope (x - origin) between origin and end */
  int linear_orient[TGPU_SURF_MAXFNC];
  double slope[TGPU_SURF_MAXFNC], linear_origin[TGPU_SURF_MAXFNC], linear_end[TGPU_SURF_MAXFNC];
  int cutout;                          /* LangleCutout_surf: the surface keeps only the elements whose angle
                                          about the wall centre lies in [angle_start, angle_end] (degrees;
                                          wrapping past 360 when angle_end < angle_start) */
  double angle_start, angle_end;       /* Angle_start, Angle_end */
  int rough;                           /* Lrough_surf: roughness patches of rough_length, heights in
                                          [-rough_max/2, rough_max/2) */
  double rough_max, rough_length;      /* Rough_param_max, Rough_length */
  int ipot_wf;                         /* TGPU_VEXT_* (Ipot_wf_n) */
  int type_vext;                       /* Type_vext: 0 a 1-D wall form (VEXT_DEFINED), 1 the pair potential */
  int pot_id;                          /* Vext_PotentialID: a TGPU_WALL1D_* form, or 0 (LJ 12-6) for type_vext 1 */
  double rho_w;                        /* Rho_w: the 1-D forms' prefactor is eps_wf rho_w */
  double sigma_wf[TGPU_MAXC], eps_wf[TGPU_MAXC], cut_wf[TGPU_MAXC];   /* eps in kT */
} tgpu_wall_type;
typedef struct {
  int ndim;
  double size[3], esize[3];            /* Size_x, Esize_x */
  int bc[3][2];                        /* Type_bc, TGPU_BC_* */
  int ncomp;
  double vext_max;                     /* VEXT_MAX */
  double sigma_ff[TGPU_MAXC];          /* Sigma_ff[i][i] (the shifted 9-3 form) */
  int apply_offset[3];                 /* Lapply_offset (radius, half-length, -) of the pore and cylinder tests */
  int ntypes;
  tgpu_wall_type type[TGPU_SURF_MAXTYPES];
  int nwalls;
  int wall_type[TGPU_SURF_MAXWALLS];
  double wall_pos[TGPU_SURF_MAXWALLS][3];
} tgpu_surface_spec;
/* nodes and elements per dimension of the spec's mesh (unused dims 1); TGPU_ERR_ARG when Size_x is
 * not a multiple of Esize_x */
int tgpu_surface_mesh(const tgpu_surface_spec *s, int *nodes, int *elements);
/* the surface set-up on the GPU: vext [ncomp][nodes], zero [ncomp][nodes] (1 = zero density) and, when
 * wall_el is not NULL, the walls of each element as a bit mask [elements].  Host buffers; the
 * _device variant takes device buffers (current device, default stream, synchronised). */
int tgpu_surface_field_host(const tgpu_surface_spec *s, double *vext, signed char *zero, unsigned short *wall_el);
/* the roughness patch heights the builder uses, [ntypes][100][100] (host only, no GPU) */
int tgpu_surface_rough_table(const tgpu_surface_spec *s, double *out);
int tgpu_surface_field_device(const tgpu_surface_spec *s, double *d_vext, signed char *d_zero,
                              unsigned short *d_wall_el);
/* the WCA attraction u_att(r) in kT (uLJ12_6_ATT_CS, src/dft_pairPot_LJ12_6.c:128-168) */
double tgpu_uatt(double r, double sigma, double eps_over_kT, double rcut, double rmin);

/* ---- allocation-free stencil sum -------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory where they need a weighted-density sum: code inside a framework that
 * owns all device allocations (its buffers come in as pointers and the op may
 * not call cudaMalloc), or code that must not allocate between two phases of
 * a larger computation.  Computes, for one density field,
 *     out[i] = sum_k weights[k] * field(i + offsets[k])
 * with the reference's boundary rules (src/dft_mesh_lib.c:203-297): bulk
 * sentinel -> bulk_value, inside a wall -> 0, periodic wrap, mirror for
 * REFLECT.  d_field and d_out are device arrays of prod(nx) doubles; bc is
 * [ndim][2] flattened; offsets/weights are host arrays ([length][ndim], [length]).
 * The padded copy of the field, the boundary maps and the stencil table live in
 * fixed arrays inside the library (about 18 MB per GPU that loads it, held
 * until exit): the padded box (nx + 2*reach per dimension, multiplied) may
 * not exceed TGPU_NOALLOC_MAX_PADDED points, nor the stencil
 * TGPU_NOALLOC_MAX_STENCIL points, nor any padded extent 4096; larger inputs
 * return TGPU_ERR_ARG with a message in tgpu_noalloc_last_error().  A stencil
 * that reaches past what the boundary rules can map (a periodic reach longer
 * than the box, or a mirrored point beyond the far side when that side is
 * periodic or reflecting) returns TGPU_ERR_UNSUPPORTED.  These checks run on
 * the host before any device work.  The first
 * call on a device looks up the device addresses of those arrays.  Every call shares the arrays and
 * rewrites what it reads; calls whose work overlaps on the GPU race.  Returns
 * after the sum is complete on `stream` (NULL: the legacy default stream). */
#define TGPU_NOALLOC_MAX_PADDED 2097152
#define TGPU_NOALLOC_MAX_STENCIL 131072
int tgpu_stencil_sum_noalloc(int ndim, const int *nx, const int *bc, double bulk_value, int length,
                             const short *offsets, const double *weights, const double *d_field, double *d_out,
                             void *stream);
const char *tgpu_noalloc_last_error(void);

/* Benchmark hook: device time (CUDA events on the handle's stream) of one
 * forward stencil sum with stencil (type, index) over the density of the last
 * fill, in TGPU_FP64, TGPU_FP32, TGPU_FP16TC, TGPU_FILL_FF (the float-float sum
 * of the accurate fills), TGPU_FILL_FFT (the FP64 FFT convolution, forward transform included) or
 * TGPU_TIME_FFT32 (the FP32 FFT convolution that FP32 products and fills take where it is faster),
 * averaged over reps launches.  TGPU_FP32 and TGPU_FP16TC time the direct kernels. */
#define TGPU_TIME_FFT32 16
int tgpu_time_stencil_sum(tgpu_handle h, int type, int index, int precision, int reps, double *ms_per_sum);

/* Times every launch of the FP32 y/z FFT pass kernel (the solves' leading kernel) between begin and end with a CUDA
 * event pair on its stream: launches, summed duration, algorithmic bytes (per transform the complex FP32 half
 * spectrum written once and read once, or each spectral product's two operands read) and transforms.  The
 * timer is process-wide; the events add gaps between launches, not to them. */
int tgpu_pass_timer_begin(tgpu_handle h);
int tgpu_pass_timer_end(tgpu_handle h, long *launches, double *ms_total, double *bytes_total, long *transforms);
/* Benchmark hook: device time (CUDA events on the handle's stream) of one forward y (axis 1) or z (axis 2) pass of
 * the 3-D FFT sums over a half-spectrum work box, TGPU_FP32 or TGPU_FP64, averaged over reps; box_points receives
 * the half spectrum's size (each pass reads and writes it once), real_points the real transform box's (either may
 * be NULL).  No reference counterpart. */
int tgpu_time_fft_pass(tgpu_handle h, int precision, int axis, int reps, double *ms_per_pass, long *box_points,
                       long *real_points);

/* Diagnostics hook: the limit (try-wait attempts) of the tensor-core stencil sum's pipeline waits; spins <= 0
 * restores the default.  A wait that runs out stops the kernel's pipeline, which drains the copies and MMAs it
 * started (those waits keep the default limit), frees its tensor memory and leaves an error flag that the call
 * reports as TGPU_ERR_CUDA ("a bounded wait ran out").  A tiny limit makes the waits run out on purpose, to
 * exercise that path.  No reference counterpart. */
int tgpu_set_tc_wait_limit(tgpu_handle h, long spins);

/* Timing of the device work of the last call, per kernel family (ms), for benchmarks. */
typedef struct {
  double fill_ms, schur_ms, conv_ms, gmres_ms;
  long schur_applies, conv_launches, kernel_launches, fp64_refreshes;
} tgpu_stats;
int tgpu_get_stats(tgpu_handle h, tgpu_stats *out);
int tgpu_reset_stats(tgpu_handle h);

#ifdef __cplusplus
}
#endif
#endif
