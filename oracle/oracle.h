/* CPU restatement of the reference's nonlocal-density path (test infrastructure).
 *
 * This is the oracle the GPU path is checked against.  It restates, in plain
 * serial C with the reference's own loop order, the residual and Jacobian of
 * Tramonto's hard-sphere FMT + WCA mean-field fill:
 *   - calc_FMT_derivatives / FMT{1,2,3,4}_1stderiv (src/dft_fill_FMT.c:349-385,
 *       src/dft_physics_FMT1.c:59-77, src/dft_physics_FMT2.c:60-99, src/dft_physics_FMT3.c:61-96,
 *       src/dft_physics_FMT4.c:61-97)
 *   - load_rho_bar_s / load_rho_bar_v / resid_and_Jac_sten_fill_sum_Ncomp
 *       (src/dft_fill_FMT.c:195-347, src/dft_fill_CLSmf.c:38-171)
 *   - load_nonlocal_hs_rosen_rb with d2phi_drb2_{delta,theta}_rb_FMT{1,2,3,4}
 *       (src/dft_fill_FMT.c:41-189, src/dft_physics_FMT1.c:79-168, src/dft_physics_FMT2.c:104-250,
 *       src/dft_physics_FMT3.c:101-265, src/dft_physics_FMT4.c:102-275)
 *   - load_euler_lagrange (src/dft_fill_EL.c:38-196, 351-444) and load_mean_field (src/dft_fill_mf.c:38-63)
 *   - offset_to_node_box (src/dft_mesh_lib.c:203-297), HW_boundary_weight (src/dft_utils.c:41-62),
 *     constant_boundary (src/dft_utils.c:89-110)
 *   - the hard-sphere Schur operator S = A22 - A21 A11^-1 A12 (src/dft_Schur_Epetra_Operator.cpp:86-119,
 *     src/dft_HardSphereA11_Epetra_Operator.cpp:130-197)
 * It is pinned against golden vectors produced by the reference itself
 * (tests/golden).  Only tests, the smoke check and the CPU baseline of
 * bench.py use it; the product never links it.
 *
 * Conventions: one process, the box equals the mesh; fields are SoA
 * [unknown][node] with node = ix + nx*(iy + ny*iz); unknown order as
 * setup_nunk_per_node (src/dft_defs_unknowns.c:37-176): densities,
 * weighted densities in solution-vector order (n3, n2, n1, n0, V2[d], V1[d]),
 * then mean-field unknowns. */
#ifndef TRAMONTO_ORACLE_H
#define TRAMONTO_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXC 4
#define ORC_MAXZ 5

enum { ORC_DELTA = 0, ORC_THETA = 1, ORC_UATT = 2 };
enum { ORC_BC_IN_WALL = -1, ORC_BC_IN_BULK = 0, ORC_BC_PERIODIC = 1, ORC_BC_REFLECT = 2 };
enum { ORC_FMT1 = 0, ORC_FMT2 = 1, ORC_FMT3 = 2, ORC_FMT4 = 3 };

typedef struct {
  int ndim, nx[3];
  double esize[3];
  int bc[3][2];
  int ncomp;
  int functional;      /* ORC_FMT1 .. ORC_FMT4 (Type_func) */
  int attraction;      /* WCA mean field on/off */
  int att_in_a22;      /* 0: mean field is its own unknown (MF_EQ rows); 1: summed into the EL rows */
  int single_size;     /* n1, n0, V1 are dependent unknowns (one particle size) */
  int hard_surf;       /* Lhard_surf: hard-wall boundary weights */
  int nlists_hw;
  int first_rho, first_rb, first_mf, nunk;
  double rho_b[ORC_MAXC], betamu_hs_ex[ORC_MAXC], betamu_att[ORC_MAXC];
  double inv_rad[ORC_MAXC], inv_4pir[ORC_MAXC], inv_4pirsq[ORC_MAXC], fac_overlap[ORC_MAXC];
  double dphi_bulk[4];        /* Dphi_Drhobar_b: bulk dPhi/dn0..dn3 */
  double vext_max;
  const double *vext;         /* [ncomp][N] */
  const signed char *zero_density; /* [ncomp][N] */
  const int *boundary_nodes;  /* [nlists][N], -1 when not a hard-wall boundary node */
  const short *fluid_masks;   /* [nlists][2^ndim][N], see tests/golden/make_golden.py */
  int sten_len[3][ORC_MAXC * ORC_MAXC];
  const short *sten_off[3][ORC_MAXC * ORC_MAXC];   /* [L][ndim] */
  const double *sten_w[3][ORC_MAXC * ORC_MAXC];    /* [L] */
  const double *sten_hw[3][ORC_MAXC * ORC_MAXC];   /* [L][2^ndim] or NULL */
  /* phase interface (Type_interface = PHASE_INTERFACE): stencil points beyond the low / high
   * bulk boundaries read the LBB / RTF states (offset_to_node_box -3 / -4), the Euler-Lagrange
   * rows take -Betamu as their chemical potential, and with Lconstrain_interface the first
   * density at pin_node is held at pin_value (fill_constant_density, src/dft_fill_EL.c:286-305) */
  int interface;              /* 0: uniform, 2: phase interface */
  double rho_b_lbb[ORC_MAXC], rho_b_rtf[ORC_MAXC];
  double dphi_lbb[4], dphi_rtf[4];
  double betamu[ORC_MAXC];
  long pin_node;              /* -1: no pinned density */
  double pin_value;
  /* quadrature zones and mesh coarsening (Nzone, Mesh_coarsening, Coarser_jac; calc_stencils
   * src/dft_stencil.c:96-109, 229-236; set_mesh_coarsen_flag src/dft_mesh.c:2788-2850):
   * zone_flag[N] is Mesh_coarsen_flag (NULL: zone 0 everywhere); a node with flag >= 0 fills its
   * residual with that zone's stencils (offsets in fine-node units), its Jacobian with find_jzone's
   * (src/dft_utils.c:67-86); flag -1/-2/-3 rows average the two neighbours along x/y/z
   * (load_coarse_node_Ndim, src/dft_fill_coarse.c:66-123).  Zone 0 uses the sten_* tables. */
  int nzone, mesh_coarsening, coarser_jac, nwall;
  const int *zone_flag;
  int zsten_len[ORC_MAXZ][3][ORC_MAXC * ORC_MAXC];
  const short *zsten_off[ORC_MAXZ][3][ORC_MAXC * ORC_MAXC];
  const double *zsten_w[ORC_MAXZ][3][ORC_MAXC * ORC_MAXC];
  const double *zsten_hw[ORC_MAXZ][3][ORC_MAXC * ORC_MAXC];
  double rhobar_bc[10];       /* Rhobar_b in solution order: constant_boundary of the rb unknowns */
  /* L1D_bc (src/dft_mesh.c:165-185, 2835-2841): nodes flagged -999 hold every unknown equal to the node
   * with the same coordinate along dim_1dbc and 0 along the others (load_coarse_node_1dim,
   * src/dft_fill_coarse.c:37-64).  Flags -888 (BULK_ZONE) and -777 (PB_ZONE) keep the bulk density, or
   * the ideal gas in the external field, in the Euler-Lagrange rows (fill_bulk_density
   * src/dft_fill_EL.c:265-284; the FLAG_PBELEC branches :132, :405-410); their other rows take zone 0's
   * stencils (the reference indexes its stencil table with the negative flag there). */
  int l1d_bc, dim_1dbc;
  double rhobar_lbb[10], rhobar_rtf[10];   /* Rhobar_b_LBB / _RTF (phase interface) in solution order */
} orc_problem;

long orc_nnodes(const orc_problem *p);
/* dPhi/dn at every node, [4+2*ndim][N] in reference order S0,S1,S2,S3,V1[d],V2[d] */
int orc_dphi(const orc_problem *p, const double *x, double *dphi);
/* full residual R(x) for every unknown and node (the reference's rhs is -R) */
int orc_resid(const orc_problem *p, const double *x, double *R);
/* Jacobian products with the reference's Jacobian entries at state x */
int orc_jv(const orc_problem *p, const double *x, const double *v, double *Jv);
int orc_jtv(const orc_problem *p, const double *x, const double *w, double *JTw);
/* Schur product S v2 on the density block ([ncomp][N] in and out); -2 with coarsened nodes, whose
 * unknowns the reference moves into the second block */
int orc_schur(const orc_problem *p, const double *x, const double *v2, double *Sv2);
/* Residual of the first `nrows` nodes only (bounded CPU samples); R is [nunk][N], other rows untouched */
int orc_resid_rows(const orc_problem *p, const double *x, double *R, long node_begin, long node_end);

#ifdef __cplusplus
}
#endif
#endif
