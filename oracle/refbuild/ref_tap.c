/* Harness entry points into the reference's own C code (oracle build only).
 *
 * tref_setup() runs the set-up half of dftmain (src/dft_main.c:134-300:
 * parameters, stencils, bulk thermodynamics, mesh, boundaries, integrals)
 * and the initial guess of solve_problem (src/dft_newton.c:58-63), then
 * stops.  tref_fill() calls the reference's fill_resid_and_matrix_control
 * (src/dft_fill_control.c:39) on a caller-supplied solution vector; the
 * recording manager in ref_linprobmgr.cpp keeps the rhs and Jacobian it
 * produced.  The tref_get_* functions copy the reference's globals (stencil
 * tables, bulk constants, external field, flags) out for the oracle tests.
 * tref_run() runs dftmain itself: Newton to convergence plus the reference's
 * post-processing, which writes dft_output.dat in the working directory.
 *
 * Nothing here changes the reference's algorithms; this file only sequences
 * calls that dftmain makes and reads the globals they fill in. */
#include <string.h>
#include <unistd.h>
#include "dft_globals_const.h"
#include "rf_allo.h"

void setup_params_for_dft(char *input_file, char *file_echoinput);
void setup_stencil_logicals(void);
void setup_stencil_uattr_core_properties(void);
void setup_nunk_per_node(char *file_echoinput);
void setup_pairPotentials(char *file_echoinput);
void calc_HS_diams(void);
void calc_stencils(void);
void thermodynamics(char *file_echoinput, int iwrite_screen, int iwrite_files);
void set_up_mesh(char *file_echoinput, char *output_file2);
void boundary_setup(char *file_echoinput);
void setup_domain_multipliers(void);
void setup_integrals(void);
void set_initial_guess(int guess_type, double **xOwned);
double fill_resid_and_matrix_control(double **x, int iter, int resid_only_flag);
int newton_solver(double **x, void *con_ptr);
void dftmain(double *engptr);

static double **g_x = NULL;

int tref_run(const char *dir, double *energy)
{
  if (chdir(dir) != 0) return -1;
  dftmain(energy);
  return 0;
}

int tref_setup(const char *dir)
{
  char *echo;
  double **xOwned;
  if (chdir(dir) != 0) return -1;
  MPI_Comm_size(MPI_COMM_WORLD, &Num_Proc);
  MPI_Comm_rank(MPI_COMM_WORLD, &Proc);
  setup_params_for_dft("dft_input.dat", "dft_out.lis");
  echo = EchoInputFile_array;
  setup_stencil_logicals();
  if (Type_attr != NONE) setup_stencil_uattr_core_properties();
  setup_nunk_per_node(echo);
  setup_pairPotentials(echo);
  Imain_loop = 0;
  if (Type_func != NONE) calc_HS_diams();
  calc_stencils();
  thermodynamics(echo, Iwrite_screen, Iwrite_files);
  set_up_mesh(echo, "dft_vext.dat");
  boundary_setup(echo);
  Nnodes_box_extra = Nnodes_box;
  setup_domain_multipliers();
  setup_integrals();
  g_x = (double **)array_alloc(2, Nunk_per_node, Nnodes_box, sizeof(double));
  xOwned = (double **)array_alloc(2, Nunk_per_node, Nnodes_per_proc, sizeof(double));
  set_initial_guess(Iguess, xOwned);
  dft_linprobmgr_importr2c(LinProbMgr_manager, xOwned, g_x);
  safe_free((void **)&xOwned);
  return 0;
}

/* ints: Ndim Nodes_x[3] Nnodes Nnodes_box Nnodes_per_proc Nunk_per_node Ncomp
 * Nrho_bar_s Type_func Type_attr ATTInA22Block Lhard_surf Nlists_HW Nwall
 * Type_bc[3][2] Phys2Unk_first[DENSITY,HSRHOBAR,MF_EQ] Nzone Nodes_x_box[3]
 * Max_sten_length[3] Pflag[3] Iguess Type_interface Mesh_coarsening Coarser_jac
 * Nnodes_per_el_V Type_pairPot Lcut_jac Type_CoreATT_R Type_CoreATT_CONST Lconstrain_interface Grad_dim
 * L1D_bc Dim_1Dbc */
int tref_info_ints(int *o)
{
  int k = 0, i;
  o[k++] = Ndim;
  for (i = 0; i < 3; i++) o[k++] = i < Ndim ? Nodes_x[i] : 1;
  o[k++] = Nnodes; o[k++] = Nnodes_box; o[k++] = Nnodes_per_proc; o[k++] = Nunk_per_node;
  o[k++] = Ncomp; o[k++] = Nrho_bar_s; o[k++] = Type_func; o[k++] = Type_attr;
  o[k++] = ATTInA22Block; o[k++] = Lhard_surf; o[k++] = Nlists_HW; o[k++] = Nwall;
  for (i = 0; i < 3; i++) { o[k++] = Type_bc[i][0]; o[k++] = Type_bc[i][1]; }
  o[k++] = Phys2Unk_first[DENSITY]; o[k++] = Phys2Unk_first[HSRHOBAR]; o[k++] = Phys2Unk_first[MF_EQ];
  o[k++] = Nzone;
  for (i = 0; i < 3; i++) o[k++] = i < Ndim ? Nodes_x_box[i] : 1;
  for (i = 0; i < 3; i++) o[k++] = Max_sten_length[i];
  for (i = 0; i < 3; i++) o[k++] = Pflag[i];
  o[k++] = Iguess; o[k++] = Type_interface; o[k++] = Mesh_coarsening; o[k++] = Coarser_jac;
  o[k++] = Nnodes_per_el_V; o[k++] = Type_pairPot; o[k++] = Lcut_jac;
  o[k++] = Type_CoreATT_R; o[k++] = Type_CoreATT_CONST;
  o[k++] = Lconstrain_interface; o[k++] = Grad_dim;
  o[k++] = L1D_bc; o[k++] = Dim_1Dbc;
  return k;
}

/* doubles: Esize_x[3] Size_x[3] VEXT_MAX then per component (NCOMP_MAX each):
 * HS_diam Rho_b Betamu_hs_ex Betamu_att Inv_rad Inv_4pir Inv_4pirsq
 * Fac_overlap_hs, then Rhobar_b[10] Dphi_Drhobar_b[10], Avdw[NCOMP_MAX^2],
 * Eps_ff Sigma_ff Cut_ff [NCOMP_MAX^2 each], Temp, Jac_threshold, then YukawaK_ff Rmin_ff Rzero_ff
 * [NCOMP_MAX^2 each], Rho_b_LBB Rho_b_RTF [NCOMP_MAX each], Dphi_Drhobar_LBB Dphi_Drhobar_RTF [10 each],
 * Betamu [NCOMP_MAX] */
int tref_info_doubles(double *o)
{
  int k = 0, i, j;
  for (i = 0; i < 3; i++) o[k++] = i < Ndim ? Esize_x[i] : 0.0;
  for (i = 0; i < 3; i++) o[k++] = i < Ndim ? Size_x[i] : 0.0;
  o[k++] = VEXT_MAX;
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = HS_diam[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Rho_b[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Betamu_hs_ex[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Betamu_att[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Inv_rad[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Inv_4pir[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Inv_4pirsq[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Fac_overlap_hs[i];
  for (i = 0; i < 10; i++) o[k++] = Rhobar_b[i];
  for (i = 0; i < 10; i++) o[k++] = Dphi_Drhobar_b[i];
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = Avdw[i][j];
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = Eps_ff[i][j];
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = Sigma_ff[i][j];
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = Cut_ff[i][j];
  o[k++] = Temp;
  o[k++] = Jac_threshold;
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = YukawaK_ff[i][j];
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = Rmin_ff[i][j];
  for (i = 0; i < NCOMP_MAX; i++) for (j = 0; j < NCOMP_MAX; j++) o[k++] = Rzero_ff[i][j];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Rho_b_LBB[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Rho_b_RTF[i];
  for (i = 0; i < 10; i++) o[k++] = Dphi_Drhobar_LBB[i];
  for (i = 0; i < 10; i++) o[k++] = Dphi_Drhobar_RTF[i];
  for (i = 0; i < NCOMP_MAX; i++) o[k++] = Betamu[i];
  return k;
}

int tref_get_x(double *out)
{
  int u;
  for (u = 0; u < Nunk_per_node; u++) memcpy(out + (size_t)u * Nnodes_box, g_x[u], sizeof(double) * Nnodes_box);
  return 0;
}

int tref_set_x(const double *in)
{
  int u;
  for (u = 0; u < Nunk_per_node; u++) memcpy(g_x[u], in + (size_t)u * Nnodes_box, sizeof(double) * Nnodes_box);
  return 0;
}

/* One call of the reference fill on the current x; resid_only_flag as in
 * src/dft_globals_const.h:422-424 (0 = rhs + Jacobian, 1 = rhs only). */
int tref_fill(int iter, int flag, double *resid_sum)
{
  dft_linprobmgr_initializeproblemvalues(LinProbMgr_manager);
  *resid_sum = fill_resid_and_matrix_control(g_x, iter, flag);
  dft_linprobmgr_finalizeproblemvalues(LinProbMgr_manager);
  return 0;
}

int tref_newton(void)
{
  return newton_solver(g_x, NULL);
}

int tref_stencil_length(int isten, int izone, int index)
{
  if (!Sten_Type[isten]) return -1;
  return Stencil[isten][izone][index].Length;
}

int tref_stencil(int isten, int izone, int index, int *offsets, double *weights, double *hw)
{
  struct Stencil_Struct *s = &Stencil[isten][izone][index];
  int i, d, l;
  for (i = 0; i < s->Length; i++) {
    for (d = 0; d < Ndim; d++) offsets[i * Ndim + d] = s->Offset[i][d];
    weights[i] = s->Weight[i];
    if (hw && Lhard_surf)
      for (l = 0; l < Nnodes_per_el_V; l++) hw[i * Nnodes_per_el_V + l] = s->HW_Weight[i][l];
  }
  return s->Length;
}

/* Vext[loc_inode][icomp] -> out[icomp][loc_inode] */
int tref_get_vext(double *out)
{
  int i, c;
  for (c = 0; c < Ncomp; c++)
    for (i = 0; i < Nnodes_per_proc; i++) out[(size_t)c * Nnodes_per_proc + i] = Nwall > 0 ? Vext[i][c] : 0.0;
  return 0;
}

/* Replace the external field (same layout as tref_get_vext) */
int tref_set_vext(const double *in)
{
  int i, c;
  if (Nwall <= 0) return -1;
  for (c = 0; c < Ncomp; c++)
    for (i = 0; i < Nnodes_per_proc; i++) Vext[i][c] = in[(size_t)c * Nnodes_per_proc + i];
  return 0;
}

/* Zero_density_TF[inode_box][icomp] -> out[icomp][inode_box] */
int tref_get_zero_density(int *out)
{
  int i, c;
  for (c = 0; c < Ncomp; c++)
    for (i = 0; i < Nnodes_box; i++) out[(size_t)c * Nnodes_box + i] = Zero_density_TF[i][c];
  return 0;
}

/* Mesh_coarsen_flag[inode_box] (Nnodes_box): the residual zone of a node, or < 0 for a node whose
 * rows average its neighbours (set_mesh_coarsen_flag, src/dft_mesh.c:2788-2850); -1 when unset */
int tref_get_coarsen_flag(int *out)
{
  int i;
  if (Mesh_coarsen_flag == NULL) return -1;
  for (i = 0; i < Nnodes_box; i++) out[i] = Mesh_coarsen_flag[i];
  return 0;
}

/* Nodes_2_boundary_wall[ilist][inode_box] for all lists (Nlists_HW * Nnodes_box) */
int tref_get_boundary_nodes(int *out)
{
  int l, i;
  if (Nodes_2_boundary_wall == NULL) return -1;
  for (l = 0; l < Nlists_HW; l++)
    for (i = 0; i < Nnodes_box; i++) out[(size_t)l * Nnodes_box + i] = Nodes_2_boundary_wall[l][i];
  return 0;
}

/* Per box node, list and reflection pattern: bit ln set when the element that
 * has the node as local node ln (src/dft_mesh_lib.c:877
 * node_box_to_elem_box_reflect) is a fluid element in the sense of
 * HW_boundary_weight (src/dft_utils.c:41-62).  out[(ilist*2^Ndim + r)*Nnodes_box + inode]
 * with r the reflect_flag bits (bit d = reflected in dimension d). */
int node_box_to_elem_box_reflect(int inode_box, int local_node, int *reflect_flag);
int tref_get_fluid_masks(int *out)
{
  int l, r, i, ln, d, icomp, fluid, rf[3];
  int nrefl = 1 << Ndim;
  if (Wall_elems == NULL) return -1;
  for (l = 0; l < Nlists_HW; l++)
    for (r = 0; r < nrefl; r++) {
      for (d = 0; d < 3; d++) rf[d] = (d < Ndim) ? ((r >> d) & 1) : 0;
      for (i = 0; i < Nnodes_box; i++) {
        int mask = 0;
        for (ln = 0; ln < Nnodes_per_el_V; ln++) {
          int iel = node_box_to_elem_box_reflect(i, ln, rf);
          if (iel < 0) continue;
          fluid = Wall_elems[l][iel] == -1;
          if (!fluid) {
            /* semipermeable walls count as fluid for the component of the list */
            icomp = (Nlists_HW <= 2) ? 0 : l;
            if (Lsemiperm[WallType[Wall_elems[l][iel]]][icomp]) fluid = 1;
          }
          if (fluid) mask |= 1 << ln;
        }
        out[((size_t)l * nrefl + r) * Nnodes_box + i] = mask;
      }
    }
  return 0;
}

int tref_maps(int *l2b, int *b2g)
{
  int i;
  for (i = 0; i < Nnodes_per_proc; i++) l2b[i] = L2B_node[i];
  for (i = 0; i < Nnodes_box; i++) b2g[i] = B2G_node[i];
  return 0;
}

/* The classification linsolver_setup_HSTYPE applies (src/dft_linsolver_setup.c:196-226),
 * used by the recording manager when the run selected the basic manager. */
void tref_classify_unknowns(int *ind, int *nind, int *dep, int *ndep, int *dens, int *ndens)
{
  int iunk, one_size;
  *nind = *ndep = *ndens = 0;
  one_size = (Lhard_surf && Nlists_HW == 2) || (!Lhard_surf && Nlists_HW == 1);
  for (iunk = 0; iunk < Nunk_per_node; iunk++) {
    switch (Unk2Phys[iunk]) {
      case DENSITY:
        dens[(*ndens)++] = iunk;
        break;
      case HSRHOBAR:
        if (one_size && ((iunk > Phys2Unk_first[HSRHOBAR] + 1 && iunk < Phys2Unk_first[HSRHOBAR] + Nrho_bar_s) ||
                         iunk >= Phys2Unk_first[HSRHOBAR] + Nrho_bar_s + Ndim))
          dep[(*ndep)++] = iunk;
        else
          ind[(*nind)++] = iunk;
        break;
      default:
        ind[(*nind)++] = iunk;
        break;
    }
  }
}

/* Integration data of setup_integrals / setup_domain_multipliers (src/dft_out_utils.c:141-270):
 * hit = Nel_hit, hit2 = Nel_hit2 as [Ncomp][Nnodes_per_proc];
 * d = {Vol_el, Nnodes_per_el_V, Area, Fac_vol, Fac_area, Lper_area, Betamu[0..Ncomp-1]}. */
extern int **Nel_hit, **Nel_hit2;
extern double Area, Fac_vol, Fac_area, Vol_el;
extern int Lper_area;
int tref_integration(int *hit, int *hit2, double *d)
{
  int c, i;
  for (c = 0; c < Ncomp; c++)
    for (i = 0; i < Nnodes_per_proc; i++) {
      hit[(size_t)c * Nnodes_per_proc + i] = Nel_hit[c][L2B_node[i]];
      hit2[(size_t)c * Nnodes_per_proc + i] = Nel_hit2[c][L2B_node[i]];
    }
  d[0] = Vol_el;
  d[1] = Nnodes_per_el_V;
  d[2] = Area;
  d[3] = Fac_vol;
  d[4] = Fac_area;
  d[5] = Lper_area;
  for (c = 0; c < Ncomp; c++) d[6 + c] = Betamu[c];
  return 6 + Ncomp;
}

/* Surface excess free energy (calc_free_energy, src/dft_energy.c:31) and the
 * adsorption integrals of calc_adsorption (src/dft_out_ads.c:33-112) of the
 * current state: ads[icomp] over Nel_hit2, ads_b[icomp] over Nel_hit. */
double calc_free_energy(FILE *fp, double **x);
double integrateInSpace(double (*fp_integrand)(int, int, double **), int iunk, int **nelhit, double **x,
                        double *profile);
double integrand_adsorption(int iunk, int inode_box, double **x);
double integrand_adsorption_bulk(int iunk, int inode_box, double **x);
int tref_energy(double *omega_s, double *ads, double *ads_b)
{
  int c;
  *omega_s = calc_free_energy(NULL, g_x);
  for (c = 0; c < Ncomp; c++) {
    ads[c] = integrateInSpace(&integrand_adsorption, Phys2Unk_first[DENSITY] + c, Nel_hit2, g_x, NULL);
    ads_b[c] = integrateInSpace(&integrand_adsorption_bulk, Phys2Unk_first[DENSITY] + c, Nel_hit, g_x, NULL);
  }
  return 0;
}

/* Surfaces: ints Nwall Nwall_type Nlists_HW Nelements_box Nwall_Images, WallType[Nwall];
 * doubles WallPos[Nwall][3], then Sigma_wf Eps_wf Cut_wf [Ncomp][Nwall_type] each (effective values
 * after mixing and scaling), then WallPos_Images[Nwall_Images][3] */
int tref_wall_info(int *oi, double *od)
{
  int k = 0, j = 0, i, w, d;
  oi[k++] = Nwall; oi[k++] = Nwall_type; oi[k++] = Nlists_HW; oi[k++] = Nelements_box; oi[k++] = Nwall_Images;
  for (w = 0; w < Nwall; w++) oi[k++] = WallType[w];
  for (w = 0; w < Nwall; w++) for (d = 0; d < 3; d++) od[j++] = d < Ndim ? WallPos[d][w] : 0.0;
  for (i = 0; i < Ncomp; i++) for (w = 0; w < Nwall_type; w++) od[j++] = Sigma_wf[i][w];
  for (i = 0; i < Ncomp; i++) for (w = 0; w < Nwall_type; w++) od[j++] = Eps_wf[i][w];
  for (i = 0; i < Ncomp; i++) for (w = 0; w < Nwall_type; w++) od[j++] = Cut_wf[i][w];
  for (w = 0; w < Nwall_Images; w++) for (d = 0; d < 3; d++) od[j++] = d < Ndim ? WallPos_Images[w][d] : 0.0;
  return k;
}

/* Wall_elems[Nlists_HW-1][iel_box] (the last wall that owns each element, -1 for fluid) */
int tref_wall_elems(int *out)
{
  int e;
  if (Wall_elems == NULL) return -1;
  for (e = 0; e < Nelements_box; e++) out[e] = Wall_elems[Nlists_HW - 1][e];
  return 0;
}
