/* Constants of the Aztec option/parameter arrays referenced by the Tramonto
 * C sources.  Only the array indices matter for the oracle build: the
 * oracle's linear solver reads the tolerance and iteration cap from them. */
#ifndef TGPU_REF_SHIM_AZ_AZTEC_H
#define TGPU_REF_SHIM_AZ_AZTEC_H
#define AZ_OPTIONS_SIZE 48
#define AZ_PARAMS_SIZE 32
#define AZ_STATUS_SIZE 16
#define AZ_PROC_SIZE 8
/* option indices */
#define AZ_solver 0
#define AZ_scaling 1
#define AZ_precond 2
#define AZ_conv 3
#define AZ_output 4
#define AZ_pre_calc 5
#define AZ_max_iter 6
#define AZ_poly_ord 7
#define AZ_overlap 8
#define AZ_kspace 9
#define AZ_orthog 10
#define AZ_aux_vec 11
#define AZ_keep_info 12
#define AZ_subdomain_solve 13
#define AZ_reorder 14
#define AZ_type_overlap 15
/* parameter indices */
#define AZ_tol 0
#define AZ_drop 1
#define AZ_ilut_fill 2
#define AZ_omega 3
#define AZ_athresh 4
#define AZ_rthresh 5
/* option values */
#define AZ_gmres 1
#define AZ_cg 2
#define AZ_tfqmr 3
#define AZ_cgs 4
#define AZ_bicgstab 5
#define AZ_none 0
#define AZ_Jacobi 1
#define AZ_sym_GS 2
#define AZ_ls 3
#define AZ_dom_decomp 4
#define AZ_row_sum 5
#define AZ_sym_row_sum 6
#define AZ_ilut 7
#define AZ_ilu 8
#define AZ_r0 0
#define AZ_rhs 1
#define AZ_noscaled 2
#define AZ_warnings 1
#define AZ_last 2
#define AZ_all 3
#define AZ_calc 0
#define AZ_reuse 1
#define AZ_classic 0
#define AZ_modified 1
#define AZ_resid 0
#define AZ_rand 1
#define AZ_linear 0
#define AZ_file 1
#define AZ_box 2
#define AZ_MIN(a,b) (((a) < (b)) ? (a) : (b))
#define AZ_MAX(a,b) (((a) > (b)) ? (a) : (b))
#ifdef __cplusplus
extern "C" {
#endif
void AZ_defaults(int *options, double *params);
#ifdef __cplusplus
}
#endif
#endif
