// Internal declarations of the GB300 nonlocal-density path.
//
// Data layout in HBM (all SoA, node = ix + nx*(iy + ny*iz)):
//   - state x, residual R, Krylov vectors: double [unknown][node]
//   - padded channels: the convolution inputs are copied once per pass into a
//     box padded by the largest stencil reach h[d] in every dimension; the
//     copy resolves the reference's boundary rules (src/dft_mesh_lib.c:203-297:
//     bulk and in-wall sentinels, periodic wrap, mirror with vector-sign flip)
//     so the stencil sums that follow are branch-free loads at
//     (padded centre + precomputed linear offset).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>

#include <string>
#include <vector>

#include "../../include/tramonto_gpu.h"

namespace tgpu {

constexpr int kMaxC = TGPU_MAXC;
constexpr int kMaxRb = 10;            // 4 + 2*3 weighted densities
constexpr int kSentBulk = -1, kSentWall = -2, kSentBad = -9;
constexpr int kReflBit = 1 << 30;     // flag bit in a per-dimension map entry

// Geometry constants visible to every kernel (one problem per launch).
struct DevGeom {
  int ndim, nx[3], h[3], P[3];
  long N, NP, pstride[3];
  int ncomp, nrb, nunk, first_rho, first_rb, first_mf;
  int functional, attraction, single_size, hard_surf, nlists;
  double esize[3];
  double rho_b[kMaxC], betamu_hs_ex[kMaxC], betamu_att[kMaxC];
  double inv_rad[kMaxC], inv_4pir[kMaxC], inv_4pirsq[kMaxC], fac[kMaxC];
  double dphi_bulk[4], vext_max;
  const int *map[3];                   // per-dimension padded -> source maps
};

constexpr double kDensityMin = 1.e-20;   // integrands vanish at or below this density (DENSITY_MIN)

// Constants of the free-energy objective: per component the chemical potential
// betamu and the bulk integrand rho_b(ln rho_b - 1) - rho_b betamu [+ rho_b betamu_att / 2],
// and the hard-sphere energy density of the bulk weighted densities.
struct ObjConst {
  double betamu[kMaxC];
  double bulk[kMaxC];
  double phi_b;
};

// FMT free-energy density Phi(n), n in the order n0 n1 n2 n3 V1[d] V2[d]:
// Rosenfeld (FMT1_energy_density src/dft_physics_FMT1.c:39-57) or White-Bear
// (FMT3_energy_density src/dft_physics_FMT3.c:39-58).  For n3 <= 1e-10 the
// White-Bear third term takes its n3 -> 0 limit, the Rosenfeld form (the
// reference's expression is 0/0 at n3 = 0).
__host__ __device__ inline double fmt_phi(const double *n, int ndim, int functional)
{
  double dot12 = 0.0, dot22 = 0.0;
  for (int d = 0; d < ndim; d++) {
    dot12 += n[4 + d] * n[4 + ndim + d];
    dot22 += n[4 + ndim + d] * n[4 + ndim + d];
  }
  const double one = 1.0 - n[3];
  const double l = log(one);
  const double p1 = -n[0] * l;
  const double p2 = (n[1] * n[2] - dot12) / one;
  const double c3 = n[2] * n[2] * n[2] - 3.0 * n[2] * dot22;
  const double pi = 3.141592653589793238462643383279502884197;
  double p3;
  if (functional == TGPU_FMT3 && n[3] > 1.e-10)
    p3 = c3 * (n[3] + one * one * l) / (36.0 * pi * n[3] * n[3] * one * one);
  else
    p3 = c3 / (24.0 * pi * one * one);
  return p1 + p2 + p3;
}

// Tensor-core form of a large 3-D single-channel stencil sum (wca_tc.cu): tiles of
// kTcN x-outputs by kTcM y-rows; the field slab spans kTcN + 2 kTcXHalo x-inputs.
constexpr int kTcN = 64, kTcM = 128, kTcXHalo = 32, kTcCores = 24, kTcRing = 8;

struct TcTables {                 // per stencil: lines grouped by z offset, Hankel tables
  int4 *d_planes = nullptr;       // {oz, first record, records, lines}
  int4 *d_lines = nullptr;        // record headers (host reference copy)
  void *d_tables = nullptr;       // FP16 [table][high, low][24][8][8]
  int nplanes = 0, nlines = 0;
  double out_mult = 1.0;          // 1 / weight scale
  int split_first[9][9] = {};     // [ns][k]: plane ranges when ns CTAs share an output tile
  // CTAs per tile: the smallest ns (1..8) that fills the SMs' waves to 95%, else the best fill
  int split_for(int tiles, int nsm) const
  {
    int best = 1;
    double best_fill = 0.0;
    for (int ns = 1; ns <= 8 && ns <= nplanes; ns++) {
      const long ctas = (long)tiles * ns;
      const long waves = (ctas + nsm - 1) / nsm;
      const double fill = (double)ctas / (double)(waves * nsm);
      if (fill >= 0.95) return ns;
      if (fill > best_fill + 1e-9) { best_fill = fill; best = ns; }
    }
    return best;
  }
};

struct TcSlab {                   // per problem: the FP16 copy of a padded channel and its TMA map
  CUtensorMap tmap;
  void *d_slab = nullptr;         // FP16 [high, low][Zp][G][Yp][8]
  float *d_scale = nullptr;       // [0] field scale, [1] max |field| (bits)
  int *d_err = nullptr;           // nonzero after a bounded wait ran out
  int G = 0, Yp = 0, Zp = 0, R = 0, hy = 0, hz = 0, nring = 0, nsm = 1;
};

// One stencil table on the device: linear offsets in the padded box and the
// per-point coefficient rows for each output channel.
struct DevStencil {
  int L = 0;
  std::vector<short> off;               // host copy [L][ndim]
  std::vector<double> w, hw;            // host copy
  int *d_loff = nullptr;                // [L] linear offsets in the padded box
  int *d_loff_neg = nullptr;            // [L] the same offsets negated (transposed sums)
  // forward use (weighted densities / mean field of the density field)
  int nout_fwd = 0;
  double *d_coef_fwd = nullptr;         // [L][nout_fwd] FP64
  float *d_coef_fwd32 = nullptr;        // FP32 copy
  // transpose use (Euler-Lagrange sums over dPhi/dn or H v channels)
  int nin_tr = 0;
  double *d_coef_tr = nullptr;          // [L][nin_tr]
  float *d_coef_tr32 = nullptr;
  double *d_coef_adj = nullptr;         // delta only: [L][1+ndim] fac (w, e_d w) for the transposed sums
  TcTables tc;                          // tensor-core form (3-D attraction stencils)
  short *d_off = nullptr;               // [L][3] raw offsets (boundary corrections)
  double *d_w = nullptr, *d_hw = nullptr;
  // z-plane / x-line form for the FP32 single-channel sums (3-D): forward and transpose coefficients
  struct Lines {
    int4 *d_planes = nullptr, *d_lines = nullptr;
    float *d_w = nullptr;
    float *d_w_lo = nullptr;            // FP32 remainder of each weight (float-float sums)
    int nplanes = 0, max_rows = 0, max_lines = 0, max_w = 0, ncols = 0, pitch = 0;
    bool ff_ok = false;                 // the float-float slab fits in shared memory
  } lines_fwd, lines_tr;
};

}  // namespace tgpu

struct tgpu_ctx {
  tgpu_geometry g{};
  tgpu::DevGeom dg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int precision = TGPU_FP64;
  bool finalized = false;
  bool have_state = false;

  // host tables
  std::vector<tgpu::DevStencil> sten[3];   // [type][index]
  std::vector<double> h_vext;
  std::vector<signed char> h_zero;
  std::vector<int> h_bnodes;
  std::vector<short> h_fmask;
  std::vector<int> hw_targets;             // nodes whose stencils touch a hard-wall boundary node

  // device buffers
  int *d_map[3] = {nullptr, nullptr, nullptr};
  double *d_vext = nullptr;
  signed char *d_zero = nullptr;
  int *d_bnodes = nullptr;
  short *d_fmask = nullptr;
  int *d_hw_targets = nullptr;
  double *d_x = nullptr;        // state of the last mode-0 fill [nunk][N]
  double *d_work = nullptr;     // [nunk][N] scratch for host-pointer entry points
  double *d_work2 = nullptr;    // [nunk][N]
  double *d_pad = nullptr;      // padded FP64 channels [nch_max][NP]
  float *d_pad32 = nullptr;     // padded FP32 channels [nch_max][NP]
  double *d_chan = nullptr;     // unpadded channels [nch_max][N]
  double *d_conv = nullptr;     // convolution outputs [nrb + 2*ncomp][N]
  double *d_tr = nullptr;       // transpose-conv output per component [ncomp][N]
  int nch_max = 0;
  // Krylov workspace
  double *d_V = nullptr;        // [kdim+1][n2]
  double *d_partial = nullptr;  // reduction partials
  double *d_red = nullptr;      // reduction results
  double *h_red = nullptr;      // pinned host copy
  int kdim = 0;
  double *d_gw = nullptr, *d_gt = nullptr, *d_gx = nullptr, *d_gb = nullptr;  // [n2] each

  tgpu_stats stats{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace tgpu {

// ---- kernels (kernels.cu) ---------------------------------------------------
void upload_geom(const DevGeom &g, cudaStream_t s);
// Pad nch channels src[ch][N] -> dst[ch][NP]; bulk[ch] replaces the bulk
// sentinel, signmask[ch] selects the dimensions whose reflection flips the
// sign, zcomp[ch] >= 0 masks nodes flagged zero-density for that component.
template <typename T>
void launch_pad(const double *src, T *dst, int nch, const double *bulk, const int *signmask, const int *zcomp,
                const signed char *zero, bool periodic_only, cudaStream_t s);
// out[o][i] (+)= sum_k sum_c coef[k][o][c] * in[c][pad(i) + loff[k]]
template <typename T>
void launch_conv(const T *in, long in_cstride, int nin, const int *loff, const T *coef, int L, double *const *out,
                 int nout, bool accumulate, long N, cudaStream_t s);
void launch_conv_slab(const float *in, long in_total, const int4 *planes, int nplanes, const int4 *lines,
                      const float *lw, double *out, int pitch, int ncols, int max_rows, int max_lines, int max_w,
                      int nx, int ny, int nz, cudaStream_t s);
size_t conv_slab_ff_smem(int pitch, int max_rows, int max_lines, int max_w);
void launch_conv_slab_ff(const double *in, long in_total, const int4 *planes, int nplanes, const int4 *lines,
                         const float *lw, const float *lw_lo, double *out, int pitch, int ncols, int max_rows,
                         int max_lines, int max_w, int nx, int ny, int nz, cudaStream_t s);
constexpr int kSlabTileX = 128, kSlabTileY = 16;
void launch_fmt_local(const double *x, double *chan, cudaStream_t s);
void launch_assemble(const double *x, const double *vext, const signed char *zero, const double *conv,
                     const double *tr, double *R, cudaStream_t s);
void launch_schur_local(const double *x, const double *conv, double *chan, double *ymf, cudaStream_t s);
void launch_jv_local(const double *x, const double *v, double *chan, cudaStream_t s);
void launch_schur_combine(const double *x, const double *vext, const signed char *zero, const double *v2,
                          const double *tr, const double *ymf, double *y2, cudaStream_t s);
void launch_jv_combine(const double *x, const double *vext, const signed char *zero, const double *v,
                       const double *conv, const double *tr, double *out, cudaStream_t s);
void launch_hw_correct(const double *field, long field_cstride, int field_first, const DevStencil *theta,
                       const DevStencil *delta, const DevStencil *uatt, const int *targets, int ntargets,
                       const signed char *zero, const int *bnodes, const short *fmask, double *conv,
                       cudaStream_t s);
// Krylov helpers
void launch_multidot(const double *V, long ldv, int nvec, const double *w, long n, double *partial, int nblocks,
                     double *result, cudaStream_t s);
void launch_multiaxpy(double *w, const double *V, long ldv, int nvec, const double *coef, long n, cudaStream_t s);
void launch_scale(double *y, const double *x, double a, long n, cudaStream_t s);
void launch_axpby(double *y, double a, const double *x, double b, long n, cudaStream_t s);
void launch_precond(const double *x, const double *vext, const signed char *zero, const double *in, double *out,
                    cudaStream_t s);
void launch_newton_frac(const double *x, const double *dx, double floor_frac, double *partial, int nblocks,
                        double *result, cudaStream_t s);
void launch_newton_update(double *x, const double *dx, double frac, double rel, double abs, double *partial,
                          int nblocks, double *result, cudaStream_t s);
void launch_norm2(const double *x, long n, double *partial, int nblocks, double *result, cudaStream_t s);
// J^T w local step: A22, A11^T (with B^T), the MF coupling and H g for the rb columns
void launch_jtv_local(const double *x, const double *vext, const signed char *zero, const double *w,
                      const double *gel, int gstride_ic, int v2_first, double *out, cudaStream_t s);
void launch_objectives(const double *x, const double *vext, const double *satt, const double *wf, const double *wb,
                       const ObjConst &oc, int ncomp, double *partial, int nblocks, double *result, cudaStream_t s);
void launch_objective_grad(const double *x, const double *vext, const double *satt, const double *wf,
                           const double *wb, const ObjConst &oc, int kind, int icomp, double *gx, double *gv,
                           double *chan, cudaStream_t s);
void launch_vext_sens(const double *lam, const double *gv, const double *vext, const signed char *zero, double *out,
                      cudaStream_t s);
bool tc_build_tables(const std::vector<short> &off, const std::vector<double> &w, int L, int hy, TcTables &t,
                     cudaStream_t s);
void tc_free_tables(TcTables &t);
bool tc_make_slab(TcSlab &sl, const DevGeom &g, std::string &why);
void tc_free_slab(TcSlab &sl);
void launch_sten_tc(const float *pad_channel, const DevGeom &g, const TcSlab &sl, const TcTables &t, double *out,
                    bool accumulate, cudaStream_t s);
void launch_adj_rb_channels(const double *w, double *chan, cudaStream_t s);
void launch_a11inv_t(const double *u, double *y, cudaStream_t s);
void launch_mask_rows(double *out, const double *w, const double *vext, const signed char *zero, int first, int nrows,
                      int mode, cudaStream_t s);
void launch_delta_maxabs(const double *a, const double *ref, long n, double *out, double *partial, int nblocks,
                         double *result, cudaStream_t s);
void launch_check_finite(const double *x, long n, double *partial, int nblocks, double *result, cudaStream_t s);

int reduce_blocks(long n);

}  // namespace tgpu
