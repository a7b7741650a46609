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

// an FP64 value in arithmetic T, and back (conversions between FP64 and FP32 by the hardware: the same
// conversions done with integer operations on the two 32-bit halves measured slower in the FP32 products)
template <class T>
__host__ __device__ __forceinline__ T to_arith(double x)
{
  return (T)x;
}
__host__ __device__ __forceinline__ double to_f64(float x) { return (double)x; }
__host__ __device__ __forceinline__ double to_f64(double x) { return x; }

constexpr int kMaxC = TGPU_MAXC;
// words of a handle's reduction buffer; the last one counts the blocks of a norm or multi-dot product that have
// finished (zero between launches)
constexpr long kPartialWords = 1024L * 1024L;
constexpr int kMaxRb = 10;            // 4 + 2*3 weighted densities
constexpr int kSentBulk = -1, kSentWall = -2, kSentBulkHi = -3, kSentBad = -9;   // kSentBulk: the low side's bulk
constexpr int kReflBit = 1 << 30;     // flag bit in a per-dimension map entry

// Geometry constants visible to every kernel (one problem per launch).
struct DevGeom {
  int ndim, nx[3], h[3], P[3];
  long N, NP, pstride[3];
  int ncomp, nrb, nunk, first_rho, first_rb, first_mf;
  int functional, attraction, single_size, hard_surf, nlists;
  int jac_exact;                       // 1: Hessian of the energy density; 0: the reference's tables
  int interface;                       // 2: phase interface (EL rows take betamu_if)
  double betamu_if[kMaxC];
  long pin_node;                       // first component's density held at pin_value there (-1: none)
  double pin_value;
  const signed char *rowkind;          // per node: 0, or the Euler-Lagrange row of a BULK_ZONE (1) / PB_ZONE (2)
                                       // node (nullptr: none)
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
// 3-D real-to-complex FFTs for the stencil sums (fft.cu): real box [F2][F1][F0] with F_d = n_d on periodic
// dimensions (no padding) and F_d >= the padded extent elsewhere, half spectrum [F2][F1][F0/2 + 1]; each axis's
// length is a product of radices 2, 3, 4, 5
struct FftAxis {
  int n = 1, nst = 0;
  int rad[16] = {0};
  double2 *d_tw = nullptr;   // exp(-2 pi i k / n), k < n
  float2 *d_tw32 = nullptr;  // the same rounded to FP32 (the FP32 transforms)
};
struct FftPlan {
  int F[3] = {1, 1, 1};
  int Fh = 1;                // F[0] / 2 + 1
  int P[3] = {1, 1, 1}, nx[3] = {1, 1, 1}, h[3] = {0, 0, 0};
  int off[3] = {0, 0, 0};    // first padded index the box holds along d (h on an unpadded periodic dimension)
  int ext[3] = {1, 1, 1};    // padded extent the box holds (zeros beyond it)
  long NR = 0;               // real box points
  long NH = 0;               // half-spectrum points
  FftAxis ax[3];
};
bool fft_make_plan(FftPlan &p, const int P[3], const int nx[3], const int h[3], const int periodic[3], int ndim,
                   cudaStream_t s);
// One channel of a field read through the per-dimension boundary maps (the values a padded box would hold:
// bulk values at bulk sentinels, 0 inside walls, mirrored nodes with the sign flips of signmask, 0 at the
// zero-density nodes of component zc >= 0)
struct MapSrc {
  const double *src = nullptr;    // the channel [N]
  const float *src32 = nullptr;   // the channel in FP32 (read instead of src when set; FP32 transforms only)
  int ndim = 3, nx[3] = {1, 1, 1};
  const int *map[3] = {nullptr, nullptr, nullptr};
  double bulk_lo = 0.0, bulk_hi = 0.0;
  int signmask = 0, zc = -1;
  const signed char *zero = nullptr;
  long N = 0;
};
void rfft_forward_mapped(const MapSrc &m, double2 *spec, const FftPlan &p, cudaStream_t s);
void rfft_forward_mapped(const MapSrc &m, float2 *spec, const FftPlan &p, cudaStream_t s);
void fft_free_plan(FftPlan &p);
// half spectrum of a padded channel [P2][P1][P0]
void rfft_forward(const double *pad, double2 *spec, const FftPlan &p, cudaStream_t s);
void rfft_forward(const float *pad, float2 *spec, const FftPlan &p, cudaStream_t s);
// half spectrum of a real box [F2][F1][F0]
void rfft_forward_box(const double *box, double2 *spec, const FftPlan &p, cudaStream_t s);
// out[node] (+)= scale * inverse transform of sum_t a_t k_t (nterms <= fft_max_terms() spectral products, formed by
// the first inverse pass) at the interior nodes; work holds the half spectrum in between
void rfft_inverse_products(const double2 *const *a, const double2 *const *k, int nterms, double2 *work,
                           const FftPlan &p, double scale, double *out, bool accumulate, cudaStream_t s);
void rfft_inverse_products(const float2 *const *a, const float2 *const *k, int nterms, float2 *work,
                           const FftPlan &p, double scale, double *out, bool accumulate, cudaStream_t s);
void rfft_inverse_products(const float2 *const *a, const float2 *const *k, int nterms, float2 *work,
                           const FftPlan &p, double scale, float *out, bool accumulate, cudaStream_t s);
int fft_max_terms();
// several FP32 transforms of one plan per launch (blockIdx.y selects the transform): forward transforms of nb mapped
// channels into spec[b]; inverse transforms out[b] (+)= scale * inverse of a * k[b] (work[b] the half spectra)
int fft_max_batch();
void rfft_forward_mapped_batch(const MapSrc *m, int nb, float2 *const *spec, const FftPlan &p, cudaStream_t s);
void rfft_forward_mapped_batch(const MapSrc *m, int nb, double2 *const *spec, const FftPlan &p, cudaStream_t s);
void rfft_inverse_batch(const float2 *a, const float2 *const *k, int nb, float2 *const *work, const FftPlan &p,
                        double scale, double *const *out, bool accumulate, cudaStream_t s);
void rfft_inverse_batch(const float2 *a, const float2 *const *k, int nb, float2 *const *work, const FftPlan &p,
                        double scale, float *const *out, bool accumulate, cudaStream_t s);
void rfft_inverse_batch(const double2 *a, const double2 *const *k, int nb, double2 *const *work, const FftPlan &p,
                        double scale, double *const *out, bool accumulate, cudaStream_t s);
// per-launch CUDA-event timing of the FP32 y/z FFT passes (off unless enabled; collect reads and resets)
void pass_timer_enable(bool on);
void pass_timer_collect(long *launches, double *ms_total, double *bytes_total, long *fields_total);
// one y (d = 1) or z (d = 2) pass over a half spectrum, in place (benchmark hook)
void fft_pass(double2 *spec, const FftPlan &p, int d, bool inverse, cudaStream_t s);
void fft_pass(float2 *spec, const FftPlan &p, int d, bool inverse, cudaStream_t s);
void launch_to_float2(const double2 *in, float2 *out, long n, cudaStream_t s);
// real box <- the correlation kernel of coefficient q of a stencil: coef[k * ncoef + q] added at (-offset_k) mod F
void launch_fft_kernel_box(const short *off3, const double *coef, int L, int ncoef, int q, double *box,
                           const FftPlan &p, cudaStream_t s);

// Averaged rows of coarsened nodes and the prolongation onto them (coarsen.cu)
constexpr int kMaxZone = 5;
struct CoarseRows {
  int ncoarse = 0;
  int *d_node = nullptr;                  // [ncoarse] node index of each coarsened node
  int *d_rptr = nullptr;                  // row terms: [ncoarse + 1]
  long *d_rcol = nullptr;                 // node index, or -1 / -3 (bulk beyond the low / high IN_BULK boundary)
  double *d_ra = nullptr;                 // weights a_k > 0 of fac (x_c - sum_k a_k x_k)
  int *d_pptr = nullptr;                  // prolongation x_c = sum_e p_e x_col: [ncoarse + 1]
  long *d_pcol = nullptr;
  double *d_pw = nullptr;
  signed char *d_kind = nullptr;          // [ncoarse] 1: a 1-D boundary row x_c - x_line (fac 1 on every unknown)
};

struct ObjConst {
  double betamu[kMaxC];
  double bulk[kMaxC];
  double phi_b;
};

// The four hard-sphere functionals (Type_func) share Phi_1 = -n0 ln(1-n3) and
// Phi_2 = (n1 n2 - V1.V2)/(1-n3); the third term is Phi_3 = g(n2, V2) f(n3) with
//   g = n2^3 - 3 n2 V2.V2                         FMT1, FMT3 (Rosenfeld's vector form)
//   g = alpha^3, alpha = n2 - V2.V2/n2            FMT2, FMT4 (zero-dimensional crossover)
//   f = 1 / (24 pi (1-n3)^2)                      FMT1, FMT2
//   f = (n3 + (1-n3)^2 ln(1-n3)) / (36 pi n3^2 (1-n3)^2)   FMT3, FMT4 (White-Bear)
// (FMT{1,2,3,4}_energy_density, src/dft_physics_FMT{1,2,3,4}.c).  The White-Bear
// functionals are cut where n3 <= 1e-10: there the reference sets dPhi/dn2,
// dPhi/dn3, dPhi/dV2 and all second derivatives to zero.
inline __host__ __device__ bool fmt_alpha_form(int functional) { return functional == TGPU_FMT2 || functional == TGPU_FMT4; }
inline __host__ __device__ bool fmt_white_bear(int functional) { return functional == TGPU_FMT3 || functional == TGPU_FMT4; }

// g and its derivatives: gv and g2v multiply V2_d; the V2-V2 block is
// gvv delta_de + gvv_out V2_d V2_e.
struct FmtG { double g, g2, gv, g22, g2v, gvv, gvv_out; };
// f and its first two n3 derivatives
struct FmtF { double f, f1, f2; };

// g at (n2, Q = V2.V2).  The alpha form takes alpha = n2, gamma = V2/n2 = 0 where
// n2 <= 1e-15, as FMT2_1stderiv does (src/dft_physics_FMT2.c:80-91).
inline __host__ __device__ FmtG fmt_g(double n2, double Q, int functional)
{
  FmtG r;
  if (!fmt_alpha_form(functional)) {
    r.g = n2 * n2 * n2 - 3.0 * n2 * Q;
    r.g2 = 3.0 * n2 * n2 - 3.0 * Q;
    r.gv = -6.0 * n2;
    r.g22 = 6.0 * n2;
    r.g2v = -6.0;
    r.gvv = -6.0 * n2;
    r.gvv_out = 0.0;
  } else if (n2 > 1.e-15) {
    const double al = n2 - Q / n2, be = 1.0 + Q / (n2 * n2);
    r.g = al * al * al;
    r.g2 = 3.0 * al * al * be;
    r.gv = -6.0 * al * al / n2;
    r.g22 = 6.0 * al * be * be - 6.0 * al * al * Q / (n2 * n2 * n2);
    r.g2v = -12.0 * al * be / n2 + 6.0 * al * al / (n2 * n2);
    r.gvv = -6.0 * al * al / n2;
    r.gvv_out = 24.0 * al / (n2 * n2);
  } else {
    r.g = n2 * n2 * n2;
    r.g2 = 3.0 * n2 * n2;
    r.gv = 0.0;
    r.g22 = 6.0 * n2;
    r.g2v = 0.0;
    r.gvv = -6.0 * n2;
    r.gvv_out = 0.0;
  }
  return r;
}

// f at n3 (White-Bear: only called where n3 > 1e-10)
inline __host__ __device__ FmtF fmt_f(double n3, int functional)
{
  const double pi = 3.141592653589793238462643383279502884197;
  const double one = 1.0 - n3, a = 1.0 / one, a2 = a * a, a3 = a2 * a, a4 = a3 * a;
  FmtF r;
  if (!fmt_white_bear(functional)) {
    r.f = a2 / (24.0 * pi);
    r.f1 = a3 / (12.0 * pi);
    r.f2 = a4 / (4.0 * pi);
  } else {
    const double t = n3, t2 = t * t, t3 = t2 * t, t4 = t3 * t;
    const double lg = log(one);
    const double F = t + one * one * lg, F1 = t - 2.0 * one * lg, F2 = 3.0 + 2.0 * lg;
    const double G = a2 / t2, G1 = 2.0 * (-a2 / t3 + a3 / t2), G2 = 6.0 * a2 / t4 - 8.0 * a3 / t3 + 6.0 * a4 / t2;
    r.f = F * G / (36.0 * pi);
    r.f1 = (F1 * G + F * G1) / (36.0 * pi);
    r.f2 = (F2 * G + 2.0 * F1 * G1 + F * G2) / (36.0 * pi);
  }
  return r;
}

// FMT free-energy density Phi(n), n in the order n0 n1 n2 n3 V1[d] V2[d]; zero
// unless n3 < 1, n2 > 0 and n3 > 1e-10 (phispt_switch, src/dft_switch_FMT.c:41-65).
__host__ __device__ inline double fmt_phi(const double *n, int ndim, int functional)
{
  if (!(n[3] < 1.0 && n[2] > 0.0 && n[3] > 1.e-10)) return 0.0;
  double dot12 = 0.0, dot22 = 0.0;
  for (int d = 0; d < ndim; d++) {
    dot12 += n[4 + d] * n[4 + ndim + d];
    dot22 += n[4 + ndim + d] * n[4 + ndim + d];
  }
  const double one = 1.0 - n[3];
  return -n[0] * log(one) + (n[1] * n[2] - dot12) / one + fmt_g(n[2], dot22, functional).g * fmt_f(n[3], functional).f;
}

// dPhi/dn for the four functionals (FMT{1,2,3,4}_1stderiv, src/dft_physics_FMT{1,2,3,4}.c),
// Phi_3 = g f as in tgpu_internal.h, with the White-Bear cut where n3 <= 1e-10.
__host__ __device__ inline void fmt_dphi_at(const double *n, double *dphi, int nd, int functional)
{
  double dot22 = 0.0, dot12 = 0.0;
  for (int d = 0; d < nd; d++) {
    dot22 += n[4 + nd + d] * n[4 + nd + d];
    dot12 += n[4 + d] * n[4 + nd + d];
  }
  const double a = 1.0 / (1.0 - n[3]), a2 = a * a;
  dphi[0] = log(a);
  dphi[1] = n[2] * a;
  for (int d = 0; d < nd; d++) dphi[4 + d] = -n[4 + nd + d] * a;
  if (fmt_white_bear(functional) && !(n[3] > 1.e-10)) {
    dphi[2] = 0.0;
    dphi[3] = 0.0;
    for (int d = 0; d < nd; d++) dphi[4 + nd + d] = 0.0;
    return;
  }
  const FmtG g = fmt_g(n[2], dot22, functional);
  const FmtF f = fmt_f(n[3], functional);
  dphi[2] = n[1] * a + g.g2 * f.f;
  dphi[3] = n[0] * a + (n[1] * n[2] - dot12) * a2 + g.g * f.f1;
  for (int d = 0; d < nd; d++) dphi[4 + nd + d] = -n[4 + d] * a + g.gv * f.f * n[4 + nd + d];
}

// z = M y for the per-node matrix M of FMT second derivatives (n ordering); with
// transpose, z = M^T y.  With exact, M is the Hessian of Phi (symmetric).
// Otherwise M reproduces the reference's per-stencil-point tables
// d2phi_drb2_delta_rb / _theta_rb as c(offset)^T M and M row n3: the Hessian
// except for FMT2's V2-V2 block (gamma_d gamma_e replaced by |gamma|^2 delta_de,
// src/dft_physics_FMT2.c:182-183) and FMT4's n2-row V2 entries (coefficient
// -6 (fac^2 - 4 V2.V2 fac / n2) f for the Hessian's -6 fac (1 + 3 V2.V2/n2^2) f,
// src/dft_physics_FMT4.c:179, fac = 1 - V2.V2/n2^2).
// The state-dependent scalars of that matrix at one node (all zero where the White-Bear cut applies, which
// makes z = 0); split from the product so that the products of one Newton state can reuse them.
template <class T>
struct HessCoefT {
  T a, a2, h13, h22, h23, h33, ff, gvf1, g2vr_f, g2vc_f, gvv, gvv_out;
};
using HessCoef = HessCoefT<double>;
constexpr int kHessCoef = 12;

__host__ __device__ inline HessCoef fmt_hess_coef_at(const double *n, int nd, int fn, bool exact)
{
  HessCoef c;
  if (fmt_white_bear(fn) && !(n[3] > 1.e-10)) {
    c.a = c.a2 = c.h13 = c.h22 = c.h23 = c.h33 = c.ff = c.gvf1 = c.g2vr_f = c.g2vc_f = c.gvv = c.gvv_out = 0.0;
    return c;
  }
  double Q = 0.0, Pd = 0.0;
  for (int d = 0; d < nd; d++) {
    Q += n[4 + nd + d] * n[4 + nd + d];
    Pd += n[4 + d] * n[4 + nd + d];
  }
  const double a = 1.0 / (1.0 - n[3]), a2 = a * a, a3 = a2 * a;
  const FmtG g = fmt_g(n[2], Q, fn);
  const FmtF f = fmt_f(n[3], fn);
  double gvv = g.gvv, gvv_out = g.gvv_out;
  double g2v_row = g.g2v, g2v_col = g.g2v;   // M[n2][V2d] / V2d and M[V2d][n2] / V2d
  if (!exact && fmt_alpha_form(fn) && n[2] > 1.e-15) {
    if (fn == TGPU_FMT2) {
      const double al = n[2] - Q / n[2];
      gvv = -6.0 * al * al / n[2] + 24.0 * al * Q / (n[2] * n[2]);
      gvv_out = 0.0;
    } else {
      const double fac = 1.0 - Q / (n[2] * n[2]);
      g2v_row = -6.0 * (fac * fac - 4.0 * Q * fac / n[2]);
    }
  }
  c.a = a;
  c.a2 = a2;
  c.h13 = n[2] * a2;
  c.h22 = g.g22 * f.f;
  c.h23 = n[1] * a2 + g.g2 * f.f1;
  c.h33 = n[0] * a2 + 2.0 * (n[1] * n[2] - Pd) * a3 + g.g * f.f2;
  c.ff = f.f;
  c.gvf1 = g.gv * f.f1;
  c.g2vr_f = g2v_row * f.f;
  c.g2vc_f = g2v_col * f.f;
  c.gvv = gvv;
  c.gvv_out = gvv_out;
  return c;
}

// z = M y from the node's scalars and its vector densities (n ordering); transpose swaps the n2-V2 entries
// T = double, or float for the products of FP32 arithmetic (coefficients of the state rounded once)
template <class T>
__host__ __device__ inline void fmt_hess_apply_coef(const HessCoefT<T> &c, const T *n, const T *y, T *z, int nd,
                                                    bool transpose)
{
  const T g2v_row = transpose ? c.g2vc_f : c.g2vr_f, g2v_col = transpose ? c.g2vr_f : c.g2vc_f;
  T Vy = 0;
  for (int d = 0; d < nd; d++) Vy += n[4 + nd + d] * y[4 + nd + d];
  const T a = c.a, a2 = c.a2;
  T s2 = 0, s3 = 0;
  for (int d = 0; d < nd; d++) {
    const T V1 = n[4 + d], V2 = n[4 + nd + d];
    const T yV1 = y[4 + d], yV2 = y[4 + nd + d];
    const T h3v2 = -V1 * a2 + c.gvf1 * V2;    // M[n3][V2d] = M[V2d][n3]
    s2 += g2v_row * V2 * yV2;
    s3 += -V2 * a2 * yV1 + h3v2 * yV2;
    z[4 + d] = -V2 * a2 * y[3] - a * yV2;
    z[4 + nd + d] = g2v_col * V2 * y[2] + h3v2 * y[3] - a * yV1 + c.ff * (c.gvv * yV2 + c.gvv_out * V2 * Vy);
  }
  z[0] = a * y[3];
  z[1] = a * y[2] + c.h13 * y[3];
  z[2] = a * y[1] + c.h22 * y[2] + c.h23 * y[3] + s2;
  z[3] = a * y[0] + c.h13 * y[1] + c.h23 * y[2] + c.h33 * y[3] + s3;
}

__host__ __device__ inline void fmt_hess_apply_at(const double *n, const double *y, double *z, int nd, int fn,
                                                  bool exact, bool transpose)
{
  fmt_hess_apply_coef(fmt_hess_coef_at(n, nd, fn, exact), n, y, z, nd, transpose);
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
  long spin = 0;                  // limit of the pipeline's waits (0: the kernel's default)
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
    int ncoef = 1, wstride = 0;         // coefficients per stencil point, stored wstride apart
    bool ff_ok = false;                 // the float-float slab fits in shared memory
    bool mc_ok = false;                 // the multi-channel slab fits in shared memory
  } lines_fwd, lines_tr;
  // float-float single-coefficient tables of a multi-channel stencil (3-D delta, one size): per forward
  // output channel and per transpose input channel, for the accurate fills
  std::vector<Lines> ff_fwd, ff_tr;
  // FFT spectra of the correlation kernels (FP64 fills by FFT): per forward output, per transpose input;
  // FP32 copies of the forward ones for the FP32 sums (products, FP32 fills)
  std::vector<double2 *> spec_fwd, spec_tr;
  std::vector<float2 *> spec_fwd32, spec_tr32;
  int fft32_fwd = 0, fft32_tr = 0;      // short stencils: FP32 FFT (1) or slab (-1) sums, 0 undecided
  float t32[2][2] = {{0.f, 0.f}, {0.f, 0.f}};  // [forward, transposed][direct, FFT] ms of the timing that decided
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
size_t conv_slab_mc_smem(int nin, int ncoef, int pitch, int max_rows, int max_lines, int max_w);
// false when (nin, nout) has no multi-channel slab kernel (1x4 and 4x1 exist: 3-D delta sums, one particle size)
bool launch_conv_slab_mc(const float *in, long cstride, long in_total, int nin, const int4 *planes, int nplanes,
                         const int4 *lines, const float *lw, int wstride, double *const *out, int nout, int pitch,
                         int ncols, int max_rows, int max_lines, int max_w, int nx, int ny, int nz, cudaStream_t s);
void launch_split_hilo(const double *in, long n, float *hi, float *lo, cudaStream_t s);
void launch_conv_slab_ff(const float *in_hi, const float *in_lo, long in_total, const int4 *planes, int nplanes,
                         const int4 *lines, const float *lw, const float *lw_lo, double *out, int pitch, int ncols,
                         int max_rows, int max_lines, int max_w, int nx, int ny, int nz, cudaStream_t s);
constexpr int kSlabTileX = 128, kSlabTileY = 16;
// domain flags of a fill (launch_fmt_local / launch_assemble with a non-null flag word)
constexpr unsigned kDomainN3 = 1u, kDomainRho = 2u;
void launch_fmt_local(const double *x, double *chan, cudaStream_t s, unsigned *domain = nullptr);
void launch_assemble(const double *x, const double *vext, const signed char *zero, const double *conv,
                     const double *tr, double *R, cudaStream_t s, unsigned *domain = nullptr);
// coef: the state's Hessian scalars ([kHessCoef][N], launch_hess_coef) or null to evaluate them in place
void launch_hess_coef(const double *x, double *coef, cudaStream_t s, float *coef32 = nullptr);
// FP32 storage variants of the FP32 Schur product: the state's Hessian scalars and weighted densities as FP32 rows
// [kHessCoef + nrb][N]; the local step and the combination on FP32 sums, channels and transposed sums
void launch_hess_coef32(const double *x, float *coef, cudaStream_t s);
void launch_schur_local32(int ndim, const float *conv, const float *coef, float *chan, float *ymf, cudaStream_t s);
void launch_rhs_local32(int ndim, const double *b, const float *coef, float *chan, float *ymf, cudaStream_t s);
void launch_rhs_combine32(const signed char *kind, const double *b, const float *tr, const float *ymf, double *b2s,
                          cudaStream_t s);
void launch_row_info32(const double *x, const double *vext, const signed char *zero, double *inv, signed char *kind,
                       cudaStream_t s);
void launch_schur_combine32(const double *inv, const signed char *kind, const double *v2, const float *tr,
                            const float *ymf, double *y2, cudaStream_t s);
void launch_schur_local(const double *x, const double *conv, double *chan, double *ymf, const double *coef,
                        cudaStream_t s, bool f32 = false);
// f32: the per-node Hessian in FP32 arithmetic (FP32 products)
void launch_jv_local(const double *x, const double *v, double *chan, const double *coef, cudaStream_t s,
                     bool f32 = false);
void launch_schur_combine(const double *x, const double *vext, const signed char *zero, const double *v2,
                          const double *tr, const double *ymf, double *y2, cudaStream_t s);
void launch_jv_combine(const double *x, const double *vext, const signed char *zero, const double *v,
                       const double *conv, const double *tr, double *out, cudaStream_t s);
void launch_hw_correct(const double *field, long fcs, int ffirst, const DevStencil *theta, const DevStencil *delta,
                       const DevStencil *uatt, int ncomp, bool do_fmt, bool do_mf, const int *targets, int ntargets,
                       const signed char *zero, const int *bnodes, const short *fmask, double *conv, cudaStream_t s);
void launch_reflect_fold(const double *in, long cstride, int nin, const short *off, const double *coef, int L,
                         double *const *outs, const int *signmask, int nout, cudaStream_t s);
void launch_hw_correct_t(const double *w, const double *mfw, const DevStencil *theta, const DevStencil *delta,
                         const DevStencil *uatt, int ncomp, bool do_fmt, bool do_mf, const int *targets, int ntargets,
                         const signed char *zero, const int *bnodes, const short *fmask, double *out, cudaStream_t s);
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
// coarsen.cu: dst[r][i] = src[r][i] where zone[i] == z; buf[r][i] = 0 where zone[i] != z
void launch_zone_merge(const double *src, double *dst, int nrows, long N, const int *zone, int z, cudaStream_t s);
void launch_zone_mask(double *buf, int nrows, long N, const int *zone, int z, cudaStream_t s);
// averaged rows at coarsened nodes (bulk: per-unknown value at -1 columns, or null for a linear product),
// their transpose (accumulated into out), the prolongation of rows row0.. and zeroing of coarsened nodes
void launch_coarse_rows(const double *in, double *out, int nunk, int first_rho, int ncomp, long N,
                        const CoarseRows &cr, const double *bulk, cudaStream_t s);
void launch_coarse_rows_t(const double *w, double *out, int nunk, int first_rho, int ncomp, long N,
                          const CoarseRows &cr, cudaStream_t s);
void launch_prolong(double *vec, int row0, int nrows, int nunk, long N, const CoarseRows &cr, const double *bulk,
                    cudaStream_t s);
void launch_prolong_t(double *vec, int row0, int nrows, long N, const CoarseRows &cr, cudaStream_t s);
void launch_zero_nodes(double *vec, int nrows, long N, const CoarseRows &cr, cudaStream_t s);
void launch_mask_rows(double *out, const double *w, const double *vext, const signed char *zero, int first, int nrows,
                      int mode, cudaStream_t s);
void launch_delta_maxabs(const double *a, const double *ref, long n, double *out, double *partial, int nblocks,
                         double *result, cudaStream_t s);
void launch_check_finite(const double *x, long n, double *partial, int nblocks, double *result, cudaStream_t s);

int reduce_blocks(long n);

// the n-point Gauss-Legendre rule mapped to [0,1] (nodes ascending, weights summing to 1; stencils.cu)
void gauss_rule01(int n, double *x, double *w);

// the text tgpu_last_error() returns (api.cu), for entry points outside api.cu
void set_last_error(const std::string &text);

}  // namespace tgpu
