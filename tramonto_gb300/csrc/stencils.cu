// Stencil tables (set-up, run once per problem), on the host and on the GPU.
//
// Builds the integration stencils the nonlocal sums use, with the
// construction of calc_stencils (src/dft_stencil.c:40-287): every lattice
// element of the stencil's bounding box is classified as outside, inside or
// straddling the stencil radius (calc_in_out_on :764-813); inside elements are
// integrated with tensor Gauss-Legendre rules, straddling ones with a
// midpoint rule on a finer sub-grid; each quadrature point's weight goes to
// the element's corner nodes by trilinear interpolation
// (distribute_weight_to_nodes :498-525) while the per-corner parts are kept
// for hard walls (merge_load_stencil :598-650); the table is finally
// renormalised to the analytic volume (renormalize_stencil :685-711).
// Weight functions: delta shell (src/dft_stencil_delta_R.c:34-79), theta ball
// (src/dft_stencil_theta_R.c:34-75) and the mean-field attraction
// (src/dft_stencil_theta_uattr.c:35-158) with the attractive parts of the
// cut-and-shifted pair potentials: Lennard-Jones 12-6 with the cores of
// Type_CoreATT_R / Type_CoreATT_CONST (src/dft_pairPot_LJ12_6.c:96-230),
// Yukawa (src/dft_pairPot_Yukawa.c:96-175), exponential
// (src/dft_pairPot_EXP.c:98-170) and square well (src/dft_pairPot_SW.c:96-145).
//
// The per-element quadrature (elem_weights) is one __host__ __device__ routine.
// The host builder (tgpu_make_stencil) runs it element by element and merges
// corner weights into the table in element order; the device builder
// (tgpu_make_stencil_device) runs one thread per element, then one thread per
// node adds that node's corner weights in the same element order, orders the
// nodes by first touch (the host's insertion order) and renormalises with a
// sequential sum in table order.  This file is compiled without contraction of
// multiply-adds (nvcc -fmad=false, host -ffp-contract=off), so both builders
// perform the same IEEE operations and their tables are bit-identical (the
// Yukawa and exponential weights call exp(), whose last bit may differ between
// the host's and the GPU's libraries: those tables agree to rounding).
//
// Gauss-Legendre nodes are computed here (Newton iteration on the Legendre
// recurrence) rather than taken from tables, so weights agree with the
// reference's to rounding, not bit for bit.
#include <cuda_runtime.h>
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/tramonto_gpu.h"

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr int kMaxRule = 40;

// nodes and weights of the n-point Gauss-Legendre rule mapped to [0,1]
void gauss01(int n, double *x, double *w)
{
  for (int i = 0; i < (n + 1) / 2; i++) {
    double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; it++) {
      double p0 = 1.0, p1 = z;
      for (int k = 2; k <= n; k++) {
        const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    if (n == 1) { z = 0.0; dp = 1.0; }
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= n; k++) {
      const double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n == 1 ? 1.0 : n * (z * p1 - p0) / (z * z - 1.0);
    const double wt = n == 1 ? 2.0 : 2.0 / ((1.0 - z * z) * dp * dp);
    x[i] = (1.0 - z) / 2.0;          // ascending on [0, 1/2]
    x[n - 1 - i] = (1.0 + z) / 2.0;
    w[i] = w[n - 1 - i] = wt / 2.0;
  }
}

// gauss01 for every rule size up to 40: [n][i]
struct GaussTable {
  double x[kMaxRule + 1][kMaxRule];
  double w[kMaxRule + 1][kMaxRule];
};

const GaussTable &gauss_table()
{
  struct Init {
    GaussTable t;
    Init()
    {
      std::memset(&t, 0, sizeof(t));
      for (int n = 1; n <= kMaxRule; n++) gauss01(n, t.x[n], t.w[n]);
    }
  };
  static const Init init;   // thread-safe static initialisation
  return init.t;
}

struct StenSpec {
  int type, ndim;
  double esize[3];
  double R;                          // stencil radius
  double sigma, eps, rcut, rmin;     // mean-field attraction
  int pot, core_r, core_const;       // pair potential, core range and core value (TGPU_PAIR_*, TGPU_CORE_*)
  double rzero, kappa;               // LJ: zero of the cut-shifted potential; Yukawa K sigma / decay length
  int ext[3];                        // elements per half-axis
  int lo[3], n[3];                   // element box: first index and count per dimension
  int nel;                           // corners per element
};

// r where the LJ core ends (uLJ12_6_ATT_CS's r_min for each Type_CoreATT_R)
__host__ __device__ inline double lj_core_r(const StenSpec &p)
{
  if (p.core_r == TGPU_CORE_SIGMA) return p.sigma;
  if (p.core_r == TGPU_CORE_UCSZERO) return p.rzero;
  return p.rmin;   // UMIN, SIGTOUMIN
}

// The attractive part of the cut-and-shifted pair potential (pairPot_ATT_CS_switch): the LJ form is held at
// its core value inside the core (or zero there with CORECONST_ZERO; zero inside sigma for SIGTOUMIN).
__host__ __device__ inline double u_att_cs(double r, const StenSpec &p)
{
  if (p.pot == TGPU_PAIR_YUKAWA_CS) {
    const double a = p.kappa * p.sigma;
    const double cut = exp(-a * (p.rcut / p.sigma - 1.)) / (p.rcut / p.sigma);
    if (r < p.sigma) return p.core_const == TGPU_CORECONST_ZERO ? 0.0 : p.eps * (1.0 - cut);
    if (r <= p.rcut) return p.eps * exp(-a * (r / p.sigma - 1.)) / (r / p.sigma) - p.eps * cut;
    return 0.0;
  }
  if (p.pot == TGPU_PAIR_EXP_CS) {
    const double cut = exp(-(p.rcut - p.sigma) / p.kappa);
    if (r < p.sigma) return p.core_const == TGPU_CORECONST_ZERO ? 0.0 : p.eps * (-1.0 + cut);
    if (r <= p.rcut) return -p.eps * exp(-(r - p.sigma) / p.kappa) + p.eps * cut;
    return 0.0;
  }
  if (p.pot == TGPU_PAIR_SW) {
    if (r < p.sigma) return 0.0;
    if (r <= p.rcut) return -p.eps;
    return 0.0;
  }
  const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2;
  const double rc = 1.0 / p.rcut, rc2 = rc * rc, rc6 = rc2 * rc2 * rc2, rc12 = rc6 * rc6;
  const double rm = lj_core_r(p);
  if ((r < rm && p.core_const == TGPU_CORECONST_ZERO) || (r < p.sigma && p.core_r == TGPU_CORE_SIGTOUMIN)) return 0.0;
  if (r > p.rcut) return 0.0;
  if (r < rm) r = rm;
  const double ri = 1.0 / r, r2 = ri * ri, r6 = r2 * r2 * r2, r12 = r6 * r6;
  return 4.0 * p.eps * s6 * (s6 * (r12 - rc12) - (r6 - rc6));
}

// The attractive part without the cut and shift (pairPot_ATT_noCS_switch)
double u_att_nocs(double r, const StenSpec &p)
{
  if (p.pot == TGPU_PAIR_YUKAWA_CS) {
    if (r < p.sigma) return p.core_const == TGPU_CORECONST_ZERO ? 0.0 : p.eps;
    return p.eps * exp(-p.kappa * p.sigma * (r / p.sigma - 1.)) / (r / p.sigma);
  }
  if (p.pot == TGPU_PAIR_EXP_CS) {
    if (r < p.sigma) return p.core_const == TGPU_CORECONST_ZERO ? 0.0 : -p.eps;
    return -p.eps * exp(-(r - p.sigma) / p.kappa);
  }
  if (p.pot == TGPU_PAIR_SW) return r < p.sigma ? 0.0 : -p.eps;
  const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2;
  const double rm = lj_core_r(p);
  if ((r < rm && p.core_const == TGPU_CORECONST_ZERO) || (r < p.sigma && p.core_r == TGPU_CORE_SIGTOUMIN)) return 0.0;
  if (r < rm) r = rm;
  const double ri = 1.0 / r, r2 = ri * ri, r6 = r2 * r2 * r2, r12 = r6 * r6;
  return 4.0 * p.eps * s6 * (s6 * r12 - r6);
}

// The integral that sets the stencil's magnitude (pairPot_integral_switch)
double u_integral(double r, const StenSpec &p)
{
  if (p.pot == TGPU_PAIR_YUKAWA_CS) {
    const double a = p.kappa * p.sigma, c = a / p.sigma;
    return 4 * kPi * p.eps * p.sigma * std::exp(a) * ((std::exp(-c * r) / (c * c)) * (-c * r - 1.0));
  }
  if (p.pot == TGPU_PAIR_EXP_CS) {
    const double al = p.kappa, a3 = al * al * al;
    return -4.0 * kPi * p.eps * std::exp(-(r - p.sigma) / al) * (-al * r * r + 2 * a3 * (-r / al - 1.));
  }
  if (p.pot == TGPU_PAIR_SW) return -(4.0 / 3.0) * kPi * p.eps * std::pow(r, 3);
  const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2;
  const double ri = 1.0 / r, r3 = ri * ri * ri, r9 = r3 * r3 * r3;
  return 16 * kPi * p.eps * s6 * (-s6 * r9 / 9.0 + r3 / 3.0);
}

// The potential's inner core (pairPot_InnerCore_switch): [0, left) and [left, right) with value eps_core
void inner_core(const StenSpec &p, double *left, double *right, double *eps_core)
{
  *left = 0.0;
  if (p.pot == TGPU_PAIR_LJ12_6_CS) {
    *right = lj_core_r(p);
    if (p.core_r == TGPU_CORE_SIGTOUMIN) *left = p.sigma;
  } else {
    *right = p.sigma;
  }
  *eps_core = (p.pot == TGPU_PAIR_SW || p.core_const == TGPU_CORECONST_ZERO) ? 0.0 : u_att_nocs(*right, p);
}

// StenTheta_uattr_sten_vol (src/dft_stencil_theta_uattr.c:39-87)
double uattr_volume(const StenSpec &p)
{
  double left, right, epsc;
  inner_core(p, &left, &right, &epsc);
  const double rc = p.rcut, rm = right;
  if (std::fabs(epsc) >= 1.e-8) {
    if (std::fabs(left) < p.esize[0])
      return (4.0 / 3.0) * kPi * std::pow(rm, 3.0) * u_att_nocs(rm, p) -
             (4.0 / 3.0) * kPi * std::pow(rc, 3.0) * u_att_nocs(rc, p) + u_integral(rc, p) - u_integral(rm, p);
    return (4.0 / 3.0) * kPi * std::pow(rm, 3.0) * u_att_nocs(rm, p) -
           (4.0 / 3.0) * kPi * std::pow(rc, 3.0) * u_att_nocs(rc, p) -
           (4.0 / 3.0) * kPi * std::pow(left, 3.0) * u_att_nocs(rm, p) +
           (4.0 / 3.0) * kPi * std::pow(left, 3.0) * u_att_nocs(rc, p) + u_integral(rc, p) - u_integral(rm, p);
  }
  if (p.pot == TGPU_PAIR_SW) return u_integral(rc, p) - u_integral(rm, p);
  return (u_integral(rc, p) - (4.0 / 3.0) * kPi * std::pow(rc, 3.0) * u_att_nocs(rc, p)) -
         (u_integral(rm, p) - (4.0 / 3.0) * kPi * std::pow(rm, 3.0) * u_att_nocs(rc, p));
}

double u_lj_cs(double r, double sigma, double eps, double rc)
{
  if (r > rc) return 0.0;
  return 4.0 * eps * ((std::pow(sigma / r, 12) - std::pow(sigma / rc, 12)) - (std::pow(sigma / r, 6) - std::pow(sigma / rc, 6)));
}

__host__ __device__ inline bool is_delta(const StenSpec &s) { return s.type == TGPU_STEN_DELTA; }

__host__ __device__ inline int npt_boundary(const StenSpec &s)
{
  if (s.type == TGPU_STEN_DELTA) return s.ndim == 3 ? 40 : 150;
  if (s.type == TGPU_STEN_THETA) return s.ndim == 3 ? 20 : 40;
  return s.ndim == 3 ? 1 : 20;
}

__host__ __device__ inline int ngauss(const StenSpec &s, double r)
{
  if (s.type == TGPU_STEN_UATT) return 1;
  return r <= 4.000000001 ? 6 : 3;
}

__host__ __device__ inline int ngauss_integrand(const StenSpec &s, double r)
{
  if (s.type != TGPU_STEN_UATT) return 0;
  if (r <= 4.000000001) return 40;
  if (r <= 16.00000001) return 20;
  return 12;
}

__host__ __device__ inline double weight(const StenSpec &s, double rsq, int ngpu, const double *gpu, const double *gwu)
{
  if (s.type == TGPU_STEN_DELTA) {
    if (s.ndim == 1) return 2.0 * kPi * s.R;
    if (s.ndim == 2) return 2.0 / sqrt(1.0 - rsq);
    return 1.0;
  }
  if (s.type == TGPU_STEN_THETA) {
    if (s.ndim == 1) return (1.0 - rsq) * kPi * s.R * s.R;
    if (s.ndim == 2) return sqrt(1.0 - rsq) * 2.0 * s.R;
    return 1.0;
  }
  const double rc = s.rcut;
  double wsum = 0.0;
  const double zmax = sqrt(1 - rsq);
  if (s.ndim == 1) {
    for (int i = 0; i < ngpu; i++) {
      const double z = zmax * gpu[i];
      const double rho = sqrt(rsq + z * z) * rc;
      wsum += gwu[i] * z * u_att_cs(rho, s);
    }
    return 2.0 * kPi * wsum * rc * rc * zmax;
  }
  if (s.ndim == 2) {
    for (int i = 0; i < ngpu; i++) {
      const double z = zmax * gpu[i];
      const double rho = sqrt(rsq + z * z) * rc;
      wsum += gwu[i] * u_att_cs(rho, s);
    }
    return 2.0 * wsum * rc * zmax;
  }
  return u_att_cs(sqrt(rsq) * rc, s);
}

__host__ __device__ inline void distribute(int ndim, double wt, const double *q, double *elw)
{
  if (ndim == 3) {
    elw[0] += wt * (1.0 - q[0]) * (1.0 - q[1]) * (1.0 - q[2]);
    elw[1] += wt * q[0] * (1.0 - q[1]) * (1.0 - q[2]);
    elw[2] += wt * (1.0 - q[0]) * q[1] * (1.0 - q[2]);
    elw[3] += wt * q[0] * q[1] * (1.0 - q[2]);
    elw[4] += wt * (1.0 - q[0]) * (1.0 - q[1]) * q[2];
    elw[5] += wt * q[0] * (1.0 - q[1]) * q[2];
    elw[6] += wt * (1.0 - q[0]) * q[1] * q[2];
    elw[7] += wt * q[0] * q[1] * q[2];
  } else if (ndim == 2) {
    elw[0] += wt * (1.0 - q[0]) * (1.0 - q[1]);
    elw[1] += wt * q[0] * (1.0 - q[1]);
    elw[2] += wt * (1.0 - q[0]) * q[1];
    elw[3] += wt * q[0] * q[1];
  } else {
    elw[0] += wt * (1.0 - q[0]);
    elw[1] += wt * q[0];
  }
}

// 1: outside the radius, -1: inside, 0: straddling
__host__ __device__ inline int in_out_on(const StenSpec &s, const double *xl, const double *xr)
{
  bool in = false, out = false;
  const int nc = 1 << s.ndim;
  for (int c = 0; c < nc; c++) {
    double r2 = 0.0;
    for (int d = 0; d < s.ndim; d++) {
      const double v = (c >> d) & 1 ? xr[d] : xl[d];
      r2 += v * v;
    }
    if (sqrt(r2) > s.R) out = true;
    else in = true;
  }
  if (!in && out) return 1;
  if (in && !out) return -1;
  return 0;
}

__host__ __device__ inline void el_inside(const StenSpec &s, const GaussTable &G, const double *xl, double rc2,
                                          double *elw)
{
  const int ndim = s.ndim;
  const double inv_r2 = 1.0 / (s.R * s.R);
  double vol = 1.0;
  for (int d = 0; d < ndim; d++) vol *= s.esize[d];
  const int ngp = ngauss(s, rc2);
  const int ngpu = ngauss_integrand(s, rc2);
  const double *gp = G.x[ngp], *gw = G.w[ngp];
  const double *gpu = G.x[ngpu], *gwu = G.w[ngpu];
  double pt[3], q[3];
  for (int ig = 0; ig < ngp; ig++) {
    pt[0] = xl[0] + gp[ig] * s.esize[0];
    q[0] = gp[ig];
    if (ndim == 1) {
      const double rsq = pt[0] * pt[0] * inv_r2;
      double wt = weight(s, rsq, ngpu, gpu, gwu);
      wt *= gw[ig] * vol;
      distribute(ndim, wt, q, elw);
      continue;
    }
    for (int jg = 0; jg < ngp; jg++) {
      pt[1] = xl[1] + gp[jg] * s.esize[1];
      q[1] = gp[jg];
      if (ndim == 2) {
        const double rsq = (pt[0] * pt[0] + pt[1] * pt[1]) * inv_r2;
        double wt = weight(s, rsq, ngpu, gpu, gwu);
        wt *= gw[ig] * gw[jg] * vol;
        distribute(ndim, wt, q, elw);
        continue;
      }
      for (int kg = 0; kg < ngp; kg++) {
        pt[2] = xl[2] + gp[kg] * s.esize[2];
        q[2] = gp[kg];
        const double rsq = (pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]) * inv_r2;
        double wt = weight(s, rsq, ngpu, gpu, gwu);
        wt *= gw[ig] * gw[jg] * gw[kg] * vol;
        distribute(ndim, wt, q, elw);
      }
    }
  }
}

__host__ __device__ inline void el_boundary(const StenSpec &s, const GaussTable &G, const double *xl, double rc2,
                                            double *elw)
{
  const int ndim = s.ndim;
  const double inv_r2 = 1.0 / (s.R * s.R);
  double vol = 1.0;
  for (int d = 0; d < ndim; d++) vol *= s.esize[d];
  const int npt = npt_boundary(s);
  const int ngpu = ngauss_integrand(s, rc2);
  const double *gpu = G.x[ngpu], *gwu = G.w[ngpu];
  const double inv = 1.0 / (double)npt;
  double ok = 0.0;
  if (ndim == 3 && is_delta(s)) {
    double t = 0.0;
    for (int d = 0; d < ndim; d++) t += s.esize[d] * s.esize[d];
    ok = 0.5 * inv * sqrt(t);
  }
  double pt[3], q[3];
  for (int ig = 0; ig < npt; ig++) {
    q[0] = ((double)ig + 0.5) * inv;
    pt[0] = xl[0] + q[0] * s.esize[0];
    if (ndim == 1) {
      const double rsq = pt[0] * pt[0] * inv_r2;
      if (rsq <= 1.000001) {
        double wt = weight(s, rsq, ngpu, gpu, gwu);
        if (fabs(rsq - 1.0) <= 1.e-8) wt *= 0.5;
        wt *= inv * vol;
        distribute(ndim, wt, q, elw);
      }
      continue;
    }
    for (int jg = 0; jg < npt; jg++) {
      q[1] = ((double)jg + 0.5) * inv;
      pt[1] = xl[1] + q[1] * s.esize[1];
      if (ndim == 2) {
        const double rsq = (pt[0] * pt[0] + pt[1] * pt[1]) * inv_r2;
        if (rsq <= 1.0000001) {
          double wt = weight(s, rsq, ngpu, gpu, gwu);
          if (fabs(rsq - 1.0) <= 1.e-8) wt *= 0.5;
          wt *= inv * inv * vol;
          distribute(ndim, wt, q, elw);
        }
        continue;
      }
      for (int kg = 0; kg < npt; kg++) {
        q[2] = ((double)kg + 0.5) * inv;
        pt[2] = xl[2] + q[2] * s.esize[2];
        const double rsq = (pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]) * inv_r2;
        if ((rsq <= 1.00000001 && !is_delta(s)) || (is_delta(s) && fabs(rsq - 1.0) < 2 * ok)) {
          double wt = weight(s, rsq, ngpu, gpu, gwu);
          if (fabs(rsq - 1.0) <= 1.e-8 && !is_delta(s)) wt *= 0.5;
          wt *= (inv * inv * inv) * vol;
          distribute(ndim, wt, q, elw);
        }
      }
    }
  }
}

// Corner weights elw[2^ndim] of the element with lower corner ijk (zeros when it is skipped).
__host__ __device__ inline void elem_weights(const StenSpec &s, const GaussTable &G, const int *ijk, double *elw)
{
  for (int c = 0; c < 8; c++) elw[c] = 0.0;
  double xl[3] = {0, 0, 0}, xr[3] = {0, 0, 0}, xm[3];
  for (int d = 0; d < s.ndim; d++) {
    xl[d] = ijk[d] * s.esize[d];
    xr[d] = (ijk[d] + 1) * s.esize[d];
  }
  double rc2 = 0.0;
  for (int d = 0; d < s.ndim; d++) {
    xm[d] = xl[d] + 0.5 * s.esize[d];
    rc2 += xm[d] * xm[d];
  }
  const int flag = in_out_on(s, xl, xr);
  if (flag == 1 || (flag == -1 && s.ndim == 3 && is_delta(s))) return;
  if (flag == -1) el_inside(s, G, xl, rc2, elw);
  else el_boundary(s, G, xl, rc2, elw);
}

// element index <-> lower corner, in the host loop order (x outermost, z innermost)
__host__ __device__ inline long elem_index(const StenSpec &s, const int *ijk)
{
  return ((long)(ijk[0] - s.lo[0]) * s.n[1] + (ijk[1] - s.lo[1])) * s.n[2] + (ijk[2] - s.lo[2]);
}

__host__ __device__ inline void elem_ijk(const StenSpec &s, long e, int *ijk)
{
  ijk[2] = s.lo[2] + (int)(e % s.n[2]);
  e /= s.n[2];
  ijk[1] = s.lo[1] + (int)(e % s.n[1]);
  ijk[0] = s.lo[0] + (int)(e / s.n[1]);
}

StenSpec make_spec(int type, int ndim, const double *esize, double hs_diam, const tgpu_pairpot &pp, double *vol)
{
  StenSpec s;
  std::memset(&s, 0, sizeof(s));
  s.type = type;
  s.ndim = ndim;
  for (int d = 0; d < 3; d++) s.esize[d] = d < ndim ? esize[d] : 0.0;
  if (type == TGPU_STEN_DELTA) {
    s.R = hs_diam / 2.0;
    *vol = kPi * std::pow(hs_diam, 2);
  } else if (type == TGPU_STEN_THETA) {
    s.R = hs_diam / 2.0;
    *vol = kPi * std::pow(hs_diam, 3) / 6.0;
  } else {
    s.R = pp.rcut;
    s.sigma = pp.sigma;
    s.eps = pp.eps_over_kT;
    s.rcut = pp.rcut;
    s.rmin = pp.rmin;
    s.rzero = pp.rzero;
    s.kappa = pp.kappa;
    s.pot = pp.pot;
    s.core_r = pp.core_r;
    s.core_const = pp.core_const;
    *vol = uattr_volume(s);
  }
  s.nel = 1 << ndim;
  for (int d = 0; d < 3; d++) {
    s.ext[d] = d < ndim ? (int)((float)s.R / (float)s.esize[d] + 0.999) : 0;
    s.lo[d] = d < ndim ? -s.ext[d] : 0;
    s.n[d] = d < ndim ? 2 * s.ext[d] : 1;
  }
  return s;
}

struct Table {
  std::vector<short> off;
  std::vector<double> w, hw;
};

// Host builder: elements in loop order, corner weights merged by first touch.
Table build_host(const StenSpec &s, double vol_sten)
{
  const GaussTable &G = gauss_table();
  Table t;
  std::map<long, int> index;
  const int nel = s.nel;
  const long ne = (long)s.n[0] * s.n[1] * s.n[2];
  for (long e = 0; e < ne; e++) {
    int ijk[3];
    elem_ijk(s, e, ijk);
    double elw[8];
    elem_weights(s, G, ijk, elw);
    for (int ln = 0; ln < nel; ln++) {
      if (elw[ln] == 0.0) continue;
      int o[3] = {0, 0, 0};
      for (int d = 0; d < s.ndim; d++) o[d] = ijk[d] + ((ln >> d) & 1);
      long key = 0;
      for (int d = s.ndim - 1; d >= 0; d--) key = key * (2 * s.ext[d] + 1) + (o[d] + s.ext[d]);
      auto it = index.find(key);
      if (it == index.end()) {
        const int k = (int)t.w.size();
        index.emplace(key, k);
        t.w.push_back(elw[ln]);
        for (int d = 0; d < s.ndim; d++) t.off.push_back((short)o[d]);
        for (int l = 0; l < nel; l++) t.hw.push_back(l == ln ? elw[ln] : 0.0);
      } else {
        t.w[it->second] += elw[ln];
        t.hw[(size_t)it->second * nel + ln] += elw[ln];
      }
    }
  }
  double sum = 0.0;
  for (double v : t.w) sum += v;
  if (sum != vol_sten) {
    const double ratio = vol_sten / sum;
    for (double &v : t.w) v *= ratio;
    for (double &v : t.hw) v *= ratio;
  }
  return t;
}

// ---- device builder ---------------------------------------------------------

__global__ void k_sten_elements(StenSpec s, const GaussTable *G, long ne, double *elw)
{
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < ne; e += (long)gridDim.x * blockDim.x) {
    int ijk[3];
    elem_ijk(s, e, ijk);
    double w[8];
    elem_weights(s, *G, ijk, w);
    for (int c = 0; c < s.nel; c++) elw[e * s.nel + c] = w[c];
  }
}

// One node of the (2 ext + 1)^ndim node box: its corner weights from the elements
// that share it, added in element order (the host's order), and its first-touch key
// (element index * 2^ndim + corner); nodes with no nonzero weight get key UINT_MAX.
__global__ void k_sten_nodes(StenSpec s, const double *elw, long nn, double *w, double *hw, unsigned *key,
                             unsigned *node)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nn; i += (long)gridDim.x * blockDim.x) {
    int o[3] = {0, 0, 0};
    long r = i;
    for (int d = 0; d < s.ndim; d++) {
      o[d] = (int)(r % (2 * s.ext[d] + 1)) - s.ext[d];
      r /= 2 * s.ext[d] + 1;
    }
    double sum = 0.0;
    unsigned first = 0xffffffffu;
    for (int ln = 0; ln < s.nel; ln++) hw[i * s.nel + ln] = 0.0;
    // elements e = o - c in ascending element order: c from the top corner down, x most significant
    for (int cc = s.nel - 1; cc >= 0; cc--) {
      int c[3] = {0, 0, 0}, ijk[3] = {0, 0, 0};
      // cc enumerates (c0, c1, c2) with c0 most significant
      if (s.ndim == 3) { c[0] = (cc >> 2) & 1; c[1] = (cc >> 1) & 1; c[2] = cc & 1; }
      else if (s.ndim == 2) { c[0] = (cc >> 1) & 1; c[1] = cc & 1; }
      else c[0] = cc & 1;
      bool inside = true;
      for (int d = 0; d < 3; d++) {
        ijk[d] = (d < s.ndim ? o[d] - c[d] : 0);
        if (ijk[d] < s.lo[d] || ijk[d] >= s.lo[d] + s.n[d]) inside = false;
      }
      if (!inside) continue;
      const int ln = c[0] | (c[1] << 1) | (c[2] << 2);
      const long e = elem_index(s, ijk);
      const double v = elw[e * s.nel + ln];
      if (v == 0.0) continue;
      if (first == 0xffffffffu) {
        sum = v;
        first = (unsigned)(e * s.nel + ln);
      } else {
        sum += v;
      }
      hw[i * s.nel + ln] = v;
    }
    w[i] = sum;
    key[i] = first;
    node[i] = (unsigned)i;
  }
}

// Table in first-touch order, then the renormalisation: a sequential sum in table order
// and one scale, as the host does.
__global__ void k_sten_gather(StenSpec s, const unsigned *order, int L, const double *w, const double *hw,
                              short *off, double *tw, double *thw)
{
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
    const long i = order[k];
    long r = i;
    for (int d = 0; d < s.ndim; d++) {
      off[(long)k * s.ndim + d] = (short)((int)(r % (2 * s.ext[d] + 1)) - s.ext[d]);
      r /= 2 * s.ext[d] + 1;
    }
    tw[k] = w[i];
    for (int ln = 0; ln < s.nel; ln++) thw[(long)k * s.nel + ln] = hw[i * s.nel + ln];
  }
}

__global__ void k_sten_sum(int L, const double *tw, double vol_sten, double *ratio)
{
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double sum = 0.0;
  for (int k = 0; k < L; k++) sum += tw[k];
  ratio[0] = sum != vol_sten ? vol_sten / sum : 1.0;
  ratio[1] = sum != vol_sten ? 1.0 : 0.0;
}

__global__ void k_sten_scale(int L, int nel, const double *ratio, double *tw, double *thw)
{
  if (ratio[1] == 0.0) return;
  const double f = ratio[0];
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < (long)L * (nel + 1);
       k += (long)gridDim.x * blockDim.x) {
    if (k < L) tw[k] *= f;
    else thw[k - L] *= f;
  }
}

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};

template <class T>
T *dev_alloc(DevBuf &b, size_t n)
{
  if (cudaMalloc(&b.p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
  return static_cast<T *>(b.p);
}

int build_device(const StenSpec &s, double vol_sten, Table &t)
{
  const long ne = (long)s.n[0] * s.n[1] * s.n[2];
  long nn = 1;
  for (int d = 0; d < s.ndim; d++) nn *= 2 * s.ext[d] + 1;
  if (ne * s.nel >= 0xffffffffL || nn >= 0x7fffffffL) return TGPU_ERR_ARG;
  DevBuf bG, bE, bW, bH, bK, bN, bK2, bN2, bT, bOff, bTw, bThw, bR;
  GaussTable *dG = dev_alloc<GaussTable>(bG, 1);
  double *elw = dev_alloc<double>(bE, (size_t)ne * s.nel);
  double *w = dev_alloc<double>(bW, nn);
  double *hw = dev_alloc<double>(bH, (size_t)nn * s.nel);
  unsigned *key = dev_alloc<unsigned>(bK, nn), *node = dev_alloc<unsigned>(bN, nn);
  unsigned *key2 = dev_alloc<unsigned>(bK2, nn), *node2 = dev_alloc<unsigned>(bN2, nn);
  double *ratio = dev_alloc<double>(bR, 2);
  if (!dG || !elw || !w || !hw || !key || !node || !key2 || !node2 || !ratio) return TGPU_ERR_CUDA;
  cudaStream_t st = 0;
  if (cudaMemcpyAsync(dG, &gauss_table(), sizeof(GaussTable), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return TGPU_ERR_CUDA;
  k_sten_elements<<<(unsigned)std::min<long>((ne + 127) / 128, 1L << 16), 128, 0, st>>>(s, dG, ne, elw);
  k_sten_nodes<<<(unsigned)std::min<long>((nn + 255) / 256, 1L << 16), 256, 0, st>>>(s, elw, nn, w, hw, key, node);
  size_t tmp_bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, key, key2, node, node2, (int)nn, 0, 32, st);
  void *tmp = dev_alloc<char>(bT, tmp_bytes);
  if (!tmp) return TGPU_ERR_CUDA;
  cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, key, key2, node, node2, (int)nn, 0, 32, st);
  // the present nodes are a prefix of the sorted keys
  std::vector<unsigned> hkey(nn);
  if (cudaMemcpyAsync(hkey.data(), key2, nn * sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return TGPU_ERR_CUDA;
  const int L = (int)(std::lower_bound(hkey.begin(), hkey.end(), 0xffffffffu) - hkey.begin());
  short *off = dev_alloc<short>(bOff, (size_t)L * s.ndim);
  double *tw = dev_alloc<double>(bTw, L), *thw = dev_alloc<double>(bThw, (size_t)L * s.nel);
  if (!off || !tw || !thw) return TGPU_ERR_CUDA;
  if (L > 0) {
    k_sten_gather<<<(unsigned)std::min((L + 255) / 256, 1 << 16), 256, 0, st>>>(s, node2, L, w, hw, off, tw, thw);
    k_sten_sum<<<1, 32, 0, st>>>(L, tw, vol_sten, ratio);
    k_sten_scale<<<(unsigned)std::min<long>(((long)L * (s.nel + 1) + 255) / 256, 1L << 16), 256, 0, st>>>(
        L, s.nel, ratio, tw, thw);
  }
  t.off.resize((size_t)L * s.ndim);
  t.w.resize(L);
  t.hw.resize((size_t)L * s.nel);
  if (L > 0 &&
      (cudaMemcpyAsync(t.off.data(), off, t.off.size() * sizeof(short), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(t.w.data(), tw, t.w.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
       cudaMemcpyAsync(t.hw.data(), thw, t.hw.size() * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess))
    return TGPU_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return TGPU_ERR_CUDA;
  return TGPU_OK;
}

// pairPot_find_rmin (src/dft_pairPot.c:98-152): grid search from 2 h in steps
// of h, then repeated refinement by factors of 100 until the minimum value
// changes by less than 1e-8 percent.
double find_rmin(double sigma, double eps, double rcut, double h0)
{
  double r = 2.0 * h0, delr = h0, rmin = 0.0, rlast = 0.0;
  double umin = u_lj_cs(r, sigma, eps, rcut);
  bool upd = false;
  while (r < rcut) {
    r += delr;
    const double u = u_lj_cs(r, sigma, eps, rcut);
    if (u < umin) { umin = u; rmin = r; upd = true; }
    rlast = r;
  }
  if (!upd || std::fabs(rmin - rlast) < 1.e-6) return sigma;
  double err = 1.0;
  while (err > 1.e-8) {
    const double uold = umin, dold = delr;
    const double rstart = rmin - dold;
    r = rstart;
    umin = u_lj_cs(rstart, sigma, eps, rcut);
    delr = dold / 100;
    while (r < rstart + 2.0 * dold) {
      r += delr;
      const double u = u_lj_cs(r, sigma, eps, rcut);
      if (u < umin) { umin = u; rmin = r; }
    }
    err = 100 * std::fabs(umin - uold) / std::fabs(umin);
  }
  return rmin;
}

int make_stencil(bool device, int type, int ndim, const double *esize, double hs_diam, const tgpu_pairpot &pp,
                 int capacity, short *offsets, double *weights, double *hw, double *volume)
{
  if (ndim < 1 || ndim > 3 || !esize) return TGPU_ERR_ARG;
  if (type != TGPU_STEN_DELTA && type != TGPU_STEN_THETA && type != TGPU_STEN_UATT) return TGPU_ERR_ARG;
  if (type == TGPU_STEN_UATT) {
    if (pp.pot != TGPU_PAIR_LJ12_6_CS && pp.pot != TGPU_PAIR_YUKAWA_CS && pp.pot != TGPU_PAIR_EXP_CS &&
        pp.pot != TGPU_PAIR_SW)
      return TGPU_ERR_UNSUPPORTED;
    if (pp.core_r < TGPU_CORE_SIGMA || pp.core_r > TGPU_CORE_SIGTOUMIN || pp.core_const < TGPU_CORECONST_UCONST ||
        pp.core_const > TGPU_CORECONST_ZERO || !(pp.rcut > 0.0) || !(pp.sigma > 0.0))
      return TGPU_ERR_ARG;
    if ((pp.pot == TGPU_PAIR_YUKAWA_CS || pp.pot == TGPU_PAIR_EXP_CS) && !(pp.kappa > 0.0)) return TGPU_ERR_ARG;
  }
  double vol = 0.0;
  const StenSpec s = make_spec(type, ndim, esize, hs_diam, pp, &vol);
  Table t;
  if (device) {
    const int st = build_device(s, vol, t);
    if (st != TGPU_OK) return st;
  } else {
    t = build_host(s, vol);
  }
  const int L = (int)t.w.size();
  if (volume) *volume = vol;
  if (!offsets || !weights) return L;   // size query
  if (L > capacity) return TGPU_ERR_ARG;
  std::memcpy(offsets, t.off.data(), sizeof(short) * t.off.size());
  std::memcpy(weights, t.w.data(), sizeof(double) * t.w.size());
  if (hw) std::memcpy(hw, t.hw.data(), sizeof(double) * t.hw.size());
  return L;
}

}  // namespace

namespace tgpu {
// the n-point Gauss-Legendre rule on [0,1] of the stencil builder, for the other set-up code
void gauss_rule01(int n, double *x, double *w) { gauss01(n, x, w); }
}  // namespace tgpu

extern "C" {

double tgpu_lj_rmin(double sigma, double eps_over_kT, double rcut, double esize0)
{
  return find_rmin(sigma, eps_over_kT, rcut, esize0);
}

static tgpu_pairpot lj_umin(double sigma, double eps_over_kT, double rcut, double rmin)
{
  tgpu_pairpot pp;
  std::memset(&pp, 0, sizeof(pp));
  pp.pot = TGPU_PAIR_LJ12_6_CS;
  pp.core_r = TGPU_CORE_UMIN;
  pp.core_const = TGPU_CORECONST_UCONST;
  pp.sigma = sigma;
  pp.eps_over_kT = eps_over_kT;
  pp.rcut = rcut;
  pp.rmin = rmin;
  return pp;
}

double tgpu_uatt(double r, double sigma, double eps_over_kT, double rcut, double rmin)
{
  double vol = 0.0;
  const double es[3] = {1.0, 1.0, 1.0};
  return u_att_cs(r, make_spec(TGPU_STEN_UATT, 1, es, 0.0, lj_umin(sigma, eps_over_kT, rcut, rmin), &vol));
}

double tgpu_pairpot_att(double r, const tgpu_pairpot *pp)
{
  if (!pp) return 0.0;
  double vol = 0.0;
  const double es[3] = {1.0, 1.0, 1.0};
  return u_att_cs(r, make_spec(TGPU_STEN_UATT, 1, es, 0.0, *pp, &vol));
}

int tgpu_make_stencil(int type, int ndim, const double *esize, double hs_diam, double sigma, double eps_over_kT,
                      double rcut, double rmin, int capacity, short *offsets, double *weights, double *hw,
                      double *volume)
{
  return make_stencil(false, type, ndim, esize, hs_diam, lj_umin(sigma, eps_over_kT, rcut, rmin), capacity, offsets,
                      weights, hw, volume);
}

int tgpu_make_stencil_device(int type, int ndim, const double *esize, double hs_diam, double sigma,
                             double eps_over_kT, double rcut, double rmin, int capacity, short *offsets,
                             double *weights, double *hw, double *volume)
{
  return make_stencil(true, type, ndim, esize, hs_diam, lj_umin(sigma, eps_over_kT, rcut, rmin), capacity, offsets,
                      weights, hw, volume);
}

int tgpu_make_attraction_stencil(const tgpu_pairpot *pp, int ndim, const double *esize, int device, int capacity,
                                 short *offsets, double *weights, double *hw, double *volume)
{
  if (!pp) return TGPU_ERR_ARG;
  return make_stencil(device != 0, TGPU_STEN_UATT, ndim, esize, 0.0, *pp, capacity, offsets, weights, hw, volume);
}

}  // extern "C"
