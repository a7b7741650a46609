// Host-side stencil tables (set-up, run once per problem).
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
// (src/dft_stencil_theta_R.c:34-75) and the WCA attraction
// (src/dft_stencil_theta_uattr.c:35-158) with the cut-and-shifted
// Lennard-Jones tail (src/dft_pairPot_LJ12_6.c:96-230).
//
// Gauss-Legendre nodes are computed here (Newton iteration on the Legendre
// recurrence) rather than taken from tables, so weights agree with the
// reference's to rounding, not bit for bit.
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/tramonto_gpu.h"

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884197;

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

struct UattParams {
  double sigma, eps, rcut, rmin;
};

// cut-and-shifted attractive tail with the core held at u(r_min) (Type_attr 0: ATTCORE_UMIN, CORECONST_UCONST)
double u_att_cs(double r, const UattParams &p)
{
  const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2;
  const double rc = 1.0 / p.rcut, rc2 = rc * rc, rc6 = rc2 * rc2 * rc2, rc12 = rc6 * rc6;
  if (r > p.rcut) return 0.0;
  if (r < p.rmin) r = p.rmin;
  const double ri = 1.0 / r, r2 = ri * ri, r6 = r2 * r2 * r2, r12 = r6 * r6;
  return 4.0 * p.eps * s6 * (s6 * (r12 - rc12) - (r6 - rc6));
}

double u_att_nocs(double r, const UattParams &p)
{
  const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2;
  if (r < p.rmin) r = p.rmin;
  const double ri = 1.0 / r, r2 = ri * ri, r6 = r2 * r2 * r2, r12 = r6 * r6;
  return 4.0 * p.eps * s6 * (s6 * r12 - r6);
}

double u_integral(double r, const UattParams &p)
{
  const double s2 = p.sigma * p.sigma, s6 = s2 * s2 * s2;
  const double ri = 1.0 / r, r3 = ri * ri * ri, r9 = r3 * r3 * r3;
  return 16 * kPi * p.eps * s6 * (-s6 * r9 / 9.0 + r3 / 3.0);
}

double u_lj_cs(double r, double sigma, double eps, double rc)
{
  if (r > rc) return 0.0;
  return 4.0 * eps * ((std::pow(sigma / r, 12) - std::pow(sigma / rc, 12)) - (std::pow(sigma / r, 6) - std::pow(sigma / rc, 6)));
}

struct Builder {
  int type, ndim;
  double esize[3];
  double R;           // stencil radius
  UattParams up{};
  int nel;            // corners per element
  std::vector<short> off;
  std::vector<double> w, hw;
  std::map<long, int> index;
  int ext[3] = {0, 0, 0};

  bool is_delta() const { return type == TGPU_STEN_DELTA; }

  int npt_boundary() const
  {
    if (type == TGPU_STEN_DELTA) return ndim == 3 ? 40 : 150;
    if (type == TGPU_STEN_THETA) return ndim == 3 ? 20 : 40;
    return ndim == 3 ? 1 : 20;
  }
  int ngauss(double r) const
  {
    if (type == TGPU_STEN_UATT) return 1;
    return r <= 4.000000001 ? 6 : 3;
  }
  int ngauss_integrand(double r) const
  {
    if (type != TGPU_STEN_UATT) return 0;
    if (r <= 4.000000001) return 40;
    if (r <= 16.00000001) return 20;
    return 12;
  }
  double weight(double rsq, int ngpu, const double *gpu, const double *gwu) const
  {
    if (type == TGPU_STEN_DELTA) {
      if (ndim == 1) return 2.0 * kPi * R;
      if (ndim == 2) return 2.0 / std::sqrt(1.0 - rsq);
      return 1.0;
    }
    if (type == TGPU_STEN_THETA) {
      if (ndim == 1) return (1.0 - rsq) * kPi * R * R;
      if (ndim == 2) return std::sqrt(1.0 - rsq) * 2.0 * R;
      return 1.0;
    }
    const double rc = up.rcut;
    double wsum = 0.0;
    const double zmax = std::sqrt(1 - rsq);
    if (ndim == 1) {
      for (int i = 0; i < ngpu; i++) {
        const double z = zmax * gpu[i];
        const double rho = std::sqrt(rsq + z * z) * rc;
        wsum += gwu[i] * z * u_att_cs(rho, up);
      }
      return 2.0 * kPi * wsum * rc * rc * zmax;
    }
    if (ndim == 2) {
      for (int i = 0; i < ngpu; i++) {
        const double z = zmax * gpu[i];
        const double rho = std::sqrt(rsq + z * z) * rc;
        wsum += gwu[i] * u_att_cs(rho, up);
      }
      return 2.0 * wsum * rc * zmax;
    }
    return u_att_cs(std::sqrt(rsq) * rc, up);
  }

  void distribute(double wt, const double *q, double *elw) const
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

  int in_out_on(const double *xl, const double *xr) const
  {
    bool in = false, out = false;
    const int nc = 1 << ndim;
    for (int c = 0; c < nc; c++) {
      double r2 = 0.0;
      for (int d = 0; d < ndim; d++) {
        const double v = (c >> d) & 1 ? xr[d] : xl[d];
        r2 += v * v;
      }
      (std::sqrt(r2) > R ? out : in) = true;
    }
    if (!in && out) return 1;
    if (in && !out) return -1;
    return 0;
  }

  void el_inside(const double *xl, double rc2, double *elw) const
  {
    double gp[12], gw[12], gpu[40], gwu[40];
    const double inv_r2 = 1.0 / (R * R);
    double vol = 1.0;
    for (int d = 0; d < ndim; d++) vol *= esize[d];
    const int ngp = ngauss(rc2);
    const int ngpu = ngauss_integrand(rc2);
    gauss01(ngp, gp, gw);
    if (ngpu > 0) gauss01(ngpu, gpu, gwu);
    double pt[3], q[3];
    for (int ig = 0; ig < ngp; ig++) {
      pt[0] = xl[0] + gp[ig] * esize[0];
      q[0] = gp[ig];
      if (ndim == 1) {
        const double rsq = pt[0] * pt[0] * inv_r2;
        double wt = weight(rsq, ngpu, gpu, gwu);
        wt *= gw[ig] * vol;
        distribute(wt, q, elw);
        continue;
      }
      for (int jg = 0; jg < ngp; jg++) {
        pt[1] = xl[1] + gp[jg] * esize[1];
        q[1] = gp[jg];
        if (ndim == 2) {
          const double rsq = (pt[0] * pt[0] + pt[1] * pt[1]) * inv_r2;
          double wt = weight(rsq, ngpu, gpu, gwu);
          wt *= gw[ig] * gw[jg] * vol;
          distribute(wt, q, elw);
          continue;
        }
        for (int kg = 0; kg < ngp; kg++) {
          pt[2] = xl[2] + gp[kg] * esize[2];
          q[2] = gp[kg];
          const double rsq = (pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]) * inv_r2;
          double wt = weight(rsq, ngpu, gpu, gwu);
          wt *= gw[ig] * gw[jg] * gw[kg] * vol;
          distribute(wt, q, elw);
        }
      }
    }
  }

  void el_boundary(const double *xl, double rc2, double *elw) const
  {
    double gpu[40], gwu[40];
    const double inv_r2 = 1.0 / (R * R);
    double vol = 1.0;
    for (int d = 0; d < ndim; d++) vol *= esize[d];
    const int npt = npt_boundary();
    const int ngpu = ngauss_integrand(rc2);
    if (ngpu > 0) gauss01(ngpu, gpu, gwu);
    const double inv = 1.0 / (double)npt;
    double ok = 0.0;
    if (ndim == 3 && is_delta()) {
      double t = 0.0;
      for (int d = 0; d < ndim; d++) t += esize[d] * esize[d];
      ok = 0.5 * inv * std::sqrt(t);
    }
    double pt[3], q[3];
    for (int ig = 0; ig < npt; ig++) {
      q[0] = ((double)ig + 0.5) * inv;
      pt[0] = xl[0] + q[0] * esize[0];
      if (ndim == 1) {
        const double rsq = pt[0] * pt[0] * inv_r2;
        if (rsq <= 1.000001) {
          double wt = weight(rsq, ngpu, gpu, gwu);
          if (std::fabs(rsq - 1.0) <= 1.e-8) wt *= 0.5;
          wt *= inv * vol;
          distribute(wt, q, elw);
        }
        continue;
      }
      for (int jg = 0; jg < npt; jg++) {
        q[1] = ((double)jg + 0.5) * inv;
        pt[1] = xl[1] + q[1] * esize[1];
        if (ndim == 2) {
          const double rsq = (pt[0] * pt[0] + pt[1] * pt[1]) * inv_r2;
          if (rsq <= 1.0000001) {
            double wt = weight(rsq, ngpu, gpu, gwu);
            if (std::fabs(rsq - 1.0) <= 1.e-8) wt *= 0.5;
            wt *= inv * inv * vol;
            distribute(wt, q, elw);
          }
          continue;
        }
        for (int kg = 0; kg < npt; kg++) {
          q[2] = ((double)kg + 0.5) * inv;
          pt[2] = xl[2] + q[2] * esize[2];
          const double rsq = (pt[0] * pt[0] + pt[1] * pt[1] + pt[2] * pt[2]) * inv_r2;
          if ((rsq <= 1.00000001 && !is_delta()) || (is_delta() && std::fabs(rsq - 1.0) < 2 * ok)) {
            double wt = weight(rsq, ngpu, gpu, gwu);
            if (std::fabs(rsq - 1.0) <= 1.e-8 && !is_delta()) wt *= 0.5;
            wt *= (inv * inv * inv) * vol;
            distribute(wt, q, elw);
          }
        }
      }
    }
  }

  void merge(const int *ijk, const double *elw)
  {
    for (int ln = 0; ln < nel; ln++) {
      if (elw[ln] == 0.0) continue;
      int o[3] = {0, 0, 0};
      for (int d = 0; d < ndim; d++) o[d] = ijk[d] + ((ln >> d) & 1);
      long key = 0;
      for (int d = ndim - 1; d >= 0; d--) key = key * (2 * ext[d] + 1) + (o[d] + ext[d]);
      auto it = index.find(key);
      if (it == index.end()) {
        const int k = (int)w.size();
        index.emplace(key, k);
        w.push_back(elw[ln]);
        for (int d = 0; d < ndim; d++) off.push_back((short)o[d]);
        for (int l = 0; l < nel; l++) hw.push_back(l == ln ? elw[ln] : 0.0);
      } else {
        w[it->second] += elw[ln];
        hw[(size_t)it->second * nel + ln] += elw[ln];
      }
    }
  }

  void run(double vol_sten, bool renormalize)
  {
    nel = 1 << ndim;
    for (int d = 0; d < ndim; d++) ext[d] = (int)((float)R / (float)esize[d] + 0.999);
    const int i0 = -ext[0], i1 = ext[0];
    const int j0 = ndim >= 2 ? -ext[1] : 0, j1 = ndim >= 2 ? ext[1] : 1;
    const int k0 = ndim == 3 ? -ext[2] : 0, k1 = ndim == 3 ? ext[2] : 1;
    for (int i = i0; i < i1; i++)
      for (int j = j0; j < j1; j++)
        for (int k = k0; k < k1; k++) {
          const int ijk[3] = {i, j, k};
          double xl[3] = {0, 0, 0}, xr[3] = {0, 0, 0}, xm[3];
          for (int d = 0; d < ndim; d++) {
            xl[d] = ijk[d] * esize[d];
            xr[d] = (ijk[d] + 1) * esize[d];
          }
          double rc2 = 0.0;
          for (int d = 0; d < ndim; d++) {
            xm[d] = xl[d] + 0.5 * esize[d];
            rc2 += xm[d] * xm[d];
          }
          double elw[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          const int flag = in_out_on(xl, xr);
          if (flag == 1 || (flag == -1 && ndim == 3 && is_delta())) continue;
          if (flag == -1) el_inside(xl, rc2, elw);
          else el_boundary(xl, rc2, elw);
          merge(ijk, elw);
        }
    if (renormalize) {
      double sum = 0.0;
      for (double v : w) sum += v;
      if (sum != vol_sten) {
        const double ratio = vol_sten / sum;
        for (double &v : w) v *= ratio;
        for (double &v : hw) v *= ratio;
      }
    }
  }
};

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

}  // namespace

extern "C" {

double tgpu_lj_rmin(double sigma, double eps_over_kT, double rcut, double esize0)
{
  return find_rmin(sigma, eps_over_kT, rcut, esize0);
}

double tgpu_uatt(double r, double sigma, double eps_over_kT, double rcut, double rmin)
{
  UattParams p{sigma, eps_over_kT, rcut, rmin};
  return u_att_cs(r, p);
}

int tgpu_make_stencil(int type, int ndim, const double *esize, double hs_diam, double sigma, double eps_over_kT,
                      double rcut, double rmin, int capacity, short *offsets, double *weights, double *hw,
                      double *volume)
{
  if (ndim < 1 || ndim > 3 || !esize) return TGPU_ERR_ARG;
  Builder b;
  b.type = type;
  b.ndim = ndim;
  for (int d = 0; d < 3; d++) b.esize[d] = d < ndim ? esize[d] : 0.0;
  double vol = 0.0;
  if (type == TGPU_STEN_DELTA) {
    b.R = hs_diam / 2.0;
    vol = kPi * std::pow(hs_diam, 2);
  } else if (type == TGPU_STEN_THETA) {
    b.R = hs_diam / 2.0;
    vol = kPi * std::pow(hs_diam, 3) / 6.0;
  } else if (type == TGPU_STEN_UATT) {
    b.R = rcut;
    b.up = UattParams{sigma, eps_over_kT, rcut, rmin};
    // StenTheta_uattr_sten_vol (src/dft_stencil_theta_uattr.c:39-88), WCA core held at u(r_min)
    vol = (4.0 / 3.0) * kPi * std::pow(rmin, 3.0) * u_att_nocs(rmin, b.up) -
          (4.0 / 3.0) * kPi * std::pow(rcut, 3.0) * u_att_nocs(rcut, b.up) + u_integral(rcut, b.up) -
          u_integral(rmin, b.up);
  } else {
    return TGPU_ERR_ARG;
  }
  b.run(vol, true);
  const int L = (int)b.w.size();
  if (volume) *volume = vol;
  if (!offsets || !weights) return L;   // size query
  if (L > capacity) return TGPU_ERR_ARG;
  std::memcpy(offsets, b.off.data(), sizeof(short) * b.off.size());
  std::memcpy(weights, b.w.data(), sizeof(double) * b.w.size());
  if (hw) std::memcpy(hw, b.hw.data(), sizeof(double) * b.hw.size());
  return L;
}

}  // extern "C"
