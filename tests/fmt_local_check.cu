// Per-node FMT math of the device path (tgpu_internal.h: fmt_dphi_at, fmt_hess_apply_at, fmt_phi)
// against the oracle's restatement of the reference's tables (oracle.c, included for its static
// functions) and against central differences, for the four functionals in 1, 2 and 3 dimensions.
// Built and run by tests/test_fmt_local_cpu.py; exits 1 when a bound is exceeded.
#include "oracle.c"
#include "tgpu_internal.h"
#include <cstdio>
#include <random>
#include <cmath>
using namespace tgpu;
static double rel(double a, double b, double s) { return std::fabs(a - b) / (std::fabs(b) + s); }
int main()
{
  int bad = 0;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  for (int fn = 0; fn < 4; fn++)
    for (int nd = 1; nd <= 3; nd++) {
      orc_problem p;
      memset(&p, 0, sizeof(p));
      p.ndim = nd;
      p.functional = fn;
      for (int d = 0; d < 3; d++) p.esize[d] = 0.1;
      const double R = 0.5;
      p.inv_rad[0] = 1.0 / R;
      p.inv_4pir[0] = 1.0 / (4 * PI * R);
      p.inv_4pirsq[0] = 1.0 / (4 * PI * R * R);
      double e_d1 = 0, e_del = 0, e_th = 0, e_ex = 0, e_g = 0, e_sym = 0;
      for (int trial = 0; trial < 2000; trial++) {
        double n[10];
        n[3] = 0.02 + 0.45 * U(rng);
        n[2] = 6.0 * n[3] * (0.7 + 0.6 * U(rng));   // n2 ~ 6 n3 / sigma
        n[1] = n[2] / (4 * PI * R) * (0.9 + 0.2 * U(rng));
        n[0] = n[2] / (4 * PI * R * R) * (0.9 + 0.2 * U(rng));
        for (int d = 0; d < nd; d++) {
          n[4 + nd + d] = (U(rng) - 0.5) * 0.8 * n[2] / std::sqrt((double)nd);
          n[4 + d] = n[4 + nd + d] / (4 * PI * R) * (0.9 + 0.2 * U(rng));
        }
        const int nrb = 4 + 2 * nd;
        // first derivatives vs the oracle's
        double inv[5];
        inv[0] = 1 - n[3]; inv[1] = 1 / inv[0]; inv[2] = inv[1] * inv[1]; inv[3] = inv[2] * inv[1]; inv[4] = inv[3] * inv[1];
        double dot12 = 0, dot22 = 0;
        for (int d = 0; d < nd; d++) { dot12 += n[4 + d] * n[4 + nd + d]; dot22 += n[4 + nd + d] * n[4 + nd + d]; }
        double o1[10], m1[10];
        if (fn == 0) fmt1_d1(nd, n, dot12, dot22, inv, o1);
        if (fn == 1) fmt2_d1(nd, n, dot12, dot22, inv, o1);
        if (fn == 2) fmt3_d1(nd, n, dot12, dot22, inv, o1);
        if (fn == 3) fmt4_d1(nd, n, dot12, dot22, inv, o1);
        fmt_dphi_at(n, m1, nd, fn);
        for (int k = 0; k < nrb; k++) e_d1 = std::max(e_d1, rel(m1[k], o1[k], 1.0));
        // gradient of phi by central differences vs dphi
        for (int k = 0; k < nrb; k++) {
          double np[10], nm[10];
          memcpy(np, n, sizeof(n)); memcpy(nm, n, sizeof(n));
          const double h = 1e-6 * std::max(std::fabs(n[k]), 1e-3);
          np[k] += h; nm[k] -= h;
          const double fd = (fmt_phi(np, nd, fn) - fmt_phi(nm, nd, fn)) / (2 * h);
          e_g = std::max(e_g, rel(fd, m1[k], 1.0));
        }
        // delta tables: column alpha = (M^T c)_alpha, reference form
        short off[3];
        double sign[3] = {1, 1, 1};
        for (int d = 0; d < nd; d++) off[d] = (short)((int)(U(rng) * 11) - 5);
        rbs t = d2_delta(&p, n, off, sign, 0);
        double c[10], z[10];
        c[0] = p.inv_4pirsq[0]; c[1] = p.inv_4pir[0]; c[2] = 1; c[3] = 0;
        for (int d = 0; d < nd; d++) {
          const double v = off[d] * p.esize[d] * p.inv_rad[0];
          c[4 + d] = -v * p.inv_4pir[0];
          c[4 + nd + d] = -v;
        }
        fmt_hess_apply_at(n, c, z, nd, fn, false, true);
        double tv[10];
        tv[0] = t.S0; tv[1] = t.S1; tv[2] = t.S2; tv[3] = t.S3;
        for (int d = 0; d < nd; d++) { tv[4 + d] = t.V1[d]; tv[4 + nd + d] = t.V2[d]; }
        for (int k = 0; k < nrb; k++) e_del = std::max(e_del, rel(z[k], tv[k], 1.0));
        // theta tables: row n3 of M
        rbs th = d2_theta(&p, n);
        double e3[10] = {0};
        e3[3] = 1;
        fmt_hess_apply_at(n, e3, z, nd, fn, false, true);
        tv[0] = th.S0; tv[1] = th.S1; tv[2] = th.S2; tv[3] = th.S3;
        for (int d = 0; d < nd; d++) { tv[4 + d] = th.V1[d]; tv[4 + nd + d] = th.V2[d]; }
        for (int k = 0; k < nrb; k++) e_th = std::max(e_th, rel(z[k], tv[k], 1.0));
        // exact form: columns of the Hessian vs central differences of dphi; and symmetry
        for (int k = 0; k < nrb; k++) {
          double np[10], nm[10], dp[10], dm[10], ek[10] = {0}, col[10], row[10];
          memcpy(np, n, sizeof(n)); memcpy(nm, n, sizeof(n));
          const double h = 1e-6 * std::max(std::fabs(n[k]), 1e-3);
          np[k] += h; nm[k] -= h;
          fmt_dphi_at(np, dp, nd, fn);
          fmt_dphi_at(nm, dm, nd, fn);
          ek[k] = 1;
          fmt_hess_apply_at(n, ek, col, nd, fn, true, false);
          fmt_hess_apply_at(n, ek, row, nd, fn, true, true);
          for (int m = 0; m < nrb; m++) {
            e_ex = std::max(e_ex, rel((dp[m] - dm[m]) / (2 * h), col[m], 1.0));
            e_sym = std::max(e_sym, rel(row[m], col[m], 1.0));
          }
        }
      }
      printf("FMT%d nd=%d  dphi-vs-oracle %.2e  dphi-vs-FD(phi) %.2e  delta %.2e  theta %.2e  exactH-vs-FD %.2e  sym %.2e\n",
             fn + 1, nd, e_d1, e_g, e_del, e_th, e_ex, e_sym);
      if (e_d1 > 1e-13 || e_del > 1e-13 || e_th > 1e-13 || e_sym > 1e-15 || e_g > 1e-5 || e_ex > 1e-5) bad = 1;
    }
  return bad;
}
