/* CPU restatement of the reference's nonlocal-density fill (test infrastructure).
 * See oracle.h for scope and conventions.  Every function names the reference
 * lines it follows; loop orders and branch structure are kept as in the
 * reference so that results agree to rounding. */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PI 3.141592653589793238462643383279502884197

long orc_nnodes(const orc_problem *p)
{
  long n = 1;
  for (int d = 0; d < p->ndim; d++) n *= p->nx[d];
  return n;
}

static void node_to_ijk(const orc_problem *p, long node, int *ijk)
{
  ijk[0] = ijk[1] = ijk[2] = 0;
  for (int d = 0; d < p->ndim; d++) {
    ijk[d] = (int)(node % p->nx[d]);
    node /= p->nx[d];
  }
}

/* offset_to_node_box (src/dft_mesh_lib.c:203-297) for one process whose box is
 * the whole mesh.  Returns a node >= 0, -1 (bulk), -3 / -4 (beyond the low / high
 * bulk boundary of a phase interface), -2 (inside a wall) or -9 for a double
 * reflection, which the reference rejects. */
static long bulk_side(const orc_problem *p, int high)
{
  return p->interface == 2 ? (high ? -4 : -3) : -1;
}

static long offset_to_node(const orc_problem *p, const int *ijk, const short *off, int *reflect)
{
  int s[3] = {0, 0, 0};
  for (int i = 0; i < p->ndim; i++) {
    const int n = p->nx[i];
    s[i] = ijk[i] + off[i];
    reflect[i] = 0;
    if (s[i] < 0) {
      switch (p->bc[i][0]) {
        case ORC_BC_IN_BULK: return bulk_side(p, 0);
        case ORC_BC_IN_WALL: return -2;
        case ORC_BC_REFLECT:
          reflect[i] = 1;
          s[i] = -s[i];
          if (s[i] >= n) {
            if (p->bc[i][1] == ORC_BC_IN_BULK) return bulk_side(p, 1);
            if (p->bc[i][1] == ORC_BC_IN_WALL) return -2;
            return -9;
          }
          break;
        case ORC_BC_PERIODIC: s[i] += n; break;
      }
    } else if (s[i] >= n) {
      switch (p->bc[i][1]) {
        case ORC_BC_IN_BULK: return bulk_side(p, 1);
        case ORC_BC_IN_WALL: return -2;
        case ORC_BC_REFLECT:
          reflect[i] = 1;
          s[i] = 2 * (n - 1) - s[i];
          if (s[i] < 0) {
            if (p->bc[i][0] == ORC_BC_IN_BULK) return bulk_side(p, 0);
            if (p->bc[i][0] == ORC_BC_IN_WALL) return -2;
            return -9;
          }
          break;
        case ORC_BC_PERIODIC: s[i] -= n; break;
      }
    }
  }
  long node = 0;
  for (int d = p->ndim - 1; d >= 0; d--) node = node * p->nx[d] + s[d];
  return node;
}

/* HW_boundary_weight (src/dft_utils.c:41-62): the weight of a stencil point at
 * a hard-wall boundary node counts only the element corners that lie in
 * fluid elements.  fluid_masks holds, per node and reflection pattern, the
 * corner bits node_box_to_elem_box_reflect would find in fluid elements. */
static double hw_weight(const orc_problem *p, int jlist, const double *hw, long jnode, const int *reflect)
{
  const long N = orc_nnodes(p);
  const int nel = 1 << p->ndim;
  int r = 0;
  for (int d = 0; d < p->ndim; d++) r |= (reflect[d] ? 1 : 0) << d;
  const int mask = p->fluid_masks[((long)jlist * nel + r) * N + jnode];
  double w = 0.0;
  for (int ln = 0; ln < nel; ln++)
    if (mask & (1 << ln)) w += hw[ln];
  return w;
}

/* solutionVec_to_nOrdering (src/dft_utils.c:205-221) */
static void sv_to_n(const orc_problem *p, const double *x, long node, double *n)
{
  const long N = orc_nnodes(p);
  const int nd = p->ndim;
  const double *rb = x + (long)p->first_rb * N;
  n[0] = rb[3 * N + node];
  n[1] = rb[2 * N + node];
  n[2] = rb[1 * N + node];
  n[3] = rb[0 * N + node];
  for (int d = 0; d < nd; d++) {
    n[4 + d] = rb[(4 + nd + d) * N + node];
    n[4 + nd + d] = rb[(4 + d) * N + node];
  }
}

/* FMT1_1stderiv (src/dft_physics_FMT1.c:59-77) */
static void fmt1_d1(int nd, const double *n, double dot12, double dot22, const double *inv, double *out)
{
  out[0] = log(inv[1]);
  out[1] = n[2] * inv[1];
  out[2] = n[1] * inv[1] + (n[2] * n[2] - dot22) * inv[2] / (8.0 * PI);
  out[3] = n[0] * inv[1] + (n[1] * n[2] - dot12) * inv[2] + (n[2] * n[2] * n[2] - 3. * n[2] * dot22) * inv[3] / (12.0 * PI);
  for (int d = 0; d < nd; d++) {
    out[4 + d] = -n[4 + nd + d] * inv[1];
    out[4 + d + nd] = -n[4 + d] * inv[1] - n[2] * n[4 + nd + d] * inv[2] / (4.0 * PI);
  }
}

/* FMT3_1stderiv (src/dft_physics_FMT3.c:61-96) */
static void fmt3_d1(int nd, const double *n, double dot12, double dot22, const double *inv, double *out)
{
  out[0] = log(inv[1]);
  out[1] = n[2] * inv[1];
  if (n[3] > 1.e-10) {
    out[2] = n[1] * inv[1] + (n[2] * n[2] - dot22) * inv[2] * (n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3])) / (12.0 * PI * n[3] * n[3]);
    out[3] = n[0] * inv[1] + (n[1] * n[2] - dot12) * inv[2] +
             (((n[2] * n[2] * n[2] - 3.0 * n[2] * dot22) * inv[2]) / (36. * PI * n[3] * n[3])) *
                 (+2. * (n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3])) * inv[1] + (-2. * (1. - n[3]) * log(1. - n[3]) + n[3]) -
                  2. * ((n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3])) / n[3]));
  } else {
    out[2] = 0.0;
    out[3] = 0.0;
  }
  for (int d = 0; d < nd; d++) {
    const int iv1 = 4 + d, iv2 = 4 + nd + d;
    out[iv1] = -n[iv2] * inv[1];
    if (n[3] > 1.e-10)
      out[iv2] = -n[iv1] * inv[1] - n[2] * n[iv2] * inv[2] * (n[3] + (1.0 - n[3]) * (1.0 - n[3]) * log(1.0 - n[3])) / (6.0 * PI * n[3] * n[3]);
    else
      out[iv2] = 0.0;
  }
}

/* FMT2_1stderiv (src/dft_physics_FMT2.c:60-99): the Rosenfeld terms with the
 * third term (n2 - V2.V2/n2)^3 / (24 pi (1-n3)^2); alpha = n2 - V2.V2/n2,
 * beta = 1 + V2.V2/n2^2, gamma = V2/n2, and alpha = n2, beta = 1, gamma = 0
 * where n2 <= 1e-15. */
static void fmt2_d1(int nd, const double *n, double dot12, double dot22, const double *inv, double *out)
{
  out[0] = log(inv[1]);
  out[1] = n[2] * inv[1];
  out[2] = n[1] * inv[1];
  out[3] = n[0] * inv[1] + (n[1] * n[2] - dot12) * inv[2];
  for (int d = 0; d < nd; d++) {
    out[4 + d] = -n[4 + nd + d] * inv[1];
    out[4 + nd + d] = -n[4 + d] * inv[1];
  }
  double alpha = n[2], beta = 1.0, gamma[3] = {0.0, 0.0, 0.0};
  if (n[2] > 1.e-15) {
    alpha = n[2] - dot22 / n[2];
    beta = 1.0 + dot22 / (n[2] * n[2]);
    for (int d = 0; d < nd; d++) gamma[d] = n[4 + nd + d] / n[2];
  }
  const double a2 = alpha * alpha, a3 = a2 * alpha;
  out[2] += a2 * beta * inv[2] / (8.0 * PI);
  out[3] += a3 * inv[3] / (12.0 * PI);
  for (int d = 0; d < nd; d++) out[4 + nd + d] -= inv[2] * a2 * gamma[d] / (4.0 * PI);
}

/* FMT4_1stderiv (src/dft_physics_FMT4.c:61-97): White-Bear n3 dependence with
 * the (1 - V2.V2/n2^2)^3 vector correction; all n2, n3 and V2 derivatives are
 * zero where n3 <= 1e-10, as in the reference. */
static void fmt4_d1(int nd, const double *n, double dot12, double dot22, const double *inv, double *out)
{
  out[0] = log(inv[1]);
  out[1] = n[2] * inv[1];
  double fac = 0.0, fac2 = 0.0;
  if (n[3] > 1.e-10) {
    fac = 1 - dot22 / (n[2] * n[2]);
    const double fac1 = n[3] - 2. * (1. - n[3]) * log(1. - n[3]);
    fac2 = (n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3]));
    const double f3 = fac * fac * fac, n2c = n[2] * n[2] * n[2];
    out[2] = n[1] * inv[1] + (n[2] * n[2] * f3 + 2 * fac * fac * dot22) * inv[2] * fac2 / (12.0 * PI * n[3] * n[3]);
    out[3] = n[0] * inv[1] + (n[1] * n[2] - dot12) * inv[2] + fac1 * n2c * f3 * inv[2] / (36.0 * PI * n[3] * n[3]) +
             fac2 * n2c * f3 * (-inv[2] / (n[3] * n[3] * n[3]) + inv[3] / (n[3] * n[3])) / (18.0 * PI);
  } else {
    out[2] = 0.0;
    out[3] = 0.0;
  }
  for (int d = 0; d < nd; d++) {
    const int iv1 = 4 + d, iv2 = 4 + nd + d;
    out[iv1] = -n[iv2] * inv[1];
    out[iv2] = (n[3] > 1.e-10)
                   ? -n[iv1] * inv[1] - n[2] * n[iv2] * fac2 * inv[2] * fac * fac / (6.0 * PI * n[3] * n[3])
                   : 0.0;
  }
}

/* calc_FMT_derivatives (src/dft_fill_FMT.c:349-385) at one node */
static void node_dphi(const orc_problem *p, const double *x, long node, double *out)
{
  double n[10], inv[5];
  const int nd = p->ndim;
  sv_to_n(p, x, node, n);
  inv[0] = (1.0 - n[3]);
  inv[1] = 1.0 / inv[0];
  inv[2] = inv[1] * inv[1];
  inv[3] = inv[2] * inv[1];
  inv[4] = inv[3] * inv[1];
  double dot22 = 0.0, dot12 = 0.0;
  for (int d = 0; d < nd; d++) {
    dot22 += n[4 + nd + d] * n[4 + nd + d];
    dot12 += n[4 + d] * n[4 + nd + d];
  }
  switch (p->functional) {
    case ORC_FMT2: fmt2_d1(nd, n, dot12, dot22, inv, out); break;
    case ORC_FMT3: fmt3_d1(nd, n, dot12, dot22, inv, out); break;
    case ORC_FMT4: fmt4_d1(nd, n, dot12, dot22, inv, out); break;
    default: fmt1_d1(nd, n, dot12, dot22, inv, out); break;
  }
}

int orc_dphi(const orc_problem *p, const double *x, double *dphi)
{
  const long N = orc_nnodes(p);
  const int nrb = 4 + 2 * p->ndim;
  double loc[10];
  for (long i = 0; i < N; i++) {
    node_dphi(p, x, i, loc);
    for (int k = 0; k < nrb; k++) dphi[(long)k * N + i] = loc[k];
  }
  return 0;
}

typedef struct { double S0, S1, S2, S3, V1[3], V2[3]; } rbs;

/* d2phi_drb2_delta_rb_FMT1 (src/dft_physics_FMT1.c:79-129) */
static rbs d2_delta_fmt1(const orc_problem *p, const double *n, const short *off, const double *sign, int ic)
{
  rbs t;
  const int nd = p->ndim;
  double n1v[3], n2v[3], v[3];
  for (int d = 0; d < nd; d++) {
    n2v[d] = sign[d] * n[4 + nd + d];
    n1v[d] = sign[d] * n[4 + d];
  }
  const double a = 1.0 / (1.0 - n[3]), a2 = a * a, a3 = a2 * a;
  const double inv4pi = 1.0 / (4.0 * PI);
  for (int d = 0; d < nd; d++) v[d] = off[d] * p->esize[d] * p->inv_rad[ic];
  t.S2 = (a * p->inv_4pir[ic] + n[2] * inv4pi * a2);
  for (int d = 0; d < nd; d++) t.S2 += v[d] * n2v[d] * inv4pi * a2;
  t.S3 = (p->inv_4pirsq[ic] * a + n[2] * p->inv_4pir[ic] * a2 + n[1] * a2 + n[2] * n[2] * inv4pi * a3);
  for (int d = 0; d < nd; d++)
    t.S3 += a2 * (-n2v[d] * n2v[d] * inv4pi * a + v[d] * (n2v[d] * p->inv_4pir[ic] + n1v[d] + n[2] * n2v[d] * a / (2 * PI)));
  t.S0 = 0.0;
  t.S1 = a;
  for (int d = 0; d < nd; d++) t.V1[d] = sign[d] * a * v[d];
  for (int d = 0; d < nd; d++)
    t.V2[d] = sign[d] * (-n2v[d] * inv4pi * a2 - (-p->inv_4pir[ic] * a - n[2] * inv4pi * a2) * v[d]);
  return t;
}

/* d2phi_drb2_theta_rb_FMT1 (src/dft_physics_FMT1.c:131-168) */
static rbs d2_theta_fmt1(const orc_problem *p, const double *n)
{
  rbs t;
  const int nd = p->ndim;
  const double a = 1.0 / (1.0 - n[3]), a2 = a * a, a3 = a2 * a, a4 = a3 * a;
  const double inv4pi = 1.0 / (4.0 * PI);
  t.S2 = (n[1] * a2 + n[2] * n[2] * inv4pi * a3);
  for (int d = 0; d < nd; d++) t.S2 += -n[4 + nd + d] * n[4 + nd + d] * inv4pi * a3;
  t.S3 = n[0] * a2 + 2 * n[1] * n[2] * a3 + n[2] * n[2] * n[2] * inv4pi * a4;
  for (int d = 0; d < nd; d++)
    t.S3 += -(2 * n[4 + d] * n[4 + nd + d] * a3 + 3 * n[2] * n[4 + nd + d] * n[4 + nd + d] * inv4pi * a4);
  t.S0 = a;
  t.S1 = n[2] * a2;
  for (int d = 0; d < nd; d++) t.V1[d] = -n[4 + nd + d] * a2;
  for (int d = 0; d < nd; d++) t.V2[d] = -(n[4 + d] * a2 + n[2] * n[4 + nd + d] * a3 / (2.0 * PI));
  return t;
}

/* d2phi_drb2_delta_rb_FMT3 (src/dft_physics_FMT3.c:101-187).  As in the
 * reference, this form uses the vector densities without the reflection sign. */
static rbs d2_delta_fmt3(const orc_problem *p, const double *n, const short *off, const double *sign, int ic)
{
  rbs t;
  const int nd = p->ndim;
  double inv[5], v[3];
  double dot22 = 0.0;
  for (int d = 0; d < nd; d++) dot22 += n[4 + nd + d] * n[4 + nd + d];
  inv[0] = (1. - n[3]);
  inv[1] = 1.0 / (1.0 - n[3]);
  inv[2] = inv[1] * inv[1];
  inv[3] = inv[2] * inv[1];
  inv[4] = inv[3] * inv[1];
  const double n3sq = n[3] * n[3], n3cb = n3sq * n[3], n2sq = n[2] * n[2];
  memset(&t, 0, sizeof(t));
  if (n[3] > 1.e-10) {
    const double fac1 = n[3] - 2 * (1. - n[3]) * log(1. - n[3]);
    const double fac2 = n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3]);
    const double fac3 = -(inv[2] / n3cb) + (inv[3] / n3sq);
    for (int d = 0; d < nd; d++) v[d] = off[d] * p->esize[d] * p->inv_rad[ic];
    t.S2 = (inv[1] * p->inv_4pir[ic] + n[2] * fac2 * inv[2] / (6. * PI * n3sq));
    for (int d = 0; d < nd; d++) t.S2 += v[d] * n[4 + nd + d] * fac2 * inv[2] / (6. * PI * n3sq);
    t.S3 = (p->inv_4pirsq[ic] * inv[1] + p->inv_4pir[ic] * n[2] * inv[2] + n[1] * inv[2] +
            (n2sq - dot22) * ((2. * fac2 * fac3) + (fac1 * inv[2] / n3sq)) / (12. * PI));
    for (int d = 0; d < nd; d++)
      t.S3 += v[d] * (n[4 + nd + d] * p->inv_4pir[ic] * inv[2] + n[4 + d] * inv[2] +
                      n[2] * n[4 + nd + d] * ((2. * fac2 * fac3) + (fac1 * inv[2] / n3sq)) / (6. * PI));
    t.S0 = 0.0;
    t.S1 = inv[1];
    for (int d = 0; d < nd; d++) t.V1[d] = sign[d] * (inv[1]) * v[d];
    for (int d = 0; d < nd; d++)
      t.V2[d] = sign[d] * (-n[4 + nd + d] * inv[2] * fac2 / (6. * PI * n3sq) -
                           (-p->inv_4pir[ic] * inv[1] - n[2] * fac2 * inv[2] / (6. * PI * n3sq)) * v[d]);
  }
  return t;
}

/* d2phi_drb2_theta_rb_FMT3 (src/dft_physics_FMT3.c:192-265) */
static rbs d2_theta_fmt3(const orc_problem *p, const double *n)
{
  rbs t;
  const int nd = p->ndim;
  double inv[5];
  double dot22 = 0.0, dot12 = 0.0;
  for (int d = 0; d < nd; d++) {
    dot22 += n[4 + nd + d] * n[4 + nd + d];
    dot12 += n[4 + d] * n[4 + nd + d];
  }
  inv[0] = (1. - n[3]);
  inv[1] = 1.0 / (1.0 - n[3]);
  inv[2] = inv[1] * inv[1];
  inv[3] = inv[2] * inv[1];
  inv[4] = inv[3] * inv[1];
  const double n3sq = n[3] * n[3], n3cb = n3sq * n[3], n3_4th = n3cb * n[3];
  const double n2sq = n[2] * n[2], n2cb = n2sq * n[2];
  memset(&t, 0, sizeof(t));
  if (n[3] > 1.e-10) {
    const double fac1 = n[3] - 2 * (1. - n[3]) * log(1. - n[3]);
    const double fac2 = n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3]);
    const double fac3 = -(inv[2] / n3cb) + (inv[3] / n3sq);
    t.S2 = (n[1] * inv[2] + (n[2] * n[2] - dot22) * (fac1 * inv[2] / n3sq + 2. * fac2 * fac3) / (12 * PI));
    t.S3 = (n[0] * inv[2] + 2 * (n[1] * n[2] - dot12) * inv[3] +
            ((n2cb - 3. * n[2] * dot22) / (36. * PI)) *
                (+(((2. * log(1. - n[3]) + 3) * inv[2]) / n3sq) + (4. * fac1 * fac3) +
                 (fac2 * (6. * inv[2] / n3_4th + 6. * inv[4] / n3sq - 8. * inv[3] / n3cb))));
    t.S0 = inv[1];
    t.S1 = n[2] * inv[2];
    for (int d = 0; d < nd; d++) t.V1[d] = -n[4 + nd + d] * inv[2];
    for (int d = 0; d < nd; d++)
      t.V2[d] = -(n[4 + d] * inv[2] + n[2] * n[4 + nd + d] * ((fac1 * inv[2] / n3sq) + (2. * fac2 * fac3)) / (6. * PI));
  }
  return t;
}

/* The n2/V2 structure of the FMT2 third term at one node: alpha, beta, gamma as
 * in fmt2_d1 (gamma from the signed vector densities), eps = alpha/n2 and
 * |gamma|^2, with eps = 1, gamma = 0 where n2 <= 1e-15. */
typedef struct { double alpha, beta, eps, gg, gamma[3]; } fmt2_terms;

static fmt2_terms fmt2_terms_of(int nd, double n2, const double *n2v)
{
  fmt2_terms t = {n2, 1.0, 1.0, 0.0, {0.0, 0.0, 0.0}};
  double q = 0.0;
  for (int d = 0; d < nd; d++) q += n2v[d] * n2v[d];
  if (n2 > 1.e-15) {
    t.alpha = n2 - q / n2;
    t.beta = 1.0 + q / (n2 * n2);
    for (int d = 0; d < nd; d++) {
      t.gamma[d] = n2v[d] / n2;
      t.gg += t.gamma[d] * t.gamma[d];
    }
    t.eps = t.alpha / n2;
  }
  return t;
}

/* d2phi_drb2_delta_rb_FMT2 (src/dft_physics_FMT2.c:104-186).  The V2-V2 entry
 * keeps the reference's form, -alpha (4 |gamma|^2 - eps) v_d / (4 pi (1-n3)^2):
 * the Hessian of the FMT2 energy density has 4 gamma_d (gamma . v) there, the
 * same in one dimension. */
static rbs d2_delta_fmt2(const orc_problem *p, const double *n, const short *off, const double *sign, int ic)
{
  rbs t;
  const int nd = p->ndim;
  double n1v[3], n2v[3], v[3];
  for (int d = 0; d < nd; d++) {
    n2v[d] = sign[d] * n[4 + nd + d];
    n1v[d] = sign[d] * n[4 + d];
  }
  const fmt2_terms g = fmt2_terms_of(nd, n[2], n2v);
  const double a = 1.0 / (1.0 - n[3]), a2 = a * a, a3 = a2 * a;
  const double i4p = 1.0 / (4.0 * PI);
  for (int d = 0; d < nd; d++) v[d] = off[d] * p->esize[d] * p->inv_rad[ic];
  t.S2 = a * p->inv_4pir[ic] + i4p * a2 * g.alpha * (g.beta * g.beta - g.eps * g.gg);
  for (int d = 0; d < nd; d++) t.S2 -= i4p * a2 * g.alpha * (g.eps - 2 * g.beta) * g.gamma[d] * v[d];
  t.S3 = (p->inv_4pirsq[ic] * a + n[2] * p->inv_4pir[ic] * a2 + n[1] * a2);
  for (int d = 0; d < nd; d++) t.S3 += a2 * v[d] * (n2v[d] * p->inv_4pir[ic] + n1v[d]);
  t.S3 += i4p * a3 * g.alpha * g.alpha * g.beta;
  for (int d = 0; d < nd; d++) t.S3 += 2.0 * i4p * a3 * g.alpha * g.alpha * g.gamma[d] * v[d];
  t.S0 = 0.0;
  t.S1 = a;
  for (int d = 0; d < nd; d++) {
    t.V1[d] = sign[d] * a * v[d];
    t.V2[d] = sign[d] * (p->inv_4pir[ic] * a) * v[d];
  }
  for (int d = 0; d < nd; d++) {
    t.V2[d] += sign[d] * i4p * a2 * g.alpha * (g.eps - 2.0 * g.beta) * g.gamma[d];
    t.V2[d] -= sign[d] * i4p * a2 * g.alpha * (4.0 * g.gg - g.eps) * v[d];
  }
  return t;
}

/* d2phi_drb2_theta_rb_FMT2 (src/dft_physics_FMT2.c:191-250) */
static rbs d2_theta_fmt2(const orc_problem *p, const double *n)
{
  rbs t;
  const int nd = p->ndim;
  double dot12 = 0.0;
  for (int d = 0; d < nd; d++) dot12 += n[4 + d] * n[4 + nd + d];
  const fmt2_terms g = fmt2_terms_of(nd, n[2], n + 4 + nd);
  const double a = 1.0 / (1.0 - n[3]), a2 = a * a, a3 = a2 * a, a4 = a3 * a;
  const double i4p = 1.0 / (4.0 * PI);
  const double al2 = g.alpha * g.alpha;
  t.S2 = n[1] * a2 + i4p * a3 * al2 * g.beta;
  t.S3 = n[0] * a2 + 2.0 * (n[1] * n[2] - dot12) * a3 + i4p * a4 * al2 * g.alpha;
  t.S0 = a;
  t.S1 = n[2] * a2;
  for (int d = 0; d < nd; d++) {
    t.V1[d] = -n[4 + nd + d] * a2;
    t.V2[d] = -n[4 + d] * a2 - 2.0 * i4p * a3 * al2 * g.gamma[d];
  }
  return t;
}

/* d2phi_drb2_delta_rb_FMT4 (src/dft_physics_FMT4.c:102-196).  As FMT3, it uses
 * the vector densities without the reflection sign.  Its V2 entry keeps the
 * reference's n2-V2 coefficient (fac^2 - 4 |V2|^2 fac / n2); the Hessian of the
 * FMT4 energy density has fac (1 + 3 |V2|^2 / n2^2) there. */
static rbs d2_delta_fmt4(const orc_problem *p, const double *n, const short *off, const double *sign, int ic)
{
  rbs t;
  const int nd = p->ndim;
  double inv[5], v[3];
  double dot22 = 0.0;
  for (int d = 0; d < nd; d++) dot22 += n[4 + nd + d] * n[4 + nd + d];
  inv[0] = (1. - n[3]);
  inv[1] = 1.0 / (1.0 - n[3]);
  inv[2] = inv[1] * inv[1];
  inv[3] = inv[2] * inv[1];
  inv[4] = inv[3] * inv[1];
  const double n3sq = n[3] * n[3], n3cb = n3sq * n[3], n2sq = n[2] * n[2], n2cb = n2sq * n[2];
  memset(&t, 0, sizeof(t));
  if (n[3] > 1.e-10) {
    const double fac1 = n[3] - 2 * (1. - n[3]) * log(1. - n[3]);
    const double fac2 = n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3]);
    const double fac3 = -(inv[2] / n3cb) + (inv[3] / n3sq);
    const double fac = 1 - dot22 / (n[2] * n[2]);
    const double k6 = fac2 * inv[2] / (6. * PI * n3sq);
    const double k3 = (2. * fac2 * fac3) + (fac1 * inv[2] / n3sq);
    for (int d = 0; d < nd; d++) v[d] = off[d] * p->esize[d] * p->inv_rad[ic];
    t.S2 = (inv[1] * p->inv_4pir[ic] +
            k6 * (n[2] * fac * fac * fac + 3 * dot22 * fac * fac / n[2] + 4 * dot22 * dot22 * fac / n2cb));
    for (int d = 0; d < nd; d++) t.S2 += v[d] * n[4 + nd + d] * k6 * (fac * fac + 4 * dot22 * fac / n2sq);
    t.S3 = (p->inv_4pirsq[ic] * inv[1] + p->inv_4pir[ic] * n[2] * inv[2] + n[1] * inv[2] +
            (n2sq * fac * fac * fac + 2 * dot22 * fac * fac) * k3 / (12. * PI));
    for (int d = 0; d < nd; d++)
      t.S3 += v[d] * (n[4 + nd + d] * p->inv_4pir[ic] * inv[2] + n[4 + d] * inv[2] +
                      n[2] * n[4 + nd + d] * fac * fac * k3 / (6. * PI));
    t.S0 = 0.0;
    t.S1 = inv[1];
    double dot_nw = 0.0;
    for (int d = 0; d < nd; d++) {
      t.V1[d] = sign[d] * inv[1] * v[d];
      dot_nw += n[4 + nd + d] * v[d];
    }
    for (int d = 0; d < nd; d++)
      t.V2[d] = sign[d] * (-(n[4 + nd + d] * k6) * (fac * fac - 4 * dot22 * fac / n[2] + 4 * dot_nw * fac / n[2]) -
                           (-p->inv_4pir[ic] * inv[1] - n[2] * fac * fac * k6) * v[d]);
  }
  return t;
}

/* d2phi_drb2_theta_rb_FMT4 (src/dft_physics_FMT4.c:201-275) */
static rbs d2_theta_fmt4(const orc_problem *p, const double *n)
{
  rbs t;
  const int nd = p->ndim;
  double inv[5];
  double dot22 = 0.0, dot12 = 0.0;
  for (int d = 0; d < nd; d++) {
    dot22 += n[4 + nd + d] * n[4 + nd + d];
    dot12 += n[4 + d] * n[4 + nd + d];
  }
  inv[0] = (1. - n[3]);
  inv[1] = 1.0 / (1.0 - n[3]);
  inv[2] = inv[1] * inv[1];
  inv[3] = inv[2] * inv[1];
  inv[4] = inv[3] * inv[1];
  const double n3sq = n[3] * n[3], n3cb = n3sq * n[3], n3_4th = n3cb * n[3];
  const double n2sq = n[2] * n[2], n2cb = n2sq * n[2];
  memset(&t, 0, sizeof(t));
  if (n[3] > 1.e-10) {
    const double fac1 = n[3] - 2 * (1. - n[3]) * log(1. - n[3]);
    const double fac2 = n[3] + (1. - n[3]) * (1. - n[3]) * log(1. - n[3]);
    const double fac3 = -(inv[2] / n3cb) + (inv[3] / n3sq);
    const double fac = 1 - dot22 / (n[2] * n[2]);
    const double k3 = (fac1 * inv[2] / n3sq) + (2. * fac2 * fac3);
    t.S2 = (n[1] * inv[2] + (n2sq * fac * fac * fac + 2 * fac * fac * dot22) * k3 / (12 * PI));
    t.S3 = (n[0] * inv[2] + 2 * (n[1] * n[2] - dot12) * inv[3] +
            ((n2cb * fac * fac * fac) / (36. * PI)) *
                (+(((2. * log(1. - n[3]) + 3) * inv[2]) / n3sq) + (4. * fac1 * fac3) +
                 (fac2 * (6. * inv[2] / n3_4th + 6. * inv[4] / n3sq - 8. * inv[3] / n3cb))));
    t.S0 = inv[1];
    t.S1 = n[2] * inv[2];
    for (int d = 0; d < nd; d++) t.V1[d] = -n[4 + nd + d] * inv[2];
    for (int d = 0; d < nd; d++) t.V2[d] = -(n[4 + d] * inv[2] + n[2] * n[4 + nd + d] * fac * fac * k3 / (6. * PI));
  }
  return t;
}

/* FMT2ndDerivDelta_switch / FMT2ndDerivTheta_switch (src/dft_switch_FMT.c:122-152) */
static rbs d2_delta(const orc_problem *p, const double *n, const short *off, const double *sign, int ic)
{
  switch (p->functional) {
    case ORC_FMT2: return d2_delta_fmt2(p, n, off, sign, ic);
    case ORC_FMT3: return d2_delta_fmt3(p, n, off, sign, ic);
    case ORC_FMT4: return d2_delta_fmt4(p, n, off, sign, ic);
    default: return d2_delta_fmt1(p, n, off, sign, ic);
  }
}

static rbs d2_theta(const orc_problem *p, const double *n)
{
  switch (p->functional) {
    case ORC_FMT2: return d2_theta_fmt2(p, n);
    case ORC_FMT3: return d2_theta_fmt3(p, n);
    case ORC_FMT4: return d2_theta_fmt4(p, n);
    default: return d2_theta_fmt1(p, n);
  }
}

/* ---------------------------------------------------------------------------
 * One pass over every row of the fill.  For each row the residual is summed in
 * the reference's order, and every Jacobian entry is handed to `entry`. */
typedef void (*entry_fn)(void *ctx, int iu, long inode, int ju, long jnode, double val);

typedef struct {
  const orc_problem *p;
  const double *x;
  const double *dphi;   /* [nrb][N] */
  double *R;            /* may be NULL */
  entry_fn entry;       /* may be NULL */
  void *ctx;
  int izone, jzone;     /* quadrature zones of the current node's residual and Jacobian */
} pass_t;

/* Stencil[stype][zone][index] (zone 0: the sten_* tables) */
static int zone_sten(const orc_problem *p, int zone, int stype, int index, const short **off, const double **w,
                     const double **hw)
{
  if (zone == 0) {
    *off = p->sten_off[stype][index];
    *w = p->sten_w[stype][index];
    *hw = p->sten_hw[stype][index];
    return p->sten_len[stype][index];
  }
  *off = p->zsten_off[zone][stype][index];
  *w = p->zsten_w[zone][stype][index];
  *hw = p->zsten_hw[zone][stype][index];
  return p->zsten_len[zone][stype][index];
}

/* find_jzone (src/dft_utils.c:67-86) */
static int find_jzone(const orc_problem *p, int izone, long inode)
{
  enum { SAME = 0, ZONE0_FAC2 = 1, ZONES_FAC2 = 2, ALLMOSTCOARSE = 3, SECONDMOSTCOARSE = 4, FIXED_ESIZE = 5 };
  if (p->coarser_jac != SAME && izone < p->nzone - 1) {
    switch (p->coarser_jac) {
      case ZONE0_FAC2: return izone == 0 ? izone + 1 : izone;
      case ZONES_FAC2: return izone + 1;
      case ALLMOSTCOARSE: case FIXED_ESIZE: return p->nzone - 1;
      case SECONDMOSTCOARSE: return p->nzone - 2;
      default: return izone;
    }
  }
  if (p->coarser_jac == SAME) {
    if (p->mesh_coarsening || p->nwall == 0 || !p->zone_flag) return izone;
    return p->zone_flag[inode];
  }
  return izone;
}

static int is_dep_rb(const orc_problem *p, int k)
{
  /* load_rho_bar_s / load_rho_bar_v shortcut (src/dft_fill_FMT.c:215, 303) */
  const int nd = p->ndim;
  return p->single_size && ((k > 1 && k < 4) || k >= 4 + nd);
}

/* resid_and_Jac_sten_fill_sum_Ncomp (src/dft_fill_CLSmf.c:38-171) for the
 * weighted-density and mean-field rows: fac(jcomp, offset) * w * rho_j */
static double sten_sum(pass_t *ps, int stype, int iu, long inode, const int *ijk, int kind, int icomp_pair)
{
  const orc_problem *p = ps->p;
  const long N = orc_nnodes(p);
  const int nd = p->ndim;
  double resid_sum = 0.0;
  int reflect[3];
  for (int jc = 0; jc < p->ncomp; jc++) {
    const int ju = p->first_rho + jc;
    const int jlist = (p->nlists_hw <= 2) ? 0 : jc;
    const int index = (stype == ORC_UATT) ? icomp_pair + p->ncomp * jc : jc;
    const short *off;
    const double *w, *hw;
    /* the weighted-density and mean-field rows take their Jacobian from the residual's zone */
    const int L = zone_sten(p, ps->izone, stype, index, &off, &w, &hw);
    for (int s = 0; s < L; s++) {
      const short *o = off + (long)s * nd;
      double weight = w[s];
      double fac;
      /* prefactor_rho_bar_s / prefactor_rho_bar_v (src/dft_fill_FMT.c:242-251, 330-347) */
      if (kind < 0) fac = 1.0;                           /* mean field: no prefactor */
      else if (kind == 0) fac = p->fac_overlap[jc];      /* n3, n2 */
      else if (kind == 1) fac = p->inv_4pir[jc] * p->fac_overlap[jc];   /* n1 */
      else if (kind == 2) fac = p->inv_4pirsq[jc] * p->fac_overlap[jc]; /* n0 */
      else {
        const int d = (kind - 3) % 3;
        const int v1 = (kind - 3) >= 3;
        fac = (v1 ? p->inv_4pir[jc] : 1.0) * p->fac_overlap[jc] * ((double)o[d] * p->esize[d] * p->inv_rad[jc]);
      }
      const long jn = offset_to_node(p, ijk, o, reflect);
      if (p->hard_surf && jn >= 0 && p->boundary_nodes[(long)jlist * N + jn] != -1)
        weight = hw_weight(p, jlist, hw + (long)s * (1 << nd), jn, reflect);
      /* resid_rho_bar (src/dft_fill_FMT.c:253-272) with constant_boundary (src/dft_utils.c:90) */
      double rho;
      if (jn >= 0 && !p->zero_density[(long)jc * N + jn]) rho = ps->x[(long)ju * N + jn];
      else if (jn == -1) rho = p->rho_b[jc];
      else if (jn == -3) rho = p->rho_b_lbb[jc];
      else if (jn == -4) rho = p->rho_b_rtf[jc];
      else rho = 0.0;
      resid_sum += fac * (weight * rho);
      if (ps->entry && jn >= 0 && !p->zero_density[(long)jc * N + jn])
        ps->entry(ps->ctx, iu, inode, ju, jn, weight * fac);
    }
  }
  return resid_sum;
}

/* load_nonlocal_hs_rosen_rb (src/dft_fill_FMT.c:41-189) */
static double rosen_rb(pass_t *ps, int stype, int iu, long inode, const int *ijk, int ic)
{
  const orc_problem *p = ps->p;
  const long N = orc_nnodes(p);
  const int nd = p->ndim;
  const short *off, *offJ;
  const double *w, *hw, *wJ, *hwJ;   /* the corner weights do not enter these rows */
  const int L = zone_sten(p, ps->izone, stype, ic, &off, &w, &hw);
  const int LJ = zone_sten(p, ps->jzone, stype, ic, &offJ, &wJ, &hwJ);
  const double fo = p->fac_overlap[ic];
  (void)hw;
  (void)hwJ;
  double resid_sum = 0.0;
  int reflect[3];
  for (int s = 0; s < L; s++) {
    const short *o = off + (long)s * nd;
    const double weight = w[s];
    double resid = 0.0;
    const long jn = offset_to_node(p, ijk, o, reflect);
    if (jn >= 0) {
      if (stype == ORC_DELTA) {
        const double *S0 = ps->dphi, *S1 = ps->dphi + N, *S2 = ps->dphi + 2 * N;
        resid = fo * weight * (S0[jn] * p->inv_4pirsq[ic] + S1[jn] * p->inv_4pir[ic] + S2[jn]);
        for (int d = 0; d < nd; d++) {
          const double sign = reflect[d] ? -1.0 : 1.0;
          const double V1 = ps->dphi[(long)(4 + d) * N + jn], V2 = ps->dphi[(long)(4 + nd + d) * N + jn];
          resid -= fo * sign * weight * (V1 * p->inv_4pir[ic] + V2) * (o[d] * p->esize[d] * p->inv_rad[ic]);
        }
      } else {
        resid = fo * weight * ps->dphi[3 * N + jn];
      }
    } else if (jn == -1 || jn == -3 || jn == -4) {   /* :104-126 */
      const double *b = jn == -1 ? p->dphi_bulk : (jn == -3 ? p->dphi_lbb : p->dphi_rtf);
      if (stype == ORC_DELTA) resid = fo * weight * (b[0] * p->inv_4pirsq[ic] + b[1] * p->inv_4pir[ic] + b[2]);
      else resid = fo * weight * b[3];
    } else {
      resid = 0.0;
    }
    resid_sum += resid;
    /* the Jacobian entries come from point s of the Jacobian zone's stencil (:144-156) */
    const short *oj = o;
    double weightJ = weight;
    long jnj = jn;
    if (ps->entry && s < LJ && ps->jzone != ps->izone) {
      oj = offJ + (long)s * nd;
      weightJ = wJ[s];
      jnj = offset_to_node(p, ijk, oj, reflect);
    }
    if (ps->entry && s < LJ && jnj >= 0) {
      double n[10], sign[3];
      for (int d = 0; d < nd; d++) sign[d] = reflect[d] ? -1.0 : 1.0;
      sv_to_n(p, ps->x, jnj, n);
      rbs t;
      if (stype == ORC_DELTA)
        t = d2_delta(p, n, oj, sign, ic);
      else
        t = d2_theta(p, n);
      const int jb = p->first_rb;
      ps->entry(ps->ctx, iu, inode, jb + 0, jnj, fo * weightJ * t.S3);
      ps->entry(ps->ctx, iu, inode, jb + 1, jnj, fo * weightJ * t.S2);
      ps->entry(ps->ctx, iu, inode, jb + 2, jnj, fo * weightJ * t.S1);
      ps->entry(ps->ctx, iu, inode, jb + 3, jnj, fo * weightJ * t.S0);
      for (int d = 0; d < nd; d++) {
        ps->entry(ps->ctx, iu, inode, jb + 4 + d, jnj, fo * weightJ * t.V2[d]);
        ps->entry(ps->ctx, iu, inode, jb + 4 + nd + d, jnj, fo * weightJ * t.V1[d]);
      }
    }
  }
  return resid_sum;
}

/* constant_boundary (src/dft_utils.c:89-110) for the unknowns of these problems */
static double coarse_value(const orc_problem *p, int iu, long jn)
{
  if (iu >= p->first_rho && iu < p->first_rho + p->ncomp) {
    const int ic = iu - p->first_rho;
    if (jn == -1) return p->rho_b[ic];
    if (jn == -3) return p->rho_b_lbb[ic];
    if (jn == -4) return p->rho_b_rtf[ic];
    return 0.0;
  }
  if (iu >= p->first_rb && iu < p->first_rb + 4 + 2 * p->ndim) {
    const int k = iu - p->first_rb;
    if (jn == -1) return p->rhobar_bc[k];
    if (jn == -3) return p->rhobar_lbb[k];
    if (jn == -4) return p->rhobar_rtf[k];
  }
  return 0.0;   /* inside a wall; (the reference leaves mean-field boundary values undefined) */
}

/* locate_neighbor_unks + load_coarse_variable (src/dft_fill_coarse.c:86-123): the two neighbours of
 * `node` along its averaging direction, each with weight fac; with two zones a coarsened neighbour is
 * replaced by its own neighbours (half the weight each) */
static void coarse_terms(pass_t *ps, int iu, long row, long node, double fac, double *R)
{
  static const short off_pm[6][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
  const orc_problem *p = ps->p;
  const long N = orc_nnodes(p);
  int ijk[3], reflect[3];
  node_to_ijk(p, node, ijk);
  const int d = -p->zone_flag[node] - 1;
  for (int loop = 0; loop < 2; loop++) {
    const long jn = offset_to_node(p, ijk, off_pm[d + 3 * loop], reflect);
    if (jn >= 0 && p->zone_flag[jn] < 0 && p->zone_flag[jn] >= -3 && p->nzone == 2) {
      coarse_terms(ps, iu, row, jn, 0.5 * fac, R);
    } else if (jn < 0) {
      *R -= fac * coarse_value(p, iu, jn);
    } else {
      *R -= fac * ps->x[(long)iu * N + jn];
      if (ps->entry) ps->entry(ps->ctx, iu, row, iu, jn, -fac);
    }
  }
}

/* the fill reads Mesh_coarsen_flag with Mesh_coarsening on and walls present, or with L1D_bc
 * (src/dft_fill_main.c:120) */
static int coarsened(const orc_problem *p)
{
  return p->zone_flag && ((p->mesh_coarsening && p->nwall > 0) || p->l1d_bc);
}

enum { FLAG_PBELEC = -777, FLAG_BULK = -888, FLAG_1DBC = -999 };

/* a row that averages neighbours or copies the 1-D line (not BULK_ZONE / PB_ZONE nodes) */
static int averaged_flag(int flag) { return flag < 0 && flag != FLAG_BULK && flag != FLAG_PBELEC; }

static void fill_node(pass_t *ps, long inode)
{
  const orc_problem *p = ps->p;
  const long N = orc_nnodes(p);
  const int nd = p->ndim;
  const int nrb = 4 + 2 * nd;
  const double *x = ps->x;
  int ijk[3];
  node_to_ijk(p, inode, ijk);
  /* fill_resid_and_matrix (src/dft_fill_main.c:118-135): the node's zone, or an averaged row */
  const int flag = coarsened(p) ? p->zone_flag[inode] : 0;
  if (flag == FLAG_1DBC) {
    /* load_coarse_node_1dim (src/dft_fill_coarse.c:37-64): x(node) - x(the node on the line through the
     * origin along Grad_dim with the same Grad_dim coordinate), for every unknown */
    int jk[3] = {0, 0, 0};
    jk[p->dim_1dbc] = ijk[p->dim_1dbc];
    const long jn = jk[0] + (long)p->nx[0] * (jk[1] + (long)p->nx[1] * jk[2]);
    for (int iu = 0; iu < p->nunk; iu++) {
      const double R = x[(long)iu * N + inode] - x[(long)iu * N + jn];
      if (ps->entry) {
        ps->entry(ps->ctx, iu, inode, iu, inode, 1.0);
        ps->entry(ps->ctx, iu, inode, iu, jn, -1.0);
      }
      if (ps->R) ps->R[(long)iu * N + inode] = R;
    }
    return;
  }
  if (averaged_flag(flag)) {
    for (int iu = 0; iu < p->nunk; iu++) {   /* load_coarse_node_Ndim (src/dft_fill_coarse.c:66-84) */
      const double fac = (iu >= p->first_rho && iu < p->first_rho + p->ncomp) ? 1.0 : -1.0;
      double R = fac * x[(long)iu * N + inode];
      if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, fac);
      coarse_terms(ps, iu, inode, inode, 0.5 * fac, &R);
      if (ps->R) ps->R[(long)iu * N + inode] = R;
    }
    return;
  }
  ps->izone = flag < 0 ? 0 : flag;
  ps->jzone = find_jzone(p, ps->izone, inode);
  if (ps->jzone < 0) ps->jzone = 0;
  for (int iu = 0; iu < p->nunk; iu++) {
    double R = 0.0;
    const double xi = x[(long)iu * N + inode];
    if (iu >= p->first_rho && iu < p->first_rho + p->ncomp) {
      /* load_euler_lagrange (src/dft_fill_EL.c:38-196) */
      const int ic = iu - p->first_rho;
      const int zero = p->zero_density[(long)ic * N + inode] || p->vext[(long)ic * N + inode] == p->vext_max;
      if (zero) {
        /* fill_zero_value (src/dft_fill_EL.c:224-240) */
        R = xi;
        if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, 1.0);
      } else if (flag == FLAG_BULK) {
        /* fill_bulk_density (src/dft_fill_EL.c:69-80, 265-284) */
        R = log(xi) - log(p->rho_b[ic]);
        if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, 1.0 / xi);
      } else if (flag == FLAG_PBELEC) {
        /* ideal gas, chemical potential without the excess terms, external field; no hard-sphere or
         * attraction terms (src/dft_fill_EL.c:132-161, 405-410) */
        R = log(xi) + (p->interface == 2 ? -p->betamu[ic] : -log(p->rho_b[ic])) + p->vext[(long)ic * N + inode];
        if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, 1.0 / xi);
      } else if (p->interface == 2 && ic == 0 && inode == p->pin_node) {
        /* fill_constant_density (src/dft_fill_EL.c:89-96, 286-305) */
        R = log(xi) - log(p->pin_value);
        if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, 1.0 / xi);
      } else {
        R += log(xi);                                   /* fill_EL_ideal_gas :351-386 */
        if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, 1.0 / xi);
        double mu = 0.0;                                /* fill_EL_chem_pot :388-433 */
        if (p->interface == 2) {
          mu = -p->betamu[ic];                          /* :412-416 */
        } else {
          mu -= log(p->rho_b[ic]);
          mu -= p->betamu_hs_ex[ic];
          if (p->attraction) mu -= p->betamu_att[ic];
        }
        R += mu;
        R += p->vext[(long)ic * N + inode];             /* fill_EL_ext_field :435-444 */
        R += rosen_rb(ps, ORC_DELTA, iu, inode, ijk, ic);
        R += rosen_rb(ps, ORC_THETA, iu, inode, ijk, ic);
        if (p->attraction) {
          if (!p->att_in_a22) {                         /* :144-155 */
            const int ium = p->first_mf + ic;
            R += x[(long)ium * N + inode];
            if (ps->entry) ps->entry(ps->ctx, iu, inode, ium, inode, 1.0);
          } else {                                      /* :156-159 load_mean_field into the EL row */
            R += sten_sum(ps, ORC_UATT, iu, inode, ijk, -1, ic);
          }
        }
      }
    } else if (iu >= p->first_rb && iu < p->first_rb + nrb) {
      const int k = iu - p->first_rb;
      R = -xi;                                          /* load_rho_bar_s/v :204-213, :293-301 */
      if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, -1.0);
      if (is_dep_rb(p, k)) {
        int ju;
        double c;
        if (k == 2) { ju = p->first_rb + 1; c = p->inv_4pir[0]; }
        else if (k == 3) { ju = p->first_rb + 1; c = p->inv_4pirsq[0]; }
        else { ju = p->first_rb + 4 + (k - 4 - nd); c = p->inv_4pir[0]; }
        R += x[(long)ju * N + inode] * c;
        if (ps->entry) ps->entry(ps->ctx, iu, inode, ju, inode, c);
      } else if (k == 0) {
        R += sten_sum(ps, ORC_THETA, iu, inode, ijk, 0, 0);
      } else if (k < 4) {
        R += sten_sum(ps, ORC_DELTA, iu, inode, ijk, k - 1 == 0 ? 0 : k - 1, 0);
      } else {
        const int d = (k - 4) % nd;
        const int v1 = (k - 4) >= nd;
        R += sten_sum(ps, ORC_DELTA, iu, inode, ijk, 3 + d + (v1 ? 3 : 0), 0);
      }
    } else if (p->attraction && !p->att_in_a22 && iu >= p->first_mf && iu < p->first_mf + p->ncomp) {
      /* load_mean_field (src/dft_fill_mf.c:38-63) */
      const int ic = iu - p->first_mf;
      R = -xi;
      if (ps->entry) ps->entry(ps->ctx, iu, inode, iu, inode, -1.0);
      R += sten_sum(ps, ORC_UATT, iu, inode, ijk, -1, ic);
    }
    if (ps->R) ps->R[(long)iu * N + inode] = R;
  }
}

static int run_pass(const orc_problem *p, const double *x, double *R, entry_fn e, void *ctx, long b, long end)
{
  const long N = orc_nnodes(p);
  const int nrb = 4 + 2 * p->ndim;
  double *dphi = (double *)malloc(sizeof(double) * (size_t)nrb * (size_t)N);
  if (!dphi) return -1;
  orc_dphi(p, x, dphi);  /* FMT1stDeriv_switch over every box node (src/dft_switch_FMT.c:68-96) */
  pass_t ps = {p, x, dphi, R, e, ctx, 0, 0};
  for (long i = b; i < end; i++) fill_node(&ps, i);
  free(dphi);
  return 0;
}

int orc_resid(const orc_problem *p, const double *x, double *R)
{
  return run_pass(p, x, R, NULL, NULL, 0, orc_nnodes(p));
}

int orc_resid_rows(const orc_problem *p, const double *x, double *R, long b, long e)
{
  return run_pass(p, x, R, NULL, NULL, b, e);
}

typedef struct { const double *v; double *out; long N; } mv_ctx;

static void jv_entry(void *c, int iu, long in, int ju, long jn, double val)
{
  mv_ctx *m = (mv_ctx *)c;
  m->out[(long)iu * m->N + in] += val * m->v[(long)ju * m->N + jn];
}

static void jtv_entry(void *c, int iu, long in, int ju, long jn, double val)
{
  mv_ctx *m = (mv_ctx *)c;
  m->out[(long)ju * m->N + jn] += val * m->v[(long)iu * m->N + in];
}

int orc_jv(const orc_problem *p, const double *x, const double *v, double *Jv)
{
  const long N = orc_nnodes(p);
  memset(Jv, 0, sizeof(double) * (size_t)p->nunk * (size_t)N);
  mv_ctx m = {v, Jv, N};
  return run_pass(p, x, NULL, jv_entry, &m, 0, N);
}

int orc_jtv(const orc_problem *p, const double *x, const double *w, double *JTw)
{
  const long N = orc_nnodes(p);
  memset(JTw, 0, sizeof(double) * (size_t)p->nunk * (size_t)N);
  mv_ctx m = {w, JTw, N};
  return run_pass(p, x, NULL, jtv_entry, &m, 0, N);
}

/* S v2 = A22 v2 - A21 A11^-1 A12 v2 (src/dft_Schur_Epetra_Operator.cpp:86-119) with
 * A11^-1 = [-I 0; -B -I] (src/dft_HardSphereA11_Epetra_Operator.cpp:176-192),
 * each block product taken from the Jacobian product J v. */
int orc_schur(const orc_problem *p, const double *x, const double *v2, double *Sv2)
{
  if (coarsened(p))
    for (long i = 0; i < orc_nnodes(p); i++)
      if (averaged_flag(p->zone_flag[i])) return -2;
  const long N = orc_nnodes(p);
  const long U = p->nunk;
  const int nrb = 4 + 2 * p->ndim;
  double *a = (double *)calloc((size_t)(U * N), sizeof(double));
  double *b = (double *)calloc((size_t)(U * N), sizeof(double));
  if (!a || !b) { free(a); free(b); return -1; }
  /* [0; v2] -> block-1 rows hold A12 v2, density rows hold A22 v2 */
  for (int c = 0; c < p->ncomp; c++) memcpy(a + (long)(p->first_rho + c) * N, v2 + (long)c * N, sizeof(double) * N);
  orc_jv(p, x, a, b);
  for (int c = 0; c < p->ncomp; c++) memcpy(Sv2 + (long)c * N, b + (long)(p->first_rho + c) * N, sizeof(double) * N);
  /* u1 = A12 v2 on block 1; a <- [u1_ind, 0_dep, 0_density] */
  memset(a, 0, sizeof(double) * (size_t)(U * N));
  for (int iu = 0; iu < U; iu++) {
    const int is_rho = iu >= p->first_rho && iu < p->first_rho + p->ncomp;
    const int is_dep = iu >= p->first_rb && iu < p->first_rb + nrb && is_dep_rb(p, iu - p->first_rb);
    if (!is_rho && !is_dep) memcpy(a + (long)iu * N, b + (long)iu * N, sizeof(double) * N);
  }
  /* B u1_ind on the dependent rows */
  double *c = (double *)calloc((size_t)(U * N), sizeof(double));
  orc_jv(p, x, a, c);
  /* y1 = A11^-1 u1: y_ind = -u_ind, y_dep = -u_dep - B u_ind (u_dep = 0: dependent rows have no density columns) */
  memset(a, 0, sizeof(double) * (size_t)(U * N));
  for (int iu = 0; iu < U; iu++) {
    const int is_rho = iu >= p->first_rho && iu < p->first_rho + p->ncomp;
    if (is_rho) continue;
    const int is_dep = iu >= p->first_rb && iu < p->first_rb + nrb && is_dep_rb(p, iu - p->first_rb);
    for (long i = 0; i < N; i++)
      a[(long)iu * N + i] = is_dep ? (-b[(long)iu * N + i] - c[(long)iu * N + i]) : -b[(long)iu * N + i];
  }
  /* A21 y1 on the density rows */
  orc_jv(p, x, a, c);
  for (int ic = 0; ic < p->ncomp; ic++)
    for (long i = 0; i < N; i++) Sv2[(long)ic * N + i] -= c[(long)(p->first_rho + ic) * N + i];
  free(a); free(b); free(c);
  return 0;
}
