// The reference's linear-problem-manager C ABI (dft_linprobmgr_*, dft_hardsphere_lin_prob_mgr_*)
// served on the GPU: see include/tramonto_legacy.h.
//
// The reference's C fill inserts the residual and the Jacobian one scalar (or one short run) at a
// time.  Inserts go to per-row host lists; finalizeproblemvalues sorts and merges them into CSR;
// setupsolver uploads CSR blocks to the GPU; solve runs GMRES there.  The hard-sphere manager
// solves through the Schur complement as dft_HardSphereLinProbMgr does
// (src/dft_HardSphereLinProbMgr.cpp:345-428): block 1 = independent then dependent non-local
// unknowns, block 2 = densities; A11 = [-I 0; B -I] (dft_HardSphereA11_Epetra_Operator.cpp:130-197,
// checked at set-up), S = A22 - A21 A11^-1 A12, GMRES on S with diag(A22) as left preconditioner (ILU(2) of
// A22 when the caller says A22 is not diagonal, as the reference),
// then x1 = A11^-1 (b1 - A12 x2).  The basic manager runs GMRES on the whole matrix with its
// diagonal as left preconditioner.  GMRES orthogonalises by classical Gram-Schmidt applied twice
// (one batched dot-product kernel per pass) and stops on ||M^-1 r|| <= tol ||M^-1 b||.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#define TGPU_LEGACY_NO_MPI 1   // the communicator is not read: an opaque word here
#include "../../include/tramonto_legacy.h"

namespace {

constexpr int kOk = 0, kErrArg = -1, kErrCuda = -2, kErrState = -3, kErrUnsup = -4, kErrNoconv = -5;
constexpr int kThreads = 256;
thread_local std::string g_err;

int fail(int code, const std::string &msg)
{
  g_err = msg;
  return code;
}

// ---- kernels ----------------------------------------------------------------

// y = alpha * A x + beta * y (beta == 0: y is not read); one warp per row
__global__ void k_spmv(int nrows, const long *__restrict__ rp, const int *__restrict__ ci,
                       const double *__restrict__ va, const double *__restrict__ x, double *__restrict__ y,
                       double alpha, double beta)
{
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long r = warp; r < nrows; r += nwarps) {
    double acc = 0.0;
    for (long k = rp[r] + lane; k < rp[r + 1]; k += 32) acc = fma(va[k], x[ci[k]], acc);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) y[r] = beta == 0.0 ? alpha * acc : fma(alpha, acc, beta * y[r]);
  }
}

__global__ void k_axpby(double *__restrict__ y, double a, const double *__restrict__ x, double b, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

// y <- U^-1 L^-1 y with the incomplete factors of A22 (L unit lower, strict part stored; U upper with its
// diagonal first in each row), level by level in one CTA: the rows of a level depend only on earlier levels
__global__ void __launch_bounds__(1024) k_ilu_solve(int nlev_l, const int *__restrict__ lp, const int *__restrict__ lr,
                                                    const long *__restrict__ Lrp, const int *__restrict__ Lci,
                                                    const double *__restrict__ Lva, int nlev_u,
                                                    const int *__restrict__ up, const int *__restrict__ ur,
                                                    const long *__restrict__ Urp, const int *__restrict__ Uci,
                                                    const double *__restrict__ Uva, double *__restrict__ y)
{
  for (int l = 0; l < nlev_l; l++) {
    for (int q = lp[l] + threadIdx.x; q < lp[l + 1]; q += blockDim.x) {
      const int r = lr[q];
      double v = y[r];
      for (long k = Lrp[r]; k < Lrp[r + 1]; k++) v -= Lva[k] * y[Lci[k]];
      y[r] = v;
    }
    __syncthreads();
  }
  for (int l = 0; l < nlev_u; l++) {
    for (int q = up[l] + threadIdx.x; q < up[l + 1]; q += blockDim.x) {
      const int r = ur[q];
      double v = y[r];
      for (long k = Urp[r] + 1; k < Urp[r + 1]; k++) v -= Uva[k] * y[Uci[k]];
      y[r] = v / Uva[Urp[r]];
    }
    __syncthreads();
  }
}

__global__ void k_divide(double *__restrict__ y, const double *__restrict__ d, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] /= d[i];
}

// partial[j][block] = sum_i V[j][i] w[i] for j < k
__global__ void k_multidot(const double *__restrict__ V, long ld, int k, const double *__restrict__ w, long n,
                           double *__restrict__ partial)
{
  __shared__ double sh[32];
  for (int j = 0; j < k; j++) {
    double s = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
      s = fma(V[(long)j * ld + i], w[i], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
      s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (threadIdx.x == 0) partial[(long)j * gridDim.x + blockIdx.x] = s;
    }
    __syncthreads();
  }
}

// w -= sum_j h[j] V[j]
__global__ void k_multiaxpy(double *__restrict__ w, const double *__restrict__ V, long ld, int k,
                            const double *__restrict__ h, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double s = w[i];
    for (int j = 0; j < k; j++) s -= h[j] * V[(long)j * ld + i];
    w[i] = s;
  }
}

// ---- host side --------------------------------------------------------------

struct DevCsr {
  int nrows = 0;
  long nnz = 0;
  long *rp = nullptr;
  int *ci = nullptr;
  double *va = nullptr;
};

struct HostCsr {
  std::vector<long> rp{0};
  std::vector<int> ci;
  std::vector<double> va;
  void add(int c, double v)
  {
    ci.push_back(c);
    va.push_back(v);
  }
  void end_row() { rp.push_back((long)ci.size()); }
};

struct Mgr {
  bool hardsphere = false;
  int nunk = 0;
  std::vector<int> ind, dep, dens;
  bool a22_diagonal = true;
  std::vector<int> row_gids, col_gids;
  bool have_rows = false, have_cols = false, structure = false;
  int N = 0, Nbox = 0;
  std::vector<int> box_to_own;   // box node -> owned node
  std::vector<std::vector<std::pair<int, double>>> rows;   // row u*N + i: (column j*N + k, value)
  std::vector<double> rhs;
  // merged matrix (after finalizeproblemvalues)
  std::vector<long> rp;
  std::vector<int> ci;
  std::vector<double> va;
  bool values_final = false;
  // device
  int device = 0;
  cudaStream_t s = nullptr;
  DevCsr dJ, dB, dA12, dA21, dA22;
  double *d_prec = nullptr;      // preconditioner diagonal (A22 or J)
  // ILU(2) of a non-diagonal A22 (the reference's Ifpack "ILU", level-of-fill 2,
  // src/dft_A22Matrix_Epetra_Operator.cpp:110-140) and the level sets of its triangular solves
  bool ilu = false;
  DevCsr dL, dU;
  int nlev_l = 0, nlev_u = 0;
  int *d_lp = nullptr, *d_lr = nullptr, *d_up = nullptr, *d_ur = nullptr;
  double *d_x = nullptr, *d_b = nullptr, *d_t1 = nullptr, *d_t2 = nullptr, *d_t3 = nullptr;
  double *d_V = nullptr, *d_partial = nullptr, *d_h = nullptr;
  int kdim = 0;
  long nvec = 0;
  bool uploaded = false;
  // solver
  double tol = 1e-10;
  int max_iter = 500;
  int last_iters = 0;
  double last_relres = 0.0;
  std::vector<double> sol;
  bool have_sol = false;
  // block-1 / block-2 positions of the unknowns (-1 where absent)
  std::vector<int> pos1, pos2;
  int n_ind = 0, n_dep = 0;
};

bool ck(cudaError_t e, std::string *why)
{
  if (e == cudaSuccess) return true;
  *why = cudaGetErrorString(e);
  return false;
}

template <typename T>
T *dalloc(size_t n, std::string *why)
{
  T *p = nullptr;
  if (!ck(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T)), why)) return nullptr;
  return p;
}

void free_csr(DevCsr &d)
{
  cudaFree(d.rp);
  cudaFree(d.ci);
  cudaFree(d.va);
  d = DevCsr{};
}

void free_dev(Mgr *m)
{
  free_csr(m->dJ);
  free_csr(m->dB);
  free_csr(m->dA12);
  free_csr(m->dA21);
  free_csr(m->dA22);
  free_csr(m->dL);
  free_csr(m->dU);
  for (int **p : {&m->d_lp, &m->d_lr, &m->d_up, &m->d_ur}) {
    cudaFree(*p);
    *p = nullptr;
  }
  m->ilu = false;
  for (double **p : {&m->d_prec, &m->d_x, &m->d_b, &m->d_t1, &m->d_t2, &m->d_t3, &m->d_V, &m->d_partial, &m->d_h}) {
    cudaFree(*p);
    *p = nullptr;
  }
  m->uploaded = false;
}

bool upload_csr(const HostCsr &h, DevCsr &d, cudaStream_t s, std::string *why)
{
  d.nrows = (int)h.rp.size() - 1;
  d.nnz = (long)h.ci.size();
  d.rp = dalloc<long>(h.rp.size(), why);
  d.ci = dalloc<int>(h.ci.size(), why);
  d.va = dalloc<double>(h.va.size(), why);
  if (!d.rp || !d.ci || !d.va) return false;
  if (!ck(cudaMemcpyAsync(d.rp, h.rp.data(), h.rp.size() * sizeof(long), cudaMemcpyHostToDevice, s), why)) return false;
  if (d.nnz > 0) {
    if (!ck(cudaMemcpyAsync(d.ci, h.ci.data(), h.ci.size() * sizeof(int), cudaMemcpyHostToDevice, s), why)) return false;
    if (!ck(cudaMemcpyAsync(d.va, h.va.data(), h.va.size() * sizeof(double), cudaMemcpyHostToDevice, s), why))
      return false;
  }
  return ck(cudaStreamSynchronize(s), why);
}

// ILU(p) by levels of fill (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed., Algorithm 10.5): row i of
// A is eliminated with the U rows of its earlier columns in increasing column order; a fill entry gets level
// lev(i,k) + lev(k,j) + 1 and is kept at level <= p (original entries have level 0).  L is unit lower (its strict
// part stored), U upper with the diagonal first in each row.  false on a zero pivot.
bool ilu_levels(const HostCsr &A, int p, HostCsr &L, HostCsr &U)
{
  const int n = (int)A.rp.size() - 1;
  std::vector<std::vector<int>> ulev(n);     // level of each stored U entry
  std::vector<double> w(n, 0.0);
  std::vector<int> lev(n, -1);               // -1: column absent from the working row
  std::vector<int> cols;
  for (int i = 0; i < n; i++) {
    cols.clear();
    for (long k = A.rp[i]; k < A.rp[i + 1]; k++) {
      const int c = A.ci[k];
      if (lev[c] < 0) cols.push_back(c);
      lev[c] = 0;
      w[c] += A.va[k];
    }
    if (lev[i] < 0) {   // keep the diagonal in the pattern
      lev[i] = 0;
      cols.push_back(i);
    }
    std::sort(cols.begin(), cols.end());
    // eliminate the columns below i in increasing order; fill may add columns between the current and i
    for (size_t q = 0; q < cols.size() && cols[q] < i; q++) {
      const int k = cols[q];
      const double piv = U.va[U.rp[k]];
      w[k] /= piv;
      const double f = w[k];
      for (long e = U.rp[k] + 1; e < U.rp[k + 1]; e++) {
        const int j = U.ci[e];
        const int nl = lev[k] + ulev[k][e - U.rp[k]] + 1;
        if (lev[j] < 0) {
          if (nl > p) continue;
          lev[j] = nl;
          w[j] = 0.0;
          cols.insert(std::upper_bound(cols.begin() + q + 1, cols.end(), j), j);
        } else if (nl < lev[j]) {
          lev[j] = nl;
        }
        w[j] -= f * U.va[e];
      }
    }
    if (w[i] == 0.0) return false;
    std::vector<int> &ul = ulev[i];
    U.add(i, w[i]);
    ul.push_back(lev[i]);
    for (int c : cols) {
      if (c < i) L.add(c, w[c]);
      else if (c > i) {
        U.add(c, w[c]);
        ul.push_back(lev[c]);
      }
    }
    L.end_row();
    U.end_row();
    for (int c : cols) {
      w[c] = 0.0;
      lev[c] = -1;
    }
  }
  return true;
}

// level sets of a triangular solve: a row's level is one more than the deepest row it reads (lower: forward
// order; upper: backward order)
void tri_levels(const HostCsr &T, bool lower, std::vector<int> &ptr, std::vector<int> &rows)
{
  const int n = (int)T.rp.size() - 1;
  std::vector<int> lv(n, 0);
  int nl = 0;
  for (int t = 0; t < n; t++) {
    const int r = lower ? t : n - 1 - t;
    int l = 0;
    for (long k = T.rp[r] + (lower ? 0 : 1); k < T.rp[r + 1]; k++) l = std::max(l, lv[T.ci[k]] + 1);
    lv[r] = l;
    nl = std::max(nl, l + 1);
  }
  ptr.assign(nl + 1, 0);
  for (int r = 0; r < n; r++) ptr[lv[r] + 1]++;
  for (int l = 0; l < nl; l++) ptr[l + 1] += ptr[l];
  rows.assign(n, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (int r = 0; r < n; r++) rows[fill[lv[r]]++] = r;
}

void spmv(Mgr *m, const DevCsr &A, const double *x, double *y, double alpha, double beta)
{
  if (A.nrows == 0) return;
  const long warps = A.nrows;
  const int blocks = (int)std::min<long>((warps * 32 + kThreads - 1) / kThreads, 4096);
  k_spmv<<<blocks, kThreads, 0, m->s>>>(A.nrows, A.rp, A.ci, A.va, x, y, alpha, beta);
}

void axpby(Mgr *m, double *y, double a, const double *x, double b, long n)
{
  if (n > 0) k_axpby<<<592, kThreads, 0, m->s>>>(y, a, x, b, n);
}

Mgr *M(void *h)
{
  return static_cast<Mgr *>(h);
}

int check_unknown(Mgr *m, int u, int node, int limit)
{
  if (!m->structure) return fail(kErrState, "insert before dft_linprobmgr_finalizeblockstructure");
  if (u < 0 || u >= m->nunk || node < 0 || node >= limit) return fail(kErrArg, "unknown or node index out of range");
  return kOk;
}

void insert(Mgr *m, int u, int i, int ju, int jbox, double v)
{
  m->rows[(size_t)u * m->N + i].emplace_back(ju * m->N + m->box_to_own[jbox], v);
  m->values_final = false;
  m->uploaded = false;
}

// y = A11^-1 u on block-1 vectors [ind | dep]: y_ind = -u_ind, y_dep = -B u_ind - u_dep
void a11_inverse(Mgr *m, const double *u, double *y)
{
  const long ni = (long)m->n_ind * m->N, nd = (long)m->n_dep * m->N;
  cudaMemcpyAsync(y, u, sizeof(double) * (ni + nd), cudaMemcpyDeviceToDevice, m->s);
  axpby(m, y, 0.0, u, -1.0, ni + nd);                 // y = -u
  if (nd > 0) spmv(m, m->dB, u, y + ni, -1.0, 1.0);    // y_dep -= B u_ind
}

// y2 = S v2 = A22 v2 - A21 A11^-1 A12 v2
void schur(Mgr *m, const double *v2, double *y2)
{
  spmv(m, m->dA12, v2, m->d_t1, 1.0, 0.0);
  a11_inverse(m, m->d_t1, m->d_t2);
  spmv(m, m->dA22, v2, y2, 1.0, 0.0);
  spmv(m, m->dA21, m->d_t2, y2, -1.0, 1.0);
}

// y <- M^-1 y: the incomplete factors of a non-diagonal A22, else the diagonal
void precondition(Mgr *m, double *y)
{
  if (m->ilu)
    k_ilu_solve<<<1, 1024, 0, m->s>>>(m->nlev_l, m->d_lp, m->d_lr, m->dL.rp, m->dL.ci, m->dL.va, m->nlev_u, m->d_up,
                                      m->d_ur, m->dU.rp, m->dU.ci, m->dU.va, y);
  else
    k_divide<<<592, kThreads, 0, m->s>>>(y, m->d_prec, m->nvec);
}

void apply_op(Mgr *m, const double *v, double *y)
{
  if (m->hardsphere) schur(m, v, y);
  else spmv(m, m->dJ, v, y, 1.0, 0.0);
  precondition(m, y);
}

// batched dots h[j] = <V_j, w>, j < k, back on the host
bool multidot(Mgr *m, int k, const double *w, std::vector<double> &h, std::string *why)
{
  const int nb = 240;
  k_multidot<<<nb, kThreads, 0, m->s>>>(m->d_V, m->nvec, k, w, m->nvec, m->d_partial);
  std::vector<double> part((size_t)k * nb);
  if (!ck(cudaMemcpyAsync(part.data(), m->d_partial, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, m->s), why))
    return false;
  if (!ck(cudaStreamSynchronize(m->s), why)) return false;
  h.assign(k, 0.0);
  for (int j = 0; j < k; j++)
    for (int b = 0; b < nb; b++) h[j] += part[(size_t)j * nb + b];
  return true;
}

double norm(Mgr *m, const double *w, std::string *why, bool *ok)
{
  // the dot kernel reads V rows; stage w in the next free Krylov slot's place is not needed: use a 1-row view
  const int nb = 240;
  k_multidot<<<nb, kThreads, 0, m->s>>>(w, m->nvec, 1, w, m->nvec, m->d_partial);
  std::vector<double> part(nb);
  *ok = ck(cudaMemcpyAsync(part.data(), m->d_partial, sizeof(double) * nb, cudaMemcpyDeviceToHost, m->s), why) &&
        ck(cudaStreamSynchronize(m->s), why);
  double s = 0.0;
  for (double v : part) s += v;
  return std::sqrt(s);
}

// GMRES(kdim) on the left-preconditioned operator; x (device) starts at zero, rhs = M^-1 b in d_t3
int gmres(Mgr *m, const double *rhs, double *x)
{
  std::string why;
  bool ok = true;
  const long n = m->nvec;
  cudaMemsetAsync(x, 0, sizeof(double) * n, m->s);
  const double bnorm = norm(m, rhs, &why, &ok);
  if (!ok) return fail(kErrCuda, why);
  m->last_iters = 0;
  m->last_relres = 0.0;
  if (bnorm == 0.0) return kOk;
  const int kdim = m->kdim;
  std::vector<double> H((size_t)(kdim + 1) * kdim), cs(kdim), sn(kdim), g(kdim + 1), h, h2;
  int total = 0;
  double relres = 1.0;
  while (total < m->max_iter) {
    // r = rhs - M^-1 A x
    double *v0 = m->d_V;
    apply_op(m, x, v0);
    axpby(m, v0, 1.0, rhs, -1.0, n);
    const double beta = norm(m, v0, &why, &ok);
    if (!ok) return fail(kErrCuda, why);
    relres = beta / bnorm;
    if (relres <= m->tol) break;
    axpby(m, v0, 0.0, v0, 1.0 / beta, n);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < kdim && total < m->max_iter; j++, total++) {
      double *w = m->d_V + (long)(j + 1) * n;
      apply_op(m, m->d_V + (long)j * n, w);
      for (int pass = 0; pass < 2; pass++) {
        if (!multidot(m, j + 1, w, h2, &why)) return fail(kErrCuda, why);
        if (!ck(cudaMemcpyAsync(m->d_h, h2.data(), sizeof(double) * (j + 1), cudaMemcpyHostToDevice, m->s), &why))
          return fail(kErrCuda, why);
        k_multiaxpy<<<592, kThreads, 0, m->s>>>(w, m->d_V, n, j + 1, m->d_h, n);
        if (pass == 0) h = h2;
        else
          for (int i = 0; i <= j; i++) h[i] += h2[i];
      }
      const double hn = norm(m, w, &why, &ok);
      if (!ok) return fail(kErrCuda, why);
      if (!std::isfinite(hn)) return fail(kErrNoconv, "non-finite Krylov vector");
      if (hn > 0.0) axpby(m, w, 0.0, w, 1.0 / hn, n);
      for (int i = 0; i <= j; i++) H[(size_t)i * kdim + j] = h[i];
      H[(size_t)(j + 1) * kdim + j] = hn;
      for (int i = 0; i < j; i++) {
        const double a = H[(size_t)i * kdim + j], b = H[(size_t)(i + 1) * kdim + j];
        H[(size_t)i * kdim + j] = cs[i] * a + sn[i] * b;
        H[(size_t)(i + 1) * kdim + j] = -sn[i] * a + cs[i] * b;
      }
      const double a = H[(size_t)j * kdim + j], b = H[(size_t)(j + 1) * kdim + j];
      const double r = std::hypot(a, b);
      cs[j] = r == 0.0 ? 1.0 : a / r;
      sn[j] = r == 0.0 ? 0.0 : b / r;
      H[(size_t)j * kdim + j] = r;
      H[(size_t)(j + 1) * kdim + j] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      relres = std::fabs(g[j + 1]) / bnorm;
      if (relres <= m->tol || hn == 0.0) {
        j++;
        total++;
        break;
      }
    }
    // x += V y, H y = g
    std::vector<double> y(j, 0.0);
    for (int i = j - 1; i >= 0; i--) {
      double s = g[i];
      for (int k = i + 1; k < j; k++) s -= H[(size_t)i * kdim + k] * y[k];
      y[i] = s / H[(size_t)i * kdim + i];
    }
    for (double &v : y) v = -v;   // multiaxpy subtracts
    if (j > 0) {
      if (!ck(cudaMemcpyAsync(m->d_h, y.data(), sizeof(double) * j, cudaMemcpyHostToDevice, m->s), &why))
        return fail(kErrCuda, why);
      k_multiaxpy<<<592, kThreads, 0, m->s>>>(x, m->d_V, n, j, m->d_h, n);
    }
    if (relres <= m->tol) break;
  }
  m->last_iters = total;
  m->last_relres = relres;
  if (!ck(cudaStreamSynchronize(m->s), &why)) return fail(kErrCuda, why);
  return relres <= m->tol ? kOk : fail(kErrNoconv, "GMRES reached its iteration cap");
}

int finalize_values(Mgr *m)
{
  if (!m->structure) return fail(kErrState, "dft_linprobmgr_finalizeblockstructure has not been called");
  const long n = (long)m->nunk * m->N;
  m->rp.assign(1, 0);
  m->ci.clear();
  m->va.clear();
  for (long r = 0; r < n; r++) {
    auto &row = m->rows[r];
    std::sort(row.begin(), row.end(), [](const auto &a, const auto &b) { return a.first < b.first; });
    for (size_t k = 0; k < row.size();) {
      const int c = row[k].first;
      double v = 0.0;
      for (; k < row.size() && row[k].first == c; k++) v += row[k].second;
      m->ci.push_back(c);
      m->va.push_back(v);
    }
    m->rp.push_back((long)m->ci.size());
  }
  m->values_final = true;
  return kOk;
}

int setup_solver(Mgr *m)
{
  if (!m->values_final) {
    const int st = finalize_values(m);
    if (st != kOk) return st;
  }
  std::string why;
  if (!m->s && !ck(cudaStreamCreateWithFlags(&m->s, cudaStreamNonBlocking), &why)) return fail(kErrCuda, why);
  free_dev(m);
  const int N = m->N;
  const long n = (long)m->nunk * N;
  HostCsr J, B, A12, A21, A22;
  std::vector<double> prec;
  for (long r = 0; r < n; r++) {
    for (long k = m->rp[r]; k < m->rp[r + 1]; k++) J.add(m->ci[k], m->va[k]);
    J.end_row();
  }
  if (m->hardsphere) {
    const int n1 = (m->n_ind + m->n_dep) * N, n2 = (int)m->dens.size() * N;
    // block rows in block order
    std::vector<int> order1, order2;
    for (int u : m->ind) order1.push_back(u);
    for (int u : m->dep) order1.push_back(u);
    for (int u : m->dens) order2.push_back(u);
    std::vector<char> is_ind(m->nunk, 0), is_dep(m->nunk, 0);
    for (int u : m->ind) is_ind[u] = 1;
    for (int u : m->dep) is_dep[u] = 1;
    for (int bu = 0; bu < (int)order1.size(); bu++) {
      const int u = order1[bu];
      for (int i = 0; i < N; i++) {
        const long r = (long)u * N + i;
        for (long k = m->rp[r]; k < m->rp[r + 1]; k++) {
          const int ju = m->ci[k] / N, j = m->ci[k] % N;
          const double v = m->va[k];
          if (m->pos2[ju] >= 0) {
            A12.add(m->pos2[ju] * N + j, v);
          } else if (ju == u && j == i) {
            if (std::fabs(v + 1.0) > 1e-12) return fail(kErrUnsup, "A11 diagonal is not -1");
          } else if (is_dep[u] && is_ind[ju]) {
            B.add(m->pos1[ju] * N + j, v);
          } else if (v != 0.0) {
            return fail(kErrUnsup, "A11 is not of the form [-I 0; B -I]");
          }
        }
        A12.end_row();
        if (is_dep[u]) B.end_row();
      }
    }
    for (int bu = 0; bu < (int)order2.size(); bu++) {
      const int u = order2[bu];
      for (int i = 0; i < N; i++) {
        const long r = (long)u * N + i;
        double diag = 0.0;
        for (long k = m->rp[r]; k < m->rp[r + 1]; k++) {
          const int ju = m->ci[k] / N, j = m->ci[k] % N;
          if (m->pos2[ju] >= 0) {
            A22.add(m->pos2[ju] * N + j, m->va[k]);
            if (ju == u && j == i) diag = m->va[k];
          } else {
            A21.add(m->pos1[ju] * N + j, m->va[k]);
          }
        }
        A21.end_row();
        A22.end_row();
        if (diag == 0.0) return fail(kErrUnsup, "zero diagonal in A22");
        prec.push_back(diag);
      }
    }
    m->nvec = n2;
    (void)n1;
    if (!upload_csr(B, m->dB, m->s, &why) || !upload_csr(A12, m->dA12, m->s, &why) ||
        !upload_csr(A21, m->dA21, m->s, &why) || !upload_csr(A22, m->dA22, m->s, &why))
      return fail(kErrCuda, why);
    if (!m->a22_diagonal) {   // the reference preconditions a non-diagonal A22 with ILU(2)
      HostCsr L, U;
      if (!ilu_levels(A22, 2, L, U)) return fail(kErrUnsup, "zero pivot in the incomplete factorisation of A22");
      std::vector<int> lp, lr, up, ur;
      tri_levels(L, true, lp, lr);
      tri_levels(U, false, up, ur);
      m->nlev_l = (int)lp.size() - 1;
      m->nlev_u = (int)up.size() - 1;
      m->d_lp = dalloc<int>(lp.size(), &why);
      m->d_lr = dalloc<int>(lr.size(), &why);
      m->d_up = dalloc<int>(up.size(), &why);
      m->d_ur = dalloc<int>(ur.size(), &why);
      if (!upload_csr(L, m->dL, m->s, &why) || !upload_csr(U, m->dU, m->s, &why) || !m->d_lp || !m->d_lr ||
          !m->d_up || !m->d_ur || !ck(cudaMemcpy(m->d_lp, lp.data(), lp.size() * sizeof(int), cudaMemcpyHostToDevice), &why) ||
          !ck(cudaMemcpy(m->d_lr, lr.data(), lr.size() * sizeof(int), cudaMemcpyHostToDevice), &why) ||
          !ck(cudaMemcpy(m->d_up, up.data(), up.size() * sizeof(int), cudaMemcpyHostToDevice), &why) ||
          !ck(cudaMemcpy(m->d_ur, ur.data(), ur.size() * sizeof(int), cudaMemcpyHostToDevice), &why))
        return fail(kErrCuda, why);
      m->ilu = true;
    }
    m->d_t1 = dalloc<double>(n1, &why);
    m->d_t2 = dalloc<double>(n1, &why);
  } else {
    for (long r = 0; r < n; r++) {
      double diag = 0.0;
      for (long k = m->rp[r]; k < m->rp[r + 1]; k++)
        if (m->ci[k] == r) diag = m->va[k];
      if (diag == 0.0) return fail(kErrUnsup, "zero diagonal");
      prec.push_back(diag);
    }
    m->nvec = n;
  }
  if (!upload_csr(J, m->dJ, m->s, &why)) return fail(kErrCuda, why);
  m->kdim = std::max(1, std::min(m->max_iter, 200));
  m->d_prec = dalloc<double>(prec.size(), &why);
  m->d_x = dalloc<double>(n, &why);
  m->d_b = dalloc<double>(n, &why);
  m->d_t3 = dalloc<double>(n, &why);
  m->d_V = dalloc<double>((size_t)(m->kdim + 1) * m->nvec, &why);
  m->d_partial = dalloc<double>((size_t)240 * (m->kdim + 1), &why);
  m->d_h = dalloc<double>(m->kdim + 1, &why);
  if (!m->d_prec || !m->d_x || !m->d_b || !m->d_t3 || !m->d_V || !m->d_partial || !m->d_h ||
      (m->hardsphere && (!m->d_t1 || !m->d_t2)))
    return fail(kErrCuda, "device allocation failed: " + why);
  if (!ck(cudaMemcpyAsync(m->d_prec, prec.data(), sizeof(double) * prec.size(), cudaMemcpyHostToDevice, m->s), &why))
    return fail(kErrCuda, why);
  m->uploaded = true;
  return ck(cudaStreamSynchronize(m->s), &why) ? kOk : fail(kErrCuda, why);
}

int solve(Mgr *m)
{
  if (!m->uploaded) {
    const int st = setup_solver(m);
    if (st != kOk) return st;
  }
  std::string why;
  const int N = m->N;
  const long n = (long)m->nunk * N;
  if (!ck(cudaMemcpyAsync(m->d_b, m->rhs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, m->s), &why))
    return fail(kErrCuda, why);
  int st;
  std::vector<double> x(n, 0.0);
  if (m->hardsphere) {
    // block vectors: b1 in d_t1 ([ind | dep]), b2 in d_t3; positions follow the equation lists
    const long n1 = (long)(m->n_ind + m->n_dep) * N, n2 = m->nvec;
    std::vector<double> b1(n1), b2(n2);
    for (int u = 0; u < m->nunk; u++)
      for (int i = 0; i < N; i++) {
        const double v = m->rhs[(size_t)u * N + i];
        if (m->pos1[u] >= 0) b1[(size_t)m->pos1[u] * N + i] = v;
        else b2[(size_t)m->pos2[u] * N + i] = v;
      }
    double *d_b1 = m->d_b, *d_rhs2 = m->d_t3, *d_x2 = m->d_x;
    if (!ck(cudaMemcpyAsync(d_b1, b1.data(), sizeof(double) * n1, cudaMemcpyHostToDevice, m->s), &why) ||
        !ck(cudaMemcpyAsync(d_rhs2, b2.data(), sizeof(double) * n2, cudaMemcpyHostToDevice, m->s), &why))
      return fail(kErrCuda, why);
    // rhs2 = M^-1 (b2 - A21 A11^-1 b1)
    a11_inverse(m, d_b1, m->d_t2);
    spmv(m, m->dA21, m->d_t2, d_rhs2, -1.0, 1.0);
    precondition(m, d_rhs2);
    st = gmres(m, d_rhs2, d_x2);
    if (st != kOk && st != kErrNoconv) return st;
    // x1 = A11^-1 (b1 - A12 x2)
    spmv(m, m->dA12, d_x2, d_b1, -1.0, 1.0);
    a11_inverse(m, d_b1, m->d_t1);
    std::vector<double> x1(n1), x2(n2);
    if (!ck(cudaMemcpyAsync(x1.data(), m->d_t1, sizeof(double) * n1, cudaMemcpyDeviceToHost, m->s), &why) ||
        !ck(cudaMemcpyAsync(x2.data(), d_x2, sizeof(double) * n2, cudaMemcpyDeviceToHost, m->s), &why) ||
        !ck(cudaStreamSynchronize(m->s), &why))
      return fail(kErrCuda, why);
    for (int u = 0; u < m->nunk; u++)
      for (int i = 0; i < N; i++)
        x[(size_t)u * N + i] = m->pos1[u] >= 0 ? x1[(size_t)m->pos1[u] * N + i] : x2[(size_t)m->pos2[u] * N + i];
  } else {
    k_divide<<<592, kThreads, 0, m->s>>>(m->d_b, m->d_prec, n);
    st = gmres(m, m->d_b, m->d_x);
    if (st != kOk && st != kErrNoconv) return st;
    if (!ck(cudaMemcpyAsync(x.data(), m->d_x, sizeof(double) * n, cudaMemcpyDeviceToHost, m->s), &why) ||
        !ck(cudaStreamSynchronize(m->s), &why))
      return fail(kErrCuda, why);
  }
  m->sol.swap(x);
  m->have_sol = true;
  return st;
}

void *create(int numUnks, bool hardsphere)
{
  if (numUnks <= 0) {
    fail(kErrArg, "numUnks must be positive");
    return nullptr;
  }
  Mgr *m = new Mgr;
  m->hardsphere = hardsphere;
  m->nunk = numUnks;
  if (cudaGetDevice(&m->device) != cudaSuccess) m->device = 0;   // the GPU is first needed by setupsolver
  return m;
}

void destroy(void *h)
{
  Mgr *m = M(h);
  if (!m) return;
  if (m->s) {
    cudaSetDevice(m->device);
    free_dev(m);
    cudaStreamDestroy(m->s);
  }
  delete m;
}

int set_ids(void *h, int numgids, const int *gids, std::vector<int> Mgr::*list)
{
  Mgr *m = M(h);
  if (!m) return fail(kErrArg, "null manager");
  if (!m->hardsphere) return fail(kErrState, "not a hard-sphere manager");
  if (m->structure) return fail(kErrState, "block structure already finalized");
  if (numgids < 0 || (numgids > 0 && !gids)) return fail(kErrArg, "bad id list");
  (m->*list).assign(gids, gids + numgids);
  for (int u : m->*list)
    if (u < 0 || u >= m->nunk) return fail(kErrArg, "equation id out of range");
  return kOk;
}

}  // namespace

extern "C" {

const char *tgpu_legacy_last_error(void) { return g_err.c_str(); }

void *dft_basic_lin_prob_mgr_create(int numUnks, void *, tgpu_legacy_comm) { return create(numUnks, false); }
void *dft_hardsphere_lin_prob_mgr_create(int numUnks, void *, tgpu_legacy_comm) { return create(numUnks, true); }
void *dft_hardsphere_lin_prob_mgr_create_debug(int numUnks, void *, tgpu_legacy_comm) { return create(numUnks, true); }
void dft_hardsphere_lin_prob_mgr_destruct(void *mgr) { destroy(mgr); }
void dft_linprobmgr_destruct(void *mgr) { destroy(mgr); }

int dft_hardsphere_lin_prob_mgr_setindnonlocalequationids(void *mgr, int numgids, int *gids)
{
  return set_ids(mgr, numgids, gids, &Mgr::ind);
}
int dft_hardsphere_lin_prob_mgr_setdepnonlocalequationids(void *mgr, int numgids, int *gids)
{
  return set_ids(mgr, numgids, gids, &Mgr::dep);
}
int dft_hardsphere_lin_prob_mgr_setdensityequationids(void *mgr, int numgids, int *gids)
{
  return set_ids(mgr, numgids, gids, &Mgr::dens);
}
int dft_hardsphere_lin_prob_mgr_seta22blockisdiagonal(void *mgr, int isa22diagonal)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  m->a22_diagonal = isa22diagonal != 0;
  return kOk;
}
int dft_hardsphere_lin_prob_mgr_seta22blockisdiagona(void *mgr, int isa22diagonal)
{
  return dft_hardsphere_lin_prob_mgr_seta22blockisdiagonal(mgr, isa22diagonal);
}

int dft_linprobmgr_setnodalrowmap(void *mgr, int numgids, int *gids)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  if (numgids <= 0 || !gids) return fail(kErrArg, "empty row map");
  m->row_gids.assign(gids, gids + numgids);
  m->have_rows = true;
  return kOk;
}
int dft_linprobmgr_setnodalcolmap(void *mgr, int numgids, int *gids)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  if (numgids <= 0 || !gids) return fail(kErrArg, "empty column map");
  m->col_gids.assign(gids, gids + numgids);
  m->have_cols = true;
  return kOk;
}
int dft_linprobmgr_setcoarsenednodeslist(void *mgr, int numgids, int *)
{
  if (!M(mgr)) return fail(kErrArg, "null manager");
  return numgids == 0 ? kOk : fail(kErrUnsup, "mesh coarsening is not supported");
}

int dft_linprobmgr_finalizeblockstructure(void *mgr)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  if (m->structure) return 1;
  if (!m->have_rows || !m->have_cols) return -1;
  if (m->hardsphere && m->dens.empty()) return -1;
  m->N = (int)m->row_gids.size();
  m->Nbox = (int)m->col_gids.size();
  std::unordered_map<int, int> own;
  for (int i = 0; i < m->N; i++) own[m->row_gids[i]] = i;
  m->box_to_own.assign(m->Nbox, -1);
  for (int k = 0; k < m->Nbox; k++) {
    auto it = own.find(m->col_gids[k]);
    if (it == own.end()) return fail(kErrUnsup, "box node outside the owned nodes (one process per GPU)");
    m->box_to_own[k] = it->second;
  }
  m->pos1.assign(m->nunk, -1);
  m->pos2.assign(m->nunk, -1);
  if (m->hardsphere) {
    int p = 0;
    for (int u : m->ind) m->pos1[u] = p++;
    for (int u : m->dep) m->pos1[u] = p++;
    p = 0;
    for (int u : m->dens) m->pos2[u] = p++;
    m->n_ind = (int)m->ind.size();
    m->n_dep = (int)m->dep.size();
    for (int u = 0; u < m->nunk; u++)
      if ((m->pos1[u] >= 0) == (m->pos2[u] >= 0)) return fail(kErrArg, "each unknown must be in exactly one block");
  }
  m->rows.assign((size_t)m->nunk * m->N, {});
  m->rhs.assign((size_t)m->nunk * m->N, 0.0);
  m->structure = true;
  return kOk;
}

int dft_linprobmgr_initializeproblemvalues(void *mgr)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  if (!m->structure) return fail(kErrState, "dft_linprobmgr_finalizeblockstructure has not been called");
  for (auto &r : m->rows) r.clear();
  std::fill(m->rhs.begin(), m->rhs.end(), 0.0);
  m->values_final = false;
  m->uploaded = false;
  return kOk;
}

int dft_linprobmgr_insertrhsvalue(void *mgr, int iunk, int inode, double value)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  const int st = check_unknown(m, iunk, inode, m->N);
  if (st != kOk) return st;
  m->rhs[(size_t)iunk * m->N + inode] += value;
  return kOk;
}

int dft_linprobmgr_insertonematrixvalue(void *mgr, int iunk, int ownednode, int junk, int boxnode, double value)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  int st = check_unknown(m, iunk, ownednode, m->N);
  if (st == kOk) st = check_unknown(m, junk, boxnode, m->Nbox);
  if (st != kOk) return st;
  insert(m, iunk, ownednode, junk, boxnode, value);
  return kOk;
}

int dft_linprobmgr_insertmultinodematrixvalues(void *mgr, int iunk, int ownednode, int junk, int *boxnodeindices,
                                               double *values, int numentries)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  int st = check_unknown(m, iunk, ownednode, m->N);
  if (st != kOk) return st;
  if (numentries < 0 || (numentries > 0 && (!boxnodeindices || !values))) return fail(kErrArg, "bad entries");
  for (int k = 0; k < numentries; k++) {
    if ((st = check_unknown(m, junk, boxnodeindices[k], m->Nbox)) != kOk) return st;
    insert(m, iunk, ownednode, junk, boxnodeindices[k], values[k]);
  }
  return kOk;
}

int dft_linprobmgr_insertmultiphysicsmatrixvalues(void *mgr, int iunk, int ownednode, int *junkindices, int boxnode,
                                                  double *values, int numentries)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  int st = check_unknown(m, iunk, ownednode, m->N);
  if (st != kOk) return st;
  if (numentries < 0 || (numentries > 0 && (!junkindices || !values))) return fail(kErrArg, "bad entries");
  for (int k = 0; k < numentries; k++) {
    if ((st = check_unknown(m, junkindices[k], boxnode, m->Nbox)) != kOk) return st;
    insert(m, iunk, ownednode, junkindices[k], boxnode, values[k]);
  }
  return kOk;
}

int dft_linprobmgr_finalizeproblemvalues(void *mgr)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  return finalize_values(m);
}

double dft_linprobmgr_getmatrixvalue(void *mgr, int iunk, int ownednode, int junk, int boxnode)
{
  Mgr *m = M(mgr);
  if (!m || check_unknown(m, iunk, ownednode, m->N) != kOk || check_unknown(m, junk, boxnode, m->Nbox) != kOk)
    return 0.0;
  const int c = junk * m->N + m->box_to_own[boxnode];
  double v = 0.0;
  for (auto &e : m->rows[(size_t)iunk * m->N + ownednode])
    if (e.first == c) v += e.second;
  return v;
}

int dft_linprobmgr_setrhs(void *mgr, double **b)
{
  Mgr *m = M(mgr);
  if (!m || !b) return fail(kErrArg, "null argument");
  if (!m->structure) return fail(kErrState, "dft_linprobmgr_finalizeblockstructure has not been called");
  for (int u = 0; u < m->nunk; u++)
    for (int i = 0; i < m->N; i++) m->rhs[(size_t)u * m->N + i] = b[u][i];
  return kOk;
}

int dft_linprobmgr_getrhs(void *mgr, double **b)
{
  Mgr *m = M(mgr);
  if (!m || !b) return fail(kErrArg, "null argument");
  if (!m->structure) return fail(kErrState, "dft_linprobmgr_finalizeblockstructure has not been called");
  for (int u = 0; u < m->nunk; u++)
    for (int i = 0; i < m->N; i++) b[u][i] = m->rhs[(size_t)u * m->N + i];
  return kOk;
}

int dft_linprobmgr_getlhs(void *mgr, double **x)
{
  Mgr *m = M(mgr);
  if (!m || !x) return fail(kErrArg, "null argument");
  if (!m->have_sol) return fail(kErrState, "no solution: call dft_linprobmgr_solve first");
  for (int u = 0; u < m->nunk; u++)
    for (int k = 0; k < m->Nbox; k++) x[u][k] = m->sol[(size_t)u * m->N + m->box_to_own[k]];
  return kOk;
}

int dft_linprobmgr_writeMatrix(void *mgr, char *filename, char *matrixName, char *matrixDescription)
{
  Mgr *m = M(mgr);
  if (!m || !filename) return fail(kErrArg, "null argument");
  if (!m->values_final) {
    const int st = finalize_values(m);
    if (st != kOk) return st;
  }
  FILE *f = std::fopen(filename, "w");
  if (!f) return fail(kErrArg, "cannot open the matrix file");
  const long n = (long)m->nunk * m->N;
  std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n%% %s\n%% %s\n", matrixName ? matrixName : "",
               matrixDescription ? matrixDescription : "");
  std::fprintf(f, "%ld %ld %ld\n", n, n, (long)m->ci.size());
  for (long r = 0; r < n; r++)
    for (long k = m->rp[r]; k < m->rp[r + 1]; k++) std::fprintf(f, "%ld %d %.17g\n", r + 1, m->ci[k] + 1, m->va[k]);
  std::fclose(f);
  return kOk;
}

int dft_linprobmgr_setupsolver(void *mgr)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  cudaSetDevice(m->device);
  return setup_solver(m);
}

int dft_linprobmgr_solve(void *mgr)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  cudaSetDevice(m->device);
  return solve(m);
}

int dft_linprobmgr_applymatrix(void *mgr, double **x, double **b)
{
  Mgr *m = M(mgr);
  if (!m || !x || !b) return fail(kErrArg, "null argument");
  if (!m->values_final) {
    const int st = finalize_values(m);
    if (st != kOk) return st;
  }
  // on the host: a product with the assembled matrix (no GPU state needed)
  std::vector<double> xo((size_t)m->nunk * m->N, 0.0);
  for (int u = 0; u < m->nunk; u++)
    for (int k = 0; k < m->Nbox; k++) xo[(size_t)u * m->N + m->box_to_own[k]] = x[u][k];
  for (int u = 0; u < m->nunk; u++)
    for (int i = 0; i < m->N; i++) {
      const long r = (long)u * m->N + i;
      double s = 0.0;
      for (long k = m->rp[r]; k < m->rp[r + 1]; k++) s += m->va[k] * xo[m->ci[k]];
      b[u][i] = s;
    }
  return kOk;
}

int dft_linprobmgr_importr2c(void *mgr, double **x, double **b)
{
  Mgr *m = M(mgr);
  if (!m || !x || !b) return fail(kErrArg, "null argument");
  if (!m->structure) return fail(kErrState, "dft_linprobmgr_finalizeblockstructure has not been called");
  for (int u = 0; u < m->nunk; u++)
    for (int k = 0; k < m->Nbox; k++) b[u][k] = x[u][m->box_to_own[k]];
  return kOk;
}

int dft_linprobmgr_importsingleunknownr2c(void *mgr, double *x, double *b)
{
  Mgr *m = M(mgr);
  if (!m || !x || !b) return fail(kErrArg, "null argument");
  if (!m->structure) return fail(kErrState, "dft_linprobmgr_finalizeblockstructure has not been called");
  for (int k = 0; k < m->Nbox; k++) b[k] = x[m->box_to_own[k]];
  return kOk;
}

int dft_linprobmgr_importnodalr2c(void *mgr, double *x, double *b)
{
  return dft_linprobmgr_importsingleunknownr2c(mgr, x, b);
}

int tgpu_legacy_set_solver(void *mgr, double tol, int max_iter)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  if (!(tol > 0.0) || max_iter < 1) return fail(kErrArg, "tolerance and iteration cap must be positive");
  m->tol = tol;
  m->max_iter = max_iter;
  m->uploaded = false;
  return kOk;
}

int tgpu_legacy_last_solve(void *mgr, int *iters, double *relres)
{
  Mgr *m = M(mgr);
  if (!m) return fail(kErrArg, "null manager");
  if (iters) *iters = m->last_iters;
  if (relres) *relres = m->last_relres;
  return kOk;
}

}  // extern "C"
