// Recording linear-problem manager for the oracle build of the reference.
//
// The Tramonto C fill hands every residual and Jacobian entry to a C++
// manager through the dft_linprobmgr_* C ABI (reference:
// src/dft_basic_lin_prob_mgr_wrapper.h:44-92,
// src/dft_hardsphere_lin_prob_mgr_wrapper.h:43-58).  The reference's manager
// sits on Trilinos, which is not available here, so this file implements the
// same ABI on plain C++ containers:
//   * it records the rhs (= -residual) and the Jacobian triplets of the last
//     fill, so the oracle harness can read them back (tref_* accessors);
//   * it solves the Newton system with the hard-sphere Schur-complement
//     method of src/dft_HardSphereLinProbMgr.cpp:345-428: block 1 holds the
//     weighted-density (and mean-field) rows, block 2 the density rows,
//     A11 = [-I 0; B -I] is inverted exactly (src/dft_HardSphereA11_Epetra_
//     Operator.cpp:130-197), and restarted GMRES runs on
//     S = A22 - A21 A11^-1 A12 with A22 as left preconditioner.
// This is test infrastructure: it is linked only into oracle/_ref.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "mpi.h"

extern "C" {
// provided by ref_tap.c: the unknown classification that
// linsolver_setup_HSTYPE (src/dft_linsolver_setup.c:182-241) would make.
void tref_classify_unknowns(int *ind, int *nind, int *dep, int *ndep, int *dens, int *ndens);
}

namespace {

struct ParamList {
  int max_iter = 500;
  double tol = 1e-8;
};

struct Csr {
  int n = 0;
  std::vector<int> ptr, col;
  std::vector<double> val;
};

struct Mgr {
  int numUnks = 0;
  int nOwned = 0, nBox = 0, nGlobal = 0;
  std::vector<int> L2G, B2G, G2L;
  std::vector<int> ind, dep, dens;
  bool haveLists = false;
  bool a22Diagonal = true;
  std::vector<char> coarse;              // per global node: rows average the neighbours (block 2)
  ParamList params;
  // values of the current fill
  std::vector<double> rhs;               // [iunk][owned]
  std::vector<long long> cooKey;         // row * ncols + col
  std::vector<double> cooVal;
  Csr A;                                 // assembled after finalize, global-id numbering
  std::vector<double> lhs;               // [iunk][owned], solution of last solve
  int lastIters = 0;
  double lastRelRes = 0.0;
};

Mgr *g_last = nullptr;

inline long long rowId(const Mgr &m, int iunk, int owned) { return (long long)iunk * m.nGlobal + m.L2G[owned]; }
inline long long colId(const Mgr &m, int junk, int box) { return (long long)junk * m.nGlobal + m.B2G[box]; }

void assemble(Mgr &m)
{
  const long long N = (long long)m.numUnks * m.nGlobal;
  std::vector<size_t> order(m.cooKey.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return m.cooKey[a] < m.cooKey[b]; });
  Csr &A = m.A;
  A.n = (int)N;
  A.ptr.assign(N + 1, 0);
  A.col.clear();
  A.val.clear();
  long long prev = -1;
  for (size_t k : order) {
    long long key = m.cooKey[k];
    if (key == prev) {
      A.val.back() += m.cooVal[k];
    } else {
      long long r = key / N;
      A.col.push_back((int)(key % N));
      A.val.push_back(m.cooVal[k]);
      A.ptr[r + 1]++;
      prev = key;
    }
  }
  for (long long r = 0; r < N; ++r) A.ptr[r + 1] += A.ptr[r];
}

// ---- Schur-complement solve -------------------------------------------------

struct Schur {
  const Mgr &m;
  int n1 = 0, n2 = 0;                   // block sizes
  std::vector<int> gid2pos;             // global id -> position in [block1 | block2], -1 if absent
  std::vector<int> pos2gid;
  std::vector<char> isDep;              // per block-1 position
  Csr A11B, A12, A21, A22;              // in block-local numbering
  std::vector<double> a22diag;
  // ILU(0) of A22 when it is not diagonal
  Csr ilu;
  std::vector<int> iluDiag;

  explicit Schur(const Mgr &mm) : m(mm) {}

  void build()
  {
    const int N = m.A.n;
    gid2pos.assign(N, -1);
    std::vector<int> order1, order2;
    for (int u : m.ind) order1.push_back(u);
    for (int u : m.dep) order1.push_back(u);
    for (int u : m.dens) order2.push_back(u);
    // every unknown of a coarsened node belongs to block 2 (src/dft_HardSphereLinProbMgr.cpp:119-158)
    auto isCoarse = [&](int g) { return !m.coarse.empty() && m.coarse[g]; };
    for (int u : order1)
      for (int g = 0; g < m.nGlobal; ++g) {
        if (isCoarse(g)) continue;
        gid2pos[u * m.nGlobal + g] = (int)pos2gid.size(); pos2gid.push_back(u * m.nGlobal + g); isDep.push_back(std::find(m.dep.begin(), m.dep.end(), u) != m.dep.end());
      }
    n1 = (int)pos2gid.size();
    for (int u : order2)
      for (int g = 0; g < m.nGlobal; ++g) {
        if (isCoarse(g)) continue;
        gid2pos[u * m.nGlobal + g] = (int)pos2gid.size(); pos2gid.push_back(u * m.nGlobal + g);
      }
    for (int g = 0; g < m.nGlobal; ++g)
      if (isCoarse(g))
        for (int u = 0; u < m.numUnks; ++u) { gid2pos[u * m.nGlobal + g] = (int)pos2gid.size(); pos2gid.push_back(u * m.nGlobal + g); }
    n2 = (int)pos2gid.size() - n1;
    auto init = [](Csr &c, int rows) { c.n = rows; c.ptr.assign(rows + 1, 0); c.col.clear(); c.val.clear(); };
    init(A11B, n1); init(A12, n1); init(A21, n2); init(A22, n2);
    a22diag.assign(n2, 0.0);
    for (int p = 0; p < n1 + n2; ++p) {
      int r = pos2gid[p];
      for (int k = m.A.ptr[r]; k < m.A.ptr[r + 1]; ++k) {
        int q = gid2pos[m.A.col[k]];
        double v = m.A.val[k];
        if (q < 0) continue;
        if (p < n1 && q < n1) {
          if (isDep[p] && q != p) { A11B.col.push_back(q); A11B.val.push_back(v); A11B.ptr[p + 1]++; }
        } else if (p < n1) {
          A12.col.push_back(q - n1); A12.val.push_back(v); A12.ptr[p + 1]++;
        } else if (q < n1) {
          A21.col.push_back(q); A21.val.push_back(v); A21.ptr[p - n1 + 1]++;
        } else {
          A22.col.push_back(q - n1); A22.val.push_back(v); A22.ptr[p - n1 + 1]++;
          if (q == p) a22diag[p - n1] += v;
        }
      }
    }
    for (Csr *c : {&A11B, &A12, &A21, &A22})
      for (int r = 0; r < c->n; ++r) c->ptr[r + 1] += c->ptr[r];
    if (!m.a22Diagonal) buildIlu0();
  }

  static void spmv(const Csr &c, const double *x, double *y)
  {
    for (int r = 0; r < c.n; ++r) {
      double s = 0.0;
      for (int k = c.ptr[r]; k < c.ptr[r + 1]; ++k) s += c.val[k] * x[c.col[k]];
      y[r] = s;
    }
  }

  void buildIlu0()
  {
    // rows of A22 with sorted columns
    ilu = A22;
    for (int r = 0; r < ilu.n; ++r) {
      std::vector<std::pair<int, double>> row;
      for (int k = ilu.ptr[r]; k < ilu.ptr[r + 1]; ++k) row.push_back({ilu.col[k], ilu.val[k]});
      std::sort(row.begin(), row.end());
      int k = ilu.ptr[r];
      for (auto &e : row) { ilu.col[k] = e.first; ilu.val[k] = e.second; ++k; }
    }
    iluDiag.assign(ilu.n, -1);
    for (int r = 0; r < ilu.n; ++r)
      for (int k = ilu.ptr[r]; k < ilu.ptr[r + 1]; ++k)
        if (ilu.col[k] == r) iluDiag[r] = k;
    std::vector<int> where(ilu.n, -1);
    for (int i = 0; i < ilu.n; ++i) {
      for (int k = ilu.ptr[i]; k < ilu.ptr[i + 1]; ++k) where[ilu.col[k]] = k;
      for (int k = ilu.ptr[i]; k < ilu.ptr[i + 1]; ++k) {
        int j = ilu.col[k];
        if (j >= i) break;
        double piv = ilu.val[iluDiag[j]];
        double lij = ilu.val[k] / piv;
        ilu.val[k] = lij;
        for (int kk = iluDiag[j] + 1; kk < ilu.ptr[j + 1]; ++kk) {
          int c = ilu.col[kk];
          if (where[c] >= 0) ilu.val[where[c]] -= lij * ilu.val[kk];
        }
      }
      for (int k = ilu.ptr[i]; k < ilu.ptr[i + 1]; ++k) where[ilu.col[k]] = -1;
    }
  }

  void precond(const double *x, double *y) const
  {
    if (m.a22Diagonal) {
      for (int i = 0; i < n2; ++i) y[i] = x[i] / a22diag[i];
      return;
    }
    // forward (unit lower) then backward (upper) triangular solves
    for (int i = 0; i < n2; ++i) {
      double s = x[i];
      for (int k = ilu.ptr[i]; k < iluDiag[i]; ++k) s -= ilu.val[k] * y[ilu.col[k]];
      y[i] = s;
    }
    for (int i = n2 - 1; i >= 0; --i) {
      double s = y[i];
      for (int k = iluDiag[i] + 1; k < ilu.ptr[i + 1]; ++k) s -= ilu.val[k] * y[ilu.col[k]];
      y[i] = s / ilu.val[iluDiag[i]];
    }
  }

  // y = A11^-1 x : y_ind = -x_ind ; y_dep = -x_dep - B x
  void a11inv(const double *x, double *y) const
  {
    std::vector<double> bx(n1);
    spmv(A11B, x, bx.data());
    for (int i = 0; i < n1; ++i) y[i] = isDep[i] ? (-x[i] - bx[i]) : -x[i];
  }

  void apply(const double *x2, double *y2) const
  {
    std::vector<double> t1(n1), t2(n1), t3(n2);
    spmv(A12, x2, t1.data());
    a11inv(t1.data(), t2.data());
    spmv(A21, t2.data(), t3.data());
    spmv(A22, x2, y2);
    for (int i = 0; i < n2; ++i) y2[i] -= t3[i];
  }
};

double dot(const std::vector<double> &a, const std::vector<double> &b)
{
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

// Left-preconditioned restarted GMRES, classical Gram-Schmidt with one
// reorthogonalisation pass, stopping on ||M^-1 r|| / ||M^-1 r0|| < tol.
template <class Op, class Prec>
int gmres(int n, const Op &A, const Prec &M, const std::vector<double> &b, std::vector<double> &x,
          int restart, int maxit, double tol, double *relres)
{
  std::vector<double> r(n), w(n), t(n);
  x.assign(n, 0.0);
  M(b.data(), r.data());
  double r0 = std::sqrt(dot(r, r));
  if (r0 == 0.0) { *relres = 0.0; return 0; }
  int it = 0;
  double rel = 1.0;
  while (it < maxit) {
    // r = M^-1 (b - A x)
    A(x.data(), t.data());
    for (int i = 0; i < n; ++i) t[i] = b[i] - t[i];
    M(t.data(), r.data());
    double beta = std::sqrt(dot(r, r));
    rel = beta / r0;
    if (rel < tol) break;
    int m = std::min(restart, maxit - it);
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<std::vector<double>> H(m + 1, std::vector<double>(m, 0.0));
    std::vector<double> cs(m), sn(m), g(m + 1, 0.0);
    for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    g[0] = beta;
    int k = 0;
    for (; k < m; ++k) {
      A(V[k].data(), t.data());
      M(t.data(), w.data());
      for (int pass = 0; pass < 2; ++pass)
        for (int j = 0; j <= k; ++j) {
          double h = dot(w, V[j]);
          H[j][k] += h;
          for (int i = 0; i < n; ++i) w[i] -= h * V[j][i];
        }
      double hn = std::sqrt(dot(w, w));
      H[k + 1][k] = hn;
      if (hn != 0.0) for (int i = 0; i < n; ++i) V[k + 1][i] = w[i] / hn;
      for (int j = 0; j < k; ++j) {
        double a = H[j][k], bb = H[j + 1][k];
        H[j][k] = cs[j] * a + sn[j] * bb;
        H[j + 1][k] = -sn[j] * a + cs[j] * bb;
      }
      double a = H[k][k], bb = H[k + 1][k];
      double den = std::sqrt(a * a + bb * bb);
      cs[k] = den == 0.0 ? 1.0 : a / den;
      sn[k] = den == 0.0 ? 0.0 : bb / den;
      H[k][k] = den;
      H[k + 1][k] = 0.0;
      g[k + 1] = -sn[k] * g[k];
      g[k] = cs[k] * g[k];
      ++it;
      rel = std::fabs(g[k + 1]) / r0;
      if (rel < tol || hn == 0.0) { ++k; break; }
    }
    // back substitution
    std::vector<double> y(k, 0.0);
    for (int i = k - 1; i >= 0; --i) {
      double s = g[i];
      for (int j = i + 1; j < k; ++j) s -= H[i][j] * y[j];
      y[i] = s / H[i][i];
    }
    for (int j = 0; j < k; ++j)
      for (int i = 0; i < n; ++i) x[i] += y[j] * V[j][i];
    if (rel < tol) break;
  }
  *relres = rel;
  return it;
}

int solveSchur(Mgr &m)
{
  if (!m.haveLists) {
    int ni = 0, nd = 0, nr = 0;
    std::vector<int> a(m.numUnks), b(m.numUnks), c(m.numUnks);
    tref_classify_unknowns(a.data(), &ni, b.data(), &nd, c.data(), &nr);
    m.ind.assign(a.begin(), a.begin() + ni);
    m.dep.assign(b.begin(), b.begin() + nd);
    m.dens.assign(c.begin(), c.begin() + nr);
    m.haveLists = true;
  }
  Schur S(m);
  S.build();
  // rhs in block numbering
  std::vector<double> b1(S.n1), b2(S.n2);
  for (int p = 0; p < S.n1 + S.n2; ++p) {
    int gid = S.pos2gid[p];
    int u = gid / m.nGlobal, g = gid % m.nGlobal;
    double v = m.rhs[(size_t)u * m.nOwned + m.G2L[g]];
    if (p < S.n1) b1[p] = v; else b2[p - S.n1] = v;
  }
  // b2S = b2 - A21 A11^-1 b1
  std::vector<double> t1(S.n1), t2(S.n2), b2s(S.n2);
  S.a11inv(b1.data(), t1.data());
  Schur::spmv(S.A21, t1.data(), t2.data());
  for (int i = 0; i < S.n2; ++i) b2s[i] = b2[i] - t2[i];
  std::vector<double> x2;
  auto op = [&](const double *x, double *y) { S.apply(x, y); };
  auto pc = [&](const double *x, double *y) { S.precond(x, y); };
  double rel = 0.0;
  int restart = 500;
  m.lastIters = gmres(S.n2, op, pc, b2s, x2, restart, m.params.max_iter, m.params.tol, &rel);
  m.lastRelRes = rel;
  // x1 = A11^-1 (b1 - A12 x2)
  std::vector<double> y1(S.n1), x1(S.n1);
  Schur::spmv(S.A12, x2.data(), y1.data());
  for (int i = 0; i < S.n1; ++i) y1[i] = b1[i] - y1[i];
  S.a11inv(y1.data(), x1.data());
  m.lhs.assign((size_t)m.numUnks * m.nOwned, 0.0);
  for (int p = 0; p < S.n1 + S.n2; ++p) {
    int gid = S.pos2gid[p];
    int u = gid / m.nGlobal, g = gid % m.nGlobal;
    m.lhs[(size_t)u * m.nOwned + m.G2L[g]] = p < S.n1 ? x1[p] : x2[p - S.n1];
  }
  return 0;
}

Mgr *M(void *h) { return static_cast<Mgr *>(h); }

void *create(int numUnks, void *plist)
{
  Mgr *m = new Mgr;
  m->numUnks = numUnks;
  if (plist) m->params = *static_cast<ParamList *>(plist);
  g_last = m;
  return m;
}

}  // namespace

extern "C" {

// ---- parameter list (src/dft_parameterlist_wrapper.h) ----------------------
void *dft_parameterlist_create() { return new ParamList; }
void dft_parameterlist_destruct(void *p) { delete static_cast<ParamList *>(p); }
void dft_parameterlist_set_int(void *p, char *name, int v)
{
  if (std::string(name) == "Max_iter") static_cast<ParamList *>(p)->max_iter = v;
}
void dft_parameterlist_set_double(void *p, char *name, double v)
{
  if (std::string(name) == "Tol") static_cast<ParamList *>(p)->tol = v;
}
void dft_parameterlist_set_int_array(void *, char *, int *) {}
void dft_parameterlist_set_double_array(void *, char *, double *) {}
void dft_parameterlist_set_all_aztec(void *p, int *options, double *params);
void AZ_defaults(int *options, double *params);

// ---- managers ----------------------------------------------------------------
void *dft_basic_lin_prob_mgr_create(int numUnks, void *plist, MPI_Comm) { return create(numUnks, plist); }
void *dft_hardsphere_lin_prob_mgr_create(int numUnks, void *plist, MPI_Comm) { return create(numUnks, plist); }
void *dft_hardsphere_lin_prob_mgr_create_debug(int numUnks, void *plist, MPI_Comm) { return create(numUnks, plist); }
void dft_hardsphere_lin_prob_mgr_destruct(void *) {}
int dft_hardsphere_lin_prob_mgr_setindnonlocalequationids(void *h, int n, int *ids) { M(h)->ind.assign(ids, ids + n); M(h)->haveLists = true; return 0; }
int dft_hardsphere_lin_prob_mgr_setdepnonlocalequationids(void *h, int n, int *ids) { M(h)->dep.assign(ids, ids + n); return 0; }
int dft_hardsphere_lin_prob_mgr_setdensityequationids(void *h, int n, int *ids) { M(h)->dens.assign(ids, ids + n); return 0; }
int dft_hardsphere_lin_prob_mgr_seta22blockisdiagonal(void *h, int d) { M(h)->a22Diagonal = d != 0; return 0; }

static int unsupported(const char *what)
{
  std::fprintf(stderr, "oracle manager: %s is outside the oracle's scope\n", what);
  std::exit(3);
  return -1;
}
void *dft_poly_lin_prob_mgr_create(int, void *, MPI_Comm) { unsupported("polymer manager"); return nullptr; }
void *dft_poly_lin_prob_mgr_create_debug(int, void *, MPI_Comm) { unsupported("polymer manager"); return nullptr; }
void dft_poly_lin_prob_mgr_destruct(void *) {}
int dft_poly_lin_prob_mgr_setgequationids(void *, int, int *) { return unsupported("polymer manager"); }
int dft_poly_lin_prob_mgr_setginvequationids(void *, int, int *) { return unsupported("polymer manager"); }
int dft_poly_lin_prob_mgr_setcmsequationids(void *, int, int *) { return unsupported("polymer manager"); }
int dft_poly_lin_prob_mgr_setdensityequationids(void *, int, int *) { return unsupported("polymer manager"); }
int dft_poly_lin_prob_mgr_setfieldondensityislinear(void *, int) { return unsupported("polymer manager"); }
int dft_poly_lin_prob_mgr_setpoissonequationids(void *, int, int *) { return unsupported("polymer manager"); }
int NOXLOCA_Solver(double **, double **, double **, int) { return unsupported("NOX/LOCA solver"); }

void dft_linprobmgr_destruct(void *h)
{
  if (g_last == M(h)) return;  // keep the last manager readable for the harness
  delete M(h);
}
int dft_linprobmgr_setnodalrowmap(void *h, int n, int *gids)
{
  Mgr &m = *M(h);
  m.nOwned = n;
  m.L2G.assign(gids, gids + n);
  int mx = 0;
  for (int g : m.L2G) mx = std::max(mx, g + 1);
  m.nGlobal = std::max(m.nGlobal, mx);
  m.G2L.assign(m.nGlobal, -1);
  for (int i = 0; i < n; ++i) m.G2L[m.L2G[i]] = i;
  return 0;
}
int dft_linprobmgr_setnodalcolmap(void *h, int n, int *gids)
{
  Mgr &m = *M(h);
  m.nBox = n;
  m.B2G.assign(gids, gids + n);
  return 0;
}
int dft_linprobmgr_setcoarsenednodeslist(void *h, int n, int *gids)
{
  Mgr &m = *M(h);
  if (n <= 0) return 0;
  m.coarse.assign(m.nGlobal, 0);
  for (int i = 0; i < n; ++i) m.coarse[gids[i]] = 1;
  m.a22Diagonal = false;   // A22 is not diagonal when some nodes are coarsened
  return 0;
}
int dft_linprobmgr_finalizeblockstructure(void *h)
{
  Mgr &m = *M(h);
  m.rhs.assign((size_t)m.numUnks * m.nOwned, 0.0);
  return 0;
}
int dft_linprobmgr_initializeproblemvalues(void *h)
{
  Mgr &m = *M(h);
  std::fill(m.rhs.begin(), m.rhs.end(), 0.0);
  m.cooKey.clear();
  m.cooVal.clear();
  return 0;
}
int dft_linprobmgr_insertrhsvalue(void *h, int iunk, int inode, double v)
{
  Mgr &m = *M(h);
  m.rhs[(size_t)iunk * m.nOwned + inode] += v;
  return 0;
}
int dft_linprobmgr_insertonematrixvalue(void *h, int iunk, int owned, int junk, int box, double v)
{
  Mgr &m = *M(h);
  const long long N = (long long)m.numUnks * m.nGlobal;
  m.cooKey.push_back(rowId(m, iunk, owned) * N + colId(m, junk, box));
  m.cooVal.push_back(v);
  return 0;
}
int dft_linprobmgr_insertmultinodematrixvalues(void *h, int iunk, int owned, int junk, int *boxes, double *v, int n)
{
  for (int i = 0; i < n; ++i) dft_linprobmgr_insertonematrixvalue(h, iunk, owned, junk, boxes[i], v[i]);
  return 0;
}
int dft_linprobmgr_insertmultiphysicsmatrixvalues(void *h, int iunk, int owned, int *junks, int box, double *v, int n)
{
  for (int i = 0; i < n; ++i) dft_linprobmgr_insertonematrixvalue(h, iunk, owned, junks[i], box, v[i]);
  return 0;
}
int dft_linprobmgr_finalizeproblemvalues(void *h)
{
  assemble(*M(h));
  return 0;
}
double dft_linprobmgr_getmatrixvalue(void *h, int iunk, int owned, int junk, int box)
{
  Mgr &m = *M(h);
  long long r = rowId(m, iunk, owned), c = colId(m, junk, box);
  for (int k = m.A.ptr[r]; k < m.A.ptr[r + 1]; ++k)
    if (m.A.col[k] == c) return m.A.val[k];
  return 0.0;
}
int dft_linprobmgr_setrhs(void *h, double **b)
{
  Mgr &m = *M(h);
  for (int u = 0; u < m.numUnks; ++u)
    for (int i = 0; i < m.nOwned; ++i) m.rhs[(size_t)u * m.nOwned + i] = b[u][i];
  return 0;
}
int dft_linprobmgr_getrhs(void *h, double **b)
{
  Mgr &m = *M(h);
  for (int u = 0; u < m.numUnks; ++u)
    for (int i = 0; i < m.nOwned; ++i) b[u][i] = m.rhs[(size_t)u * m.nOwned + i];
  return 0;
}
int dft_linprobmgr_getlhs(void *h, double **x)
{
  Mgr &m = *M(h);
  for (int u = 0; u < m.numUnks; ++u)
    for (int ib = 0; ib < m.nBox; ++ib) x[u][ib] = m.lhs[(size_t)u * m.nOwned + m.G2L[m.B2G[ib]]];
  return 0;
}
int dft_linprobmgr_writeMatrix(void *, char *, char *, char *) { return -1; }
int dft_linprobmgr_setupsolver(void *) { return 0; }
int dft_linprobmgr_solve(void *h)
{
  Mgr &m = *M(h);
  solveSchur(m);
  if (std::getenv("TREF_VERBOSE"))
    std::printf("\t[oracle manager] GMRES iterations %d, relative residual %.3e\n", m.lastIters, m.lastRelRes);
  return 0;
}
int dft_linprobmgr_applymatrix(void *h, double **x, double **b)
{
  Mgr &m = *M(h);
  std::vector<double> xg((size_t)m.numUnks * m.nGlobal, 0.0);
  for (int u = 0; u < m.numUnks; ++u)
    for (int ib = 0; ib < m.nBox; ++ib) xg[(size_t)u * m.nGlobal + m.B2G[ib]] = x[u][ib];
  for (int u = 0; u < m.numUnks; ++u)
    for (int i = 0; i < m.nOwned; ++i) {
      long long r = rowId(m, u, i);
      double s = 0.0;
      for (int k = m.A.ptr[r]; k < m.A.ptr[r + 1]; ++k) s += m.A.val[k] * xg[m.A.col[k]];
      b[u][i] = s;
    }
  return 0;
}
int dft_linprobmgr_importr2c(void *h, double **xo, double **xb)
{
  Mgr &m = *M(h);
  for (int u = 0; u < m.numUnks; ++u)
    for (int ib = 0; ib < m.nBox; ++ib) xb[u][ib] = xo[u][m.G2L[m.B2G[ib]]];
  return 0;
}
int dft_linprobmgr_importsingleunknownr2c(void *h, double *xo, double *xb)
{
  Mgr &m = *M(h);
  for (int ib = 0; ib < m.nBox; ++ib) xb[ib] = xo[m.G2L[m.B2G[ib]]];
  return 0;
}
int dft_linprobmgr_importnodalr2c(void *h, double *xo, double *xb)
{
  return dft_linprobmgr_importsingleunknownr2c(h, xo, xb);
}

// ---- harness accessors --------------------------------------------------------
int tref_mgr_sizes(int *out)
{
  if (!g_last) return -1;
  out[0] = g_last->numUnks;
  out[1] = g_last->nOwned;
  out[2] = g_last->nBox;
  out[3] = g_last->nGlobal;
  out[4] = (int)g_last->A.val.size();
  out[5] = g_last->lastIters;
  return 0;
}
int tref_mgr_rhs(double *out)
{
  if (!g_last) return -1;
  std::memcpy(out, g_last->rhs.data(), g_last->rhs.size() * sizeof(double));
  return 0;
}
// Assembled Jacobian of the last fill in global ids (row/col = unk * nGlobal + global node)
int tref_mgr_matrix(long long *rows, long long *cols, double *vals)
{
  if (!g_last) return -1;
  const Csr &A = g_last->A;
  size_t k = 0;
  for (int r = 0; r < A.n; ++r)
    for (int j = A.ptr[r]; j < A.ptr[r + 1]; ++j, ++k) { rows[k] = r; cols[k] = A.col[j]; vals[k] = A.val[j]; }
  return 0;
}
int tref_mgr_maps(int *l2g, int *b2g)
{
  if (!g_last) return -1;
  std::memcpy(l2g, g_last->L2G.data(), g_last->L2G.size() * sizeof(int));
  std::memcpy(b2g, g_last->B2G.data(), g_last->B2G.size() * sizeof(int));
  return 0;
}

}  // extern "C"

extern "C" void dft_parameterlist_set_all_aztec(void *p, int *options, double *params)
{
  ParamList *pl = static_cast<ParamList *>(p);
  pl->max_iter = options[6];  // AZ_max_iter in the oracle shim's numbering
  pl->tol = params[0];        // AZ_tol
}
extern "C" void AZ_defaults(int *options, double *params)
{
  for (int i = 0; i < 47; ++i) options[i] = 0;  // initialize_Aztec declares int options[47]
  for (int i = 0; i < 30; ++i) params[i] = 0.0;  // and double params[30] (src/dft_mesh.c:3109-3110)
  options[6] = 500;
  params[0] = 1e-6;
}
