// Host side of the C ABI declared in include/tramonto_gpu.h: problem set-up,
// the fill, Jacobian and Schur products, the Schur-complement GMRES and the
// damped Newton loop.  All device work is issued on the handle's stream.
#include <algorithm>
#include <functional>
#include <map>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "tgpu_internal.h"

using tgpu::DevStencil;

namespace {

thread_local std::string g_last_error;

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

void ck(cudaError_t e, const char *what)
{
  if (e != cudaSuccess) throw Error(TGPU_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

template <class F>
int guard(F &&f)
{
  try {
    return f();
  } catch (const Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return TGPU_ERR_ARG;
  }
}

template <class T>
T *dalloc(size_t n)
{
  void *p = nullptr;
  if (n == 0) n = 1;
  ck(cudaMalloc(&p, n * sizeof(T)), "cudaMalloc");
  return static_cast<T *>(p);
}

template <class T>
void dfree(T *&p)
{
  if (p) cudaFree(p);
  p = nullptr;
}

template <class T>
T *upload(const std::vector<T> &h, cudaStream_t s)
{
  T *d = dalloc<T>(h.size());
  if (!h.empty()) ck(cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s), "upload");
  return d;
}

// One-dimensional source map of the padded box: q -> node index (with the
// reflect bit) or a sentinel, following offset_to_node_box (src/dft_mesh_lib.c:203-297).
std::vector<int> build_map(int n, int h, int bcl, int bcr, bool interface)
{
  // bulk beyond the low side (LBB under a phase interface) and beyond the high side (RTF)
  const int blo = tgpu::kSentBulk, bhi = interface ? tgpu::kSentBulkHi : tgpu::kSentBulk;
  std::vector<int> m(n + 2 * h);
  for (int q = 0; q < n + 2 * h; q++) {
    int s = q - h;
    int v;
    if (s < 0) {
      switch (bcl) {
        case TGPU_BC_IN_BULK: v = blo; break;
        case TGPU_BC_IN_WALL: v = tgpu::kSentWall; break;
        case TGPU_BC_REFLECT:
          s = -s;
          if (s >= n) v = bcr == TGPU_BC_IN_BULK ? bhi : (bcr == TGPU_BC_IN_WALL ? tgpu::kSentWall : tgpu::kSentBad);
          else v = s | tgpu::kReflBit;
          break;
        case TGPU_BC_PERIODIC: s += n; v = s >= 0 ? s : tgpu::kSentBad; break;
        default: v = tgpu::kSentBad;
      }
    } else if (s >= n) {
      switch (bcr) {
        case TGPU_BC_IN_BULK: v = bhi; break;
        case TGPU_BC_IN_WALL: v = tgpu::kSentWall; break;
        case TGPU_BC_REFLECT:
          s = 2 * (n - 1) - s;
          if (s < 0) v = bcl == TGPU_BC_IN_BULK ? blo : (bcl == TGPU_BC_IN_WALL ? tgpu::kSentWall : tgpu::kSentBad);
          else v = s | tgpu::kReflBit;
          break;
        case TGPU_BC_PERIODIC: s -= n; v = s < n ? s : tgpu::kSentBad; break;
        default: v = tgpu::kSentBad;
      }
    } else {
      v = s;
    }
    m[q] = v;
  }
  return m;
}

// padding parameter sets (device arrays): bulk constant, reflection sign mask, zero-density component
struct PadParams {
  double *bulk = nullptr;
  int *sign = nullptr, *zc = nullptr;
  int nch = 0;
  std::vector<double> h_bulk;      // host copies: [low side channels][high side channels]
  std::vector<int> h_sign, h_zc;
};

}  // namespace

struct tgpu_pads {
  PadParams rho_res, rho_jac, tr_res, tr_jac;
  PadParams zero_ext;   // transposed sums: zero outside the mesh, no masking, no sign flips
};

namespace {

struct Ctx : tgpu_ctx {
  tgpu_pads pads;
  double *d_ymf = nullptr;
  double *d_b2s = nullptr;
  long n2 = 0;
  // residual arithmetic and the reference state of the refined fill
  int fill_mode = TGPU_FILL_FP64;
  double refine_tau = 1e-2, refine_switch = 1.0;  // change bound for a carried reference; ||R||_2 below which sums are refined
  bool have_ref = false;
  double *d_rho_ref = nullptr, *d_conv_ref = nullptr, *d_chan_ref = nullptr, *d_tr_ref = nullptr;
  double *d_drho = nullptr, *d_dchan = nullptr;
  double *d_newton_x = nullptr;   // device copy of the state for the host-pointer Newton solve
  // ATTInA22Block = 1: the caller's vectors have no mean-field rows (nunk_ext per node); internal scratch
  bool a22 = false;
  int nunk_ext = 0;
  double *d_a22[3] = {nullptr, nullptr, nullptr};
  bool gmres_transpose = false;   // GMRES operator: S (false) or S^T (adjoint solve)
  // adjoint work buffers (allocated on first use)
  double *d_adj_chan = nullptr, *d_adj_pad = nullptr, *d_adj_g = nullptr, *d_adj_v = nullptr, *d_adj_t = nullptr;
  // objectives (Omega_s, Gamma_ex): integration weights and work buffers
  // tensor-core attraction sums: the FP16 slab, whether it exists, whether the current call uses it
  tgpu::TcSlab tcslab{};
  bool tc_ready = false, tc_on = false;
  bool ff_on = false;   // the current fill's 3-D single-channel sums in float-float arithmetic
  std::string tc_why;
  bool have_integ = false;
  tgpu::ObjConst oc{};
  double *d_wf = nullptr, *d_wb = nullptr;
  double *d_obj_gx = nullptr, *d_obj_gv = nullptr, *d_obj_lam = nullptr, *d_obj_R = nullptr;
  // quadrature zones / mesh coarsening: per-node zone (>= 0) or averaging axis (< 0), the stencils of
  // zones >= 1, the averaged rows and the prolongation onto coarsened nodes
  int nzone = 1;
  std::vector<int> h_zone;       // Mesh_coarsen_flag as given (zones, averaging axes, 1-D boundary / bulk / PB flags)
  std::vector<double> h_rb_bulk; // Rhobar_b beyond IN_BULK boundaries: [low side][high side]
  int dim_1dbc = 0;              // L1D_bc: nodes flagged kFlag1dbc copy the line through the origin along it
  std::vector<tgpu::DevStencil> zsten[tgpu::kMaxZone][3];
  int *d_zone = nullptr;         // the stencil zone of every node (BULK/PB nodes 0, averaged rows < 0)
  signed char *d_rowkind = nullptr;   // BULK_ZONE (1) / PB_ZONE (2) Euler-Lagrange rows, when any
  double *d_zbuf = nullptr;      // [nrb + ncomp][N] one zone's sums
  double *d_cbulk = nullptr;     // [2][nunk] value beyond the low / high IN_BULK boundary per unknown
  double *d_cscr = nullptr;      // [nunk][N] prolonged copies
  double *d_cscr2 = nullptr;     // [nunk][N] the adjoint's folded right-hand side
  tgpu::CoarseRows cr{};
  bool coarse() const { return cr.ncoarse > 0; }
  // FP64 FFT stencil sums (TGPU_FILL_FFT): plan, work boxes, which padded channel box 0 holds the spectrum of
  tgpu::FftPlan fft{};
  int fft_state = 0;             // 0 not built, 1 ready, -1 not available for this problem
  bool fft_on = false;
  double2 *d_fbox[3] = {nullptr, nullptr, nullptr};
  long pad_gen = 0, fft_gen = -1;
  int fft_ch = -1;
  int fft_min_points = -1;       // < 0: the cost model decides which stencils take the FFT
  bool fft_plan_ok = false;
  // FP32 FFT sums of the long stencils in FP32 arithmetic: chosen per context by timing against the
  // tensor-core sum (products) and the FP32 slab sum (FP32 fills): 0 undecided, 1 FFT, -1 direct
  float2 *d_fbox32[3] = {nullptr, nullptr, nullptr};
  // spectra of a transposed sum's input channels (each transformed once, summed by one inverse)
  std::vector<double2 *> d_trbox;
  std::vector<float2 *> d_trbox32;
  int fft32_tc = 0, fft32_slab = 0;
  float t32_att[2][2] = {{0.f, 0.f}, {0.f, 0.f}};   // [slab context, tensor-core context][direct, FFT] ms
  long fft32_gen = -1;
  int fft32_ch = -1;
  double *d_dscr = nullptr;      // [4 + 2 ndim][N] outputs of the timing runs that make the choices
  bool spec32_built = false;
  // the channels of the last pad(): the padded box is written only when a direct kernel needs it (FFT sums read
  // the channels through the boundary maps)
  const double *pad_src = nullptr;
  const float *pad_src32 = nullptr;   // FP32 channels of the last pad32() (read through the boundary maps only)
  const PadParams *pad_pp = nullptr;
  bool pad_f32 = false, pad_pending = false;
  // the per-node FMT Hessian scalars of the current state (products of one Newton state share them)
  double *d_hcoef = nullptr;
  // domain flags of the last fill (tgpu::kDomainN3 | tgpu::kDomainRho), set by its local kernels
  unsigned *d_domain = nullptr;
  int hcoef_form = -1;           // the Jacobian form they were made with; -1: stale
  // FP32 storage of the FP32 Schur products whose every stencil sum is an FP32 FFT (3-D, one zone, no hard-wall
  // corrections or coarsened nodes): the sums, channels, transposed sums, -u_MF and the state's Hessian scalars
  // with its weighted densities ([kHessCoef + nrb][N]) in FP32; store32 routes the FFT sums' outputs and inputs
  // there while such a product runs
  bool store32 = false;
  float *d_conv32 = nullptr, *d_chan32 = nullptr, *d_tr32 = nullptr, *d_ymf32 = nullptr, *d_hcoef32 = nullptr;
  double *d_inv32 = nullptr;           // 1/rho of the state's Euler-Lagrange rows, and their kinds (k_row_info32)
  signed char *d_kind32 = nullptr;
  int hcoef32_form = -1;
};

// The geometry lives in one __constant__ block per device; the handle that
// last uploaded it owns it, and any other handle re-uploads before its work.
const tgpu_ctx *g_geom_owner = nullptr;

Ctx *C(tgpu_handle h)
{
  if (!h) throw Error(TGPU_ERR_ARG, "null handle");
  Ctx *c = static_cast<Ctx *>(h);
  if (c->finalized && g_geom_owner != c) {
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    tgpu::upload_geom(c->dg, c->stream);
    g_geom_owner = c;
  }
  return c;
}

void need_final(Ctx *c)
{
  if (!c->finalized) throw Error(TGPU_ERR_STATE, "tgpu_finalize has not been called");
}

// Values the padded boxes take at bulk sentinels: the bulk densities (density channels) and the
// bulk dPhi/dn combinations of the Euler-Lagrange channels (Dphi_Drhobar_b, src/dft_fill_FMT.c:104-127).
// The padded boxes hold both sides' values, [low side channels][high side channels]: the same uniform bulk
// twice, or the LBB and RTF states of a phase interface (Rho_b_LBB/_RTF, Dphi_Drhobar_LBB/_RTF).
std::vector<double> bulk_values_rho(const tgpu_geometry &g)
{
  std::vector<double> v;
  for (int side = 0; side < 2; side++)
    for (int jc = 0; jc < g.ncomp; jc++)
      v.push_back(g.interface == 2 ? (side ? g.rho_b_rtf[jc] : g.rho_b_lbb[jc]) : g.rho_b[jc]);
  return v;
}

std::vector<double> bulk_values_tr(const tgpu_geometry &g)
{
  std::vector<double> v;
  for (int side = 0; side < 2; side++)
    for (int ic = 0; ic < g.ncomp; ic++) {
      const double f = g.fac_overlap[ic];
      const double *b = g.interface == 2 ? (side ? g.dphi_rtf : g.dphi_lbb) : g.dphi_bulk;
      v.push_back(f * (b[0] * g.inv_4pirsq[ic] + b[1] * g.inv_4pir[ic] + b[2]));
      for (int d = 0; d < g.ndim; d++) v.push_back(0.0);
      v.push_back(f * b[3]);
    }
  return v;
}

// bulk: [low side][high side] (2 nch values), or nch values used for both sides
PadParams make_pad(const std::vector<double> &bulk, const std::vector<int> &sign, const std::vector<int> &zc,
                   cudaStream_t s)
{
  PadParams p;
  p.nch = (int)sign.size();
  std::vector<double> b2(bulk);
  if ((int)b2.size() == p.nch) b2.insert(b2.end(), bulk.begin(), bulk.end());
  p.bulk = upload(b2, s);
  p.sign = upload(sign, s);
  p.zc = upload(zc, s);
  p.h_bulk = b2;
  p.h_sign = sign;
  p.h_zc = zc;
  return p;
}

void free_pad(PadParams &p)
{
  dfree(p.bulk);
  dfree(p.sign);
  dfree(p.zc);
}

long nnodes(const tgpu_geometry &g)
{
  long n = 1;
  for (int d = 0; d < g.ndim; d++) n *= g.nx[d];
  return n;
}

// ---- stencil passes --------------------------------------------------------

// Pad `nch` channels of `src` with parameter set `pp`, into the FP32 or the FP64 padded box: recorded here, written
// by materialize() before the first direct kernel that reads the box (src must stay unchanged until then)
void pad(Ctx *c, const double *src, const PadParams &pp, bool f32)
{
  c->pad_gen++;   // the padded channels change: a cached spectrum of them is stale
  c->pad_src = src;
  c->pad_src32 = nullptr;
  c->pad_pp = &pp;
  c->pad_f32 = f32;
  c->pad_pending = true;
}

// FP32 channels for the FP32 FFT sums, which read them through the boundary maps (no padded box is made)
void pad32(Ctx *c, const float *src, const PadParams &pp)
{
  c->pad_gen++;
  c->pad_src = nullptr;
  c->pad_src32 = src;
  c->pad_pp = &pp;
  c->pad_f32 = true;
  c->pad_pending = false;
}

void materialize(Ctx *c)
{
  if (c->pad_src32) throw Error(TGPU_ERR_STATE, "an FP32-storage product needs a direct stencil sum");
  if (!c->pad_pending) return;
  const PadParams &pp = *c->pad_pp;
  if (!c->pad_f32)
    tgpu::launch_pad<double>(c->pad_src, c->d_pad, pp.nch, pp.bulk, pp.sign, pp.zc, c->d_zero, false, c->stream);
  else
    tgpu::launch_pad<float>(c->pad_src, c->d_pad32, pp.nch, pp.bulk, pp.sign, pp.zc, c->d_zero, false, c->stream);
  c->stats.kernel_launches++;
  c->pad_pending = false;
}

// channel ch of the last pad() as the FFT's mapped source
tgpu::MapSrc map_src(const Ctx *c, int ch)
{
  const tgpu::DevGeom &g = c->dg;
  const PadParams &pp = *c->pad_pp;
  tgpu::MapSrc m;
  if (c->pad_src32) m.src32 = c->pad_src32 + (long)ch * g.N;
  else m.src = c->pad_src + (long)ch * g.N;
  m.ndim = g.ndim;
  for (int d = 0; d < 3; d++) {
    m.nx[d] = g.nx[d];
    m.map[d] = g.map[d];
  }
  m.bulk_lo = pp.h_bulk[ch];
  m.bulk_hi = pp.h_bulk[pp.nch + ch];
  m.signmask = pp.h_sign[ch];
  m.zc = pp.h_zc[ch];
  m.zero = c->d_zero;
  m.N = g.N;
  return m;
}

// ---- FP64 stencil sums by FFT ----------------------------------------------------

// Which stencils take the FFT in TGPU_FILL_FFT (and TGPU_FP64_FFT products): those whose direct float-float sums
// (measured on GB300: ~5.4e-13 s per term and output) cost more than the transforms (one per coefficient plus the
// field's; measured ~8e-12 s per half-spectrum point and log2 of the box: 0.26 ms for the 180 x 128 x 128 box of
// the 128^3 workload), unless tgpu_set_fft_threshold fixed a length.  At 128^3 every stencil qualifies: the
// attraction stencil (7e4 points), theta (1015) and delta (844 points, four outputs).
bool fft_worth(const Ctx *c, const DevStencil &st, int nq)
{
  if (c->fft_min_points >= 0) return st.L >= c->fft_min_points;
  const double NR = (double)c->fft.NR, NH = (double)c->fft.NH;
  return (double)st.L * (double)c->dg.N * nq * 5.4e-13 > (nq + 1) * NH * std::log2(NR) * 8.0e-12;
}

// the plan's geometry: padded extents, mesh, reach, and the dimensions periodic at both ends (left unpadded)
void plan_geometry_args(const Ctx *c, int P[3], int nx[3], int h[3], int per[3])
{
  const tgpu::DevGeom &dg = c->dg;
  for (int d = 0; d < 3; d++) {
    P[d] = dg.P[d];
    nx[d] = dg.nx[d];
    h[d] = dg.h[d];
    per[d] = d < dg.ndim && c->g.bc[d][0] == TGPU_BC_PERIODIC && c->g.bc[d][1] == TGPU_BC_PERIODIC;
  }
}

// spectrum (FP64 half spectrum) of coefficient q of a stencil's forward (side 0) or transposed (side 1) table
void kernel_spectrum(Ctx *c, const DevStencil &st, int side, int q, double *rbox, double2 *spec)
{
  const double *coef = side == 0 ? st.d_coef_fwd : st.d_coef_tr;
  const int nq = side == 0 ? st.nout_fwd : st.nin_tr;
  tgpu::launch_fft_kernel_box(st.d_off, coef, st.L, nq, q, rbox, c->fft, c->stream);
  tgpu::rfft_forward_box(rbox, spec, c->fft, c->stream);
}

// plan, work boxes and the spectra of every zone-0 stencil coefficient (forward outputs, transpose inputs)
void ensure_fft(Ctx *c)
{
  if (c->fft_state != 0) return;
  c->fft_state = -1;
  const tgpu::DevGeom &dg = c->dg;
  if (dg.ndim != 3) return;
  int P[3], nx[3], h[3], per[3];
  plan_geometry_args(c, P, nx, h, per);
  if (!tgpu::fft_make_plan(c->fft, P, nx, h, per, dg.ndim, c->stream)) return;
  c->fft_plan_ok = true;
  const long NH = c->fft.NH, NR = c->fft.NR;
  // device memory: three work spectra and one spectrum per stencil coefficient
  size_t nspec = 0;
  for (int t = 0; t < 3; t++)
    for (auto &st : c->sten[t])
      if (st.L > 0 && fft_worth(c, st, st.nout_fwd)) nspec += st.nout_fwd + (st.d_coef_tr ? st.nin_tr : 0);
  if (nspec == 0) return;
  size_t free_b = 0, total_b = 0;
  ck(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  if ((nspec + 3) * (size_t)NH * sizeof(double2) + (size_t)NR * sizeof(double) > free_b / 2) return;
  for (auto &b : c->d_fbox) b = dalloc<double2>((size_t)NH);
  double *rbox = dalloc<double>((size_t)NR);
  for (int t = 0; t < 3; t++)
    for (auto &st : c->sten[t]) {
      if (st.L == 0 || !fft_worth(c, st, st.nout_fwd)) continue;
      for (int side = 0; side < 2; side++) {
        const double *coef = side == 0 ? st.d_coef_fwd : st.d_coef_tr;
        const int nq = side == 0 ? st.nout_fwd : st.nin_tr;
        if (!coef) continue;
        for (int q = 0; q < nq; q++) {
          double2 *k = dalloc<double2>((size_t)NH);
          kernel_spectrum(c, st, side, q, rbox, k);
          (side == 0 ? st.spec_fwd : st.spec_tr).push_back(k);
        }
      }
    }
  ck(cudaStreamSynchronize(c->stream), "sync");
  dfree(rbox);
  c->fft_state = 1;
}

// spectrum of padded FP64 channel ch in box 0 (kept while the padded channels stay the same)
const double2 *fft_channel(Ctx *c, int ch)
{
  if (c->fft_gen == c->pad_gen && c->fft_ch == ch) return c->d_fbox[0];
  tgpu::rfft_forward_mapped(map_src(c, ch), c->d_fbox[0], c->fft, c->stream);
  c->stats.kernel_launches += 3;
  c->fft_gen = c->pad_gen;
  c->fft_ch = ch;
  return c->d_fbox[0];
}

// FP32 spectra of the stencils (from FP64 ones) and three FP32 work spectra
bool prepare_spec32(Ctx *c)
{
  if (c->spec32_built) return true;
  ensure_fft(c);
  if (!c->fft_plan_ok) return false;
  const long NH = c->fft.NH, NR = c->fft.NR;
  double2 *tmp = dalloc<double2>((size_t)NH);
  double *rbox = dalloc<double>((size_t)NR);
  for (int t = 0; t < 3; t++)
    for (auto &st : c->sten[t]) {
      if (st.L == 0 || !st.spec_fwd32.empty()) continue;
      for (int side = 0; side < 2; side++) {
        const double *coef = side == 0 ? st.d_coef_fwd : st.d_coef_tr;
        const int nq = side == 0 ? st.nout_fwd : st.nin_tr;
        if (!coef) continue;
        for (int q = 0; q < nq; q++) {
          kernel_spectrum(c, st, side, q, rbox, tmp);
          float2 *k = dalloc<float2>((size_t)NH);
          tgpu::launch_to_float2(tmp, k, NH, c->stream);
          (side == 0 ? st.spec_fwd32 : st.spec_tr32).push_back(k);
        }
      }
    }
  ck(cudaStreamSynchronize(c->stream), "sync");
  dfree(tmp);
  dfree(rbox);
  for (auto &b : c->d_fbox32)
    if (!b) b = dalloc<float2>((size_t)NH);
  c->spec32_built = true;
  return true;
}

// spectrum of padded FP32 channel ch in FP32 box 0 (kept while the padded channels stay the same)
const float2 *fft_channel32(Ctx *c, int ch)
{
  if (c->fft32_gen == c->pad_gen && c->fft32_ch == ch) return c->d_fbox32[0];
  tgpu::rfft_forward_mapped(map_src(c, ch), c->d_fbox32[0], c->fft, c->stream);
  c->stats.kernel_launches += 3;
  c->fft32_gen = c->pad_gen;
  c->fft32_ch = ch;
  return c->d_fbox32[0];
}

// spectrum of channel ch of the last pad() into box (not cached)
template <class C>
const C *channel_into(Ctx *c, int ch, C *box)
{
  tgpu::rfft_forward_mapped(map_src(c, ch), box, c->fft, c->stream);
  c->stats.kernel_launches += 3;
  return box;
}

template <class C>
std::vector<C *> &tr_boxes(Ctx *c);
template <>
std::vector<double2 *> &tr_boxes<double2>(Ctx *c) { return c->d_trbox; }
template <>
std::vector<float2 *> &tr_boxes<float2>(Ctx *c) { return c->d_trbox32; }

// transposed sum: out += the inverse of sum_t (spectrum of channel chs[t]) * kern[t], over channels of the last
// pad(), in one inverse transform
template <class C>
void fft_tr_sum(Ctx *c, const int *chs, const C *const *kern, int n, double *out)
{
  if (n > tgpu::fft_max_terms()) throw Error(TGPU_ERR_UNSUPPORTED, "too many channels for one FFT transposed sum");
  std::vector<C *> &boxes = tr_boxes<C>(c);
  while ((int)boxes.size() < n) boxes.push_back(dalloc<C>((size_t)c->fft.NH));
  std::vector<const C *> a(n);
  {   // the channels' spectra in one launch per pass
    std::vector<tgpu::MapSrc> ms(n);
    for (int t = 0; t < n; t++) ms[t] = map_src(c, chs[t]);
    tgpu::rfft_forward_mapped_batch(ms.data(), n, boxes.data(), c->fft, c->stream);
    c->stats.kernel_launches += 3;
    for (int t = 0; t < n; t++) a[t] = boxes[t];
  }
  C *work = std::is_same<C, float2>::value ? (C *)c->d_fbox32[2] : (C *)c->d_fbox[2];
  if constexpr (std::is_same<C, float2>::value) {
    if (c->store32) {   // the FP32 shadow of the transposed-sum output
      tgpu::rfft_inverse_products(a.data(), kern, n, work, c->fft, 1.0 / (double)c->fft.NR,
                                  c->d_tr32 + (out - c->d_tr), true, c->stream);
      c->stats.kernel_launches += 3;
      c->stats.conv_launches++;
      return;
    }
  }
  tgpu::rfft_inverse_products(a.data(), kern, n, work, c->fft, 1.0 / (double)c->fft.NR, out, true, c->stream);
  c->stats.kernel_launches += 3;
  c->stats.conv_launches++;
}

// FFT sums with the stencil's spectra `spec` (FP32 or FP64): forward, one inverse per output of the field's spectrum
// times the output's kernel; transposed, one inverse of the channels' spectra times their kernels
template <class C>
void fft_conv_impl(Ctx *c, int ch0, int nin, const std::vector<C *> &spec, bool tr, double *const *outs, int nout,
                   C *const *fbox, const C *(*channel)(Ctx *, int))
{
  if (!tr) {
    const C *F = channel(c, ch0);
    {   // every output in one launch per pass
      std::vector<C *> &work = tr_boxes<C>(c);
      while ((int)work.size() < nout) work.push_back(dalloc<C>((size_t)c->fft.NH));
      tgpu::rfft_inverse_batch(F, spec.data(), nout, work.data(), c->fft, 1.0 / (double)c->fft.NR, outs, true,
                               c->stream);
      c->stats.kernel_launches += 3;
    }
    c->stats.conv_launches++;
  } else {
    std::vector<int> chs(nin);
    std::vector<const C *> k(nin);
    for (int t = 0; t < nin; t++) {
      chs[t] = ch0 + t;
      k[t] = spec[t];
    }
    fft_tr_sum<C>(c, chs.data(), k.data(), nin, outs[0]);
  }
}

void fft_conv32(Ctx *c, int ch0, int nin, const DevStencil &st, bool tr, double *const *outs, int nout)
{
  fft_conv_impl<float2>(c, ch0, nin, tr ? st.spec_tr32 : st.spec_fwd32, tr, outs, nout, c->d_fbox32, fft_channel32);
}

// FP32 FFT for this sum: the attraction stencil by its context's choice (tensor-core products or FP32 slab
// sums), the short stencils by their own (decide_fft32_sten)
bool use_fft32(const Ctx *c, const DevStencil &st, bool tr, int nin, int nout)
{
  if (tr) return (int)st.spec_tr32.size() == nin && nout == 1 && st.fft32_tr == 1;
  if ((int)st.spec_fwd32.size() != nout || nin != 1) return false;
  if (&st >= c->sten[TGPU_STEN_UATT].data() && &st < c->sten[TGPU_STEN_UATT].data() + c->sten[TGPU_STEN_UATT].size())
    return c->tc_on ? c->fft32_tc == 1 : c->fft32_slab == 1;
  return st.fft32_fwd == 1;
}

void fft_conv(Ctx *c, int ch0, int nin, const DevStencil &st, bool tr, double *const *outs, int nout)
{
  fft_conv_impl<double2>(c, ch0, nin, tr ? st.spec_tr : st.spec_fwd, tr, outs, nout, c->d_fbox, fft_channel);
}

void conv(Ctx *c, int ch0, int nin, const DevStencil &st, bool tr, double *const *outs, int nout, bool f32)
{
  const long NP = c->dg.NP;
  if (!f32 && c->fft_on && c->fft_state == 1 && (tr ? (int)st.spec_tr.size() == nin && nout == 1
                                                      : (int)st.spec_fwd.size() == nout && nin == 1)) {
    fft_conv(c, ch0, nin, st, tr, outs, nout);
    return;
  }
  if (f32 && c->spec32_built && use_fft32(c, st, tr, nin, nout)) {
    fft_conv32(c, ch0, nin, st, tr, outs, nout);
    return;
  }
  materialize(c);   // the direct kernels below read the padded box
  if (f32 && c->tc_on && !tr && nin == 1 && nout == 1 && st.tc.nplanes > 0) {
    tgpu::launch_sten_tc(c->d_pad32 + (long)ch0 * NP, c->dg, c->tcslab, st.tc, outs[0], true, c->stream);
    c->stats.conv_launches++;
    c->stats.kernel_launches += 4;
    return;
  }
  if (f32 && (nin > 1 || nout > 1)) {
    const DevStencil::Lines &ln = tr ? st.lines_tr : st.lines_fwd;
    if (ln.nplanes > 0 && ln.mc_ok && ln.ncoef == nin * nout) {
      const long total = (long)c->nch_max * NP + 64 - (long)ch0 * NP;
      if (tgpu::launch_conv_slab_mc(c->d_pad32 + (long)ch0 * NP, NP, total, nin, ln.d_planes, ln.nplanes,
                                    ln.d_lines, ln.d_w, ln.wstride, outs, nout, ln.pitch, ln.ncols, ln.max_rows,
                                    ln.max_lines, ln.max_w, c->dg.nx[0], c->dg.nx[1], c->dg.nx[2], c->stream)) {
        c->stats.conv_launches++;
        c->stats.kernel_launches++;
        return;
      }
    }
  }
  if (f32 && nin == 1 && nout == 1) {
    const DevStencil::Lines &ln = tr ? st.lines_tr : st.lines_fwd;
    if (ln.nplanes > 0 && ln.ncoef == 1) {
      // the slab loads stay inside this channel and its successors (the buffer has one spare row)
      const long total = (long)c->nch_max * NP + 64 - (long)ch0 * NP;
      tgpu::launch_conv_slab(c->d_pad32 + (long)ch0 * NP, total, ln.d_planes, ln.nplanes, ln.d_lines, ln.d_w,
                             outs[0], ln.pitch, ln.ncols, ln.max_rows, ln.max_lines, ln.max_w, c->dg.nx[0],
                             c->dg.nx[1], c->dg.nx[2], c->stream);
      c->stats.conv_launches++;
      c->stats.kernel_launches++;
      return;
    }
  }
  if (!f32 && c->ff_on && (nin > 1 || nout > 1)) {
    // multi-channel sums as one single-coefficient float-float sum per channel
    const std::vector<DevStencil::Lines> &tabs = tr ? st.ff_tr : st.ff_fwd;
    bool ok = (int)tabs.size() == std::max(nin, nout) && (nin == 1 || nout == 1);
    for (const auto &ln : tabs) ok = ok && ln.nplanes > 0 && ln.ff_ok;
    if (ok) {
      float *hi = c->d_pad32, *lo = c->d_pad32 + NP;
      for (int q = 0; q < (int)tabs.size(); q++) {
        const DevStencil::Lines &ln = tabs[q];
        if (q == 0 || nin > 1) {
          tgpu::launch_split_hilo(c->d_pad + (long)(ch0 + (nin > 1 ? q : 0)) * NP, NP, hi, lo, c->stream);
          c->stats.kernel_launches++;
        }
        tgpu::launch_conv_slab_ff(hi, lo, NP, ln.d_planes, ln.nplanes, ln.d_lines, ln.d_w, ln.d_w_lo,
                                  outs[nout > 1 ? q : 0], ln.pitch, ln.ncols, ln.max_rows, ln.max_lines, ln.max_w,
                                  c->dg.nx[0], c->dg.nx[1], c->dg.nx[2], c->stream);
        c->stats.kernel_launches++;
      }
      c->stats.conv_launches++;
      return;
    }
  }
  if (!f32 && c->ff_on && nin == 1 && nout == 1) {
    const DevStencil::Lines &ln = tr ? st.lines_tr : st.lines_fwd;
    if (ln.nplanes > 0 && ln.ncoef == 1 && ln.ff_ok) {
      // high and low FP32 parts of the channel in the (idle) FP32 padded buffer, which holds at least two
      // channels; loads past a part's end read zeros
      float *hi = c->d_pad32, *lo = c->d_pad32 + NP;
      tgpu::launch_split_hilo(c->d_pad + (long)ch0 * NP, NP, hi, lo, c->stream);
      tgpu::launch_conv_slab_ff(hi, lo, NP, ln.d_planes, ln.nplanes, ln.d_lines, ln.d_w, ln.d_w_lo, outs[0], ln.pitch,
                                ln.ncols, ln.max_rows, ln.max_lines, ln.max_w, c->dg.nx[0], c->dg.nx[1], c->dg.nx[2],
                                c->stream);
      c->stats.conv_launches++;
      c->stats.kernel_launches += 2;
      return;
    }
  }
  if (!f32)
    tgpu::launch_conv<double>(c->d_pad + (long)ch0 * NP, NP, nin, st.d_loff, tr ? st.d_coef_tr : st.d_coef_fwd, st.L,
                              outs, nout, true, c->dg.N, c->stream);
  else
    tgpu::launch_conv<float>(c->d_pad32 + (long)ch0 * NP, NP, nin, st.d_loff, tr ? st.d_coef_tr32 : st.d_coef_fwd32,
                             st.L, outs, nout, true, c->dg.N, c->stream);
  c->stats.conv_launches++;
  c->stats.kernel_launches++;
}

// Whether the FP32 attraction sums of the current context (tensor-core products, or FP32 slab sums) run
// faster as FP32 FFT convolutions: timed once per context on the padded channel 0 (values do not matter;
// the scratch output is d_tr, which every caller of forward_pass fills afterwards).
void decide_fft32(Ctx *c)
{
  int &flag = c->tc_on ? c->fft32_tc : c->fft32_slab;
  if (flag != 0) return;
  flag = -1;
  if (!prepare_spec32(c)) return;
  const DevStencil &st = c->sten[TGPU_STEN_UATT][0];
  if (st.spec_fwd32.empty()) return;
  double *o[1] = {c->d_tr};
  cudaEvent_t ev[4];
  for (auto &e : ev) ck(cudaEventCreate(&e), "event");
  flag = -1;
  conv(c, 0, 1, st, false, o, 1, true);   // warm-up of the direct sum
  ck(cudaEventRecord(ev[0], c->stream), "event");
  for (int r = 0; r < 2; r++) conv(c, 0, 1, st, false, o, 1, true);
  ck(cudaEventRecord(ev[1], c->stream), "event");
  flag = 1;
  conv(c, 0, 1, st, false, o, 1, true);   // warm-up of the FFT sum
  ck(cudaEventRecord(ev[2], c->stream), "event");
  for (int r = 0; r < 2; r++) conv(c, 0, 1, st, false, o, 1, true);
  ck(cudaEventRecord(ev[3], c->stream), "event");
  ck(cudaEventSynchronize(ev[3]), "event");
  float t_direct = 0.f, t_fft = 0.f;
  ck(cudaEventElapsedTime(&t_direct, ev[0], ev[1]), "event");
  ck(cudaEventElapsedTime(&t_fft, ev[2], ev[3]), "event");
  for (auto &e : ev) cudaEventDestroy(e);
  flag = t_fft < t_direct ? 1 : -1;
  c->t32_att[c->tc_on ? 1 : 0][0] = 0.5f * t_direct;
  c->t32_att[c->tc_on ? 1 : 0][1] = 0.5f * t_fft;
}

// The same choice for one short stencil (theta, delta) and direction: its FP32 slab / point sum against the
// FP32 FFT, timed once on the padded channels ch0.. into d_dscr.  The FFT runs after the first reuse the
// field's transform when it is the one the forward sums share (the channel's spectrum stays cached).
void decide_fft32_sten(Ctx *c, DevStencil &st, bool tr, int ch0, int nin, int nout)
{
  int &flag = tr ? st.fft32_tr : st.fft32_fwd;
  if (flag != 0) return;
  flag = -1;
  if (!prepare_spec32(c)) return;
  if (tr ? (int)st.spec_tr32.size() != nin : (int)st.spec_fwd32.size() != nout) return;
  const long N = c->dg.N;
  if (!c->d_dscr) c->d_dscr = dalloc<double>((size_t)tgpu::kMaxRb * N);
  double *o[tgpu::kMaxRb];
  for (int q = 0; q < nout; q++) o[q] = c->d_dscr + (long)q * N;
  cudaEvent_t ev[4];
  for (auto &e : ev) ck(cudaEventCreate(&e), "event");
  conv(c, ch0, nin, st, tr, o, nout, true);   // warm-up of the direct sum
  ck(cudaEventRecord(ev[0], c->stream), "event");
  for (int r = 0; r < 2; r++) conv(c, ch0, nin, st, tr, o, nout, true);
  ck(cudaEventRecord(ev[1], c->stream), "event");
  flag = 1;
  conv(c, ch0, nin, st, tr, o, nout, true);   // warm-up of the FFT sum
  ck(cudaEventRecord(ev[2], c->stream), "event");
  for (int r = 0; r < 2; r++) conv(c, ch0, nin, st, tr, o, nout, true);
  ck(cudaEventRecord(ev[3], c->stream), "event");
  ck(cudaEventSynchronize(ev[3]), "event");
  float t_direct = 0.f, t_fft = 0.f;
  ck(cudaEventElapsedTime(&t_direct, ev[0], ev[1]), "event");
  ck(cudaEventElapsedTime(&t_fft, ev[2], ev[3]), "event");
  for (auto &e : ev) cudaEventDestroy(e);
  flag = t_fft < t_direct ? 1 : -1;
  st.t32[tr ? 1 : 0][0] = 0.5f * t_direct;
  st.t32[tr ? 1 : 0][1] = 0.5f * t_fft;
}

// Weighted-density (and mean-field) sums of the padded density channels with one zone's stencils
// into out (rows as d_conv)
void forward_convs(Ctx *c, const std::vector<DevStencil> *sten, double *out, bool f32)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  const int nd = g.ndim;
  for (int jc = 0; jc < g.ncomp; jc++) {
    double *o_th[1] = {out};
    std::vector<double *> o_de;
    o_de.push_back(out + 1 * N);
    if (!g.single_size) {
      o_de.push_back(out + 2 * N);
      o_de.push_back(out + 3 * N);
    }
    for (int d = 0; d < nd; d++) o_de.push_back(out + (long)(4 + d) * N);
    if (!g.single_size)
      for (int d = 0; d < nd; d++) o_de.push_back(out + (long)(4 + nd + d) * N);
    // every sum of this density by FFT (FP64 accurate fills, or FP32): all their inverse transforms in one launch
    // per pass
    if (!f32 && sten == c->sten && c->fft_on && c->fft_state == 1) {
      const DevStencil &sth = sten[TGPU_STEN_THETA][jc], &sde = sten[TGPU_STEN_DELTA][jc];
      bool all = sth.spec_fwd.size() == 1 && sde.spec_fwd.size() == o_de.size();
      if (g.attraction)
        for (int ic = 0; ic < g.ncomp; ic++) all = all && sten[TGPU_STEN_UATT][ic + g.ncomp * jc].spec_fwd.size() == 1;
      if (all) {
        std::vector<const double2 *> ks;
        std::vector<double *> os;
        ks.push_back(sth.spec_fwd[0]);
        os.push_back(out);
        for (size_t q = 0; q < o_de.size(); q++) {
          ks.push_back(sde.spec_fwd[q]);
          os.push_back(o_de[q]);
        }
        if (g.attraction)
          for (int ic = 0; ic < g.ncomp; ic++) {
            ks.push_back(sten[TGPU_STEN_UATT][ic + g.ncomp * jc].spec_fwd[0]);
            os.push_back(out + (long)(g.nrb + ic) * N);
          }
        const double2 *F = fft_channel(c, jc);
        std::vector<double2 *> &work = tr_boxes<double2>(c);
        while (work.size() < ks.size()) work.push_back(dalloc<double2>((size_t)c->fft.NH));
        tgpu::rfft_inverse_batch(F, ks.data(), (int)ks.size(), work.data(), c->fft, 1.0 / (double)c->fft.NR,
                                 os.data(), true, c->stream);
        c->stats.kernel_launches += 3 * ((ks.size() + tgpu::fft_max_batch() - 1) / tgpu::fft_max_batch());
        c->stats.conv_launches++;
        continue;
      }
    }
    if (f32 && sten == c->sten && c->spec32_built) {
      const DevStencil &sth = sten[TGPU_STEN_THETA][jc], &sde = sten[TGPU_STEN_DELTA][jc];
      bool all = use_fft32(c, sth, false, 1, 1) && use_fft32(c, sde, false, 1, (int)o_de.size());
      if (g.attraction)
        for (int ic = 0; ic < g.ncomp; ic++) all = all && use_fft32(c, sten[TGPU_STEN_UATT][ic + g.ncomp * jc], false, 1, 1);
      if (all) {
        std::vector<const float2 *> ks;
        std::vector<double *> os;
        ks.push_back(sth.spec_fwd32[0]);
        os.push_back(out);
        for (size_t q = 0; q < o_de.size(); q++) {
          ks.push_back(sde.spec_fwd32[q]);
          os.push_back(o_de[q]);
        }
        if (g.attraction)
          for (int ic = 0; ic < g.ncomp; ic++) {
            ks.push_back(sten[TGPU_STEN_UATT][ic + g.ncomp * jc].spec_fwd32[0]);
            os.push_back(out + (long)(g.nrb + ic) * N);
          }
        const float2 *F = fft_channel32(c, jc);
        std::vector<float2 *> &work = tr_boxes<float2>(c);
        while (work.size() < ks.size()) work.push_back(dalloc<float2>((size_t)c->fft.NH));
        if (c->store32) {   // the FP32 shadows of the sums
          std::vector<float *> os32;
          for (double *o : os) os32.push_back(c->d_conv32 + (o - c->d_conv));
          tgpu::rfft_inverse_batch(F, ks.data(), (int)ks.size(), work.data(), c->fft, 1.0 / (double)c->fft.NR,
                                   os32.data(), true, c->stream);
        } else {
          tgpu::rfft_inverse_batch(F, ks.data(), (int)ks.size(), work.data(), c->fft, 1.0 / (double)c->fft.NR,
                                   os.data(), true, c->stream);
        }
        c->stats.kernel_launches += 3 * ((ks.size() + tgpu::fft_max_batch() - 1) / tgpu::fft_max_batch());
        c->stats.conv_launches++;
        continue;
      }
    }
    if (c->store32) throw Error(TGPU_ERR_STATE, "an FP32-storage product needs a direct stencil sum");
    conv(c, jc, 1, sten[TGPU_STEN_THETA][jc], false, o_th, 1, f32);
    conv(c, jc, 1, sten[TGPU_STEN_DELTA][jc], false, o_de.data(), (int)o_de.size(), f32);
    if (g.attraction)
      for (int ic = 0; ic < g.ncomp; ic++) {
        double *o_mf[1] = {out + (long)(g.nrb + ic) * N};
        conv(c, jc, 1, sten[TGPU_STEN_UATT][ic + g.ncomp * jc], false, o_mf, 1, f32);
      }
  }
}

// Weighted-density (and mean-field) sums of a density-shaped field
// (`field` points at the first density row, rows N apart) into d_conv.
void forward_pass(Ctx *c, const double *field, const PadParams &pp, bool f32, bool zero_first = true)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  const size_t nrows = (size_t)(g.nrb + g.ncomp);
  if (zero_first) {
    if (c->store32) ck(cudaMemsetAsync(c->d_conv32, 0, sizeof(float) * nrows * N, c->stream), "memset");
    else ck(cudaMemsetAsync(c->d_conv, 0, sizeof(double) * nrows * N, c->stream), "memset");
  }
  pad(c, field, pp, f32);
  if (f32 && g.attraction && g.ndim == 3) decide_fft32(c);
  if (f32 && g.ndim == 3)
    for (int jc = 0; jc < g.ncomp; jc++) {
      decide_fft32_sten(c, c->sten[TGPU_STEN_THETA][jc], false, jc, 1, 1);
      decide_fft32_sten(c, c->sten[TGPU_STEN_DELTA][jc], false, jc, 1, c->sten[TGPU_STEN_DELTA][jc].nout_fwd);
    }
  forward_convs(c, c->sten, c->d_conv, f32);
  // nodes of the coarser quadrature zones keep their own zone's sums (zero_first holds with zones)
  for (int z = 1; z < c->nzone; z++) {
    ck(cudaMemsetAsync(c->d_zbuf, 0, sizeof(double) * nrows * N, c->stream), "memset");
    forward_convs(c, c->zsten[z], c->d_zbuf, f32);
    tgpu::launch_zone_merge(c->d_zbuf, c->d_conv, (int)nrows, N, c->d_zone, z, c->stream);
    c->stats.kernel_launches++;
  }
  if (g.hard_surf && !c->hw_targets.empty()) {
    tgpu::launch_hw_correct(field, N, 0, c->sten[TGPU_STEN_THETA].data(), c->sten[TGPU_STEN_DELTA].data(),
                            g.attraction ? c->sten[TGPU_STEN_UATT].data() : nullptr, g.ncomp, true, g.attraction != 0,
                            c->d_hw_targets, (int)c->hw_targets.size(), c->d_zero, c->d_bnodes, c->d_fmask,
                            c->d_conv, c->stream);
    c->stats.kernel_launches++;
  }
}

// Euler-Lagrange stencil sums of the padded channels with one zone's stencils into out ([ncomp][N]); where both the
// delta and the theta sums of a component take FFTs, their 2 + ndim channels share one inverse transform
void transpose_convs(Ctx *c, const std::vector<DevStencil> *sten, double *out, bool f32)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  const int nd = g.ndim;
  for (int ic = 0; ic < g.ncomp; ic++) {
    double *o[1] = {out + (long)ic * N};
    const DevStencil &sd = sten[TGPU_STEN_DELTA][ic], &st = sten[TGPU_STEN_THETA][ic];
    const int base = ic * (nd + 2);
    int chs[tgpu::kMaxRb];
    for (int t = 0; t < nd + 2; t++) chs[t] = base + t;
    if (sten == c->sten && f32 && c->spec32_built && use_fft32(c, sd, true, 1 + nd, 1) &&
        use_fft32(c, st, true, 1, 1)) {
      const float2 *k[tgpu::kMaxRb];
      for (int t = 0; t <= nd; t++) k[t] = sd.spec_tr32[t];
      k[nd + 1] = st.spec_tr32[0];
      fft_tr_sum<float2>(c, chs, k, nd + 2, o[0]);
      continue;
    }
    if (sten == c->sten && !f32 && c->fft_on && c->fft_state == 1 && (int)sd.spec_tr.size() == 1 + nd &&
        st.spec_tr.size() == 1) {
      const double2 *k[tgpu::kMaxRb];
      for (int t = 0; t <= nd; t++) k[t] = sd.spec_tr[t];
      k[nd + 1] = st.spec_tr[0];
      fft_tr_sum<double2>(c, chs, k, nd + 2, o[0]);
      continue;
    }
    if (c->store32) throw Error(TGPU_ERR_STATE, "an FP32-storage product needs a direct stencil sum");
    conv(c, base, 1 + nd, sd, true, o, 1, f32);
    conv(c, base + nd + 1, 1, st, true, o, 1, f32);
  }
}

// Euler-Lagrange stencil sums over the channels in d_chan into d_tr.
void transpose_pass(Ctx *c, const PadParams &pp, bool f32, const double *chan = nullptr, bool zero_first = true)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  if (c->store32) {
    if (zero_first) ck(cudaMemsetAsync(c->d_tr32, 0, sizeof(float) * (size_t)g.ncomp * N, c->stream), "memset");
    pad32(c, c->d_chan32, pp);
  } else {
    if (zero_first) ck(cudaMemsetAsync(c->d_tr, 0, sizeof(double) * (size_t)g.ncomp * N, c->stream), "memset");
    pad(c, chan ? chan : c->d_chan, pp, f32);
  }
  if (f32 && g.ndim == 3)
    for (int ic = 0; ic < g.ncomp; ic++) {
      const int base = ic * (g.ndim + 2);
      decide_fft32_sten(c, c->sten[TGPU_STEN_DELTA][ic], true, base, 1 + g.ndim, 1);
      decide_fft32_sten(c, c->sten[TGPU_STEN_THETA][ic], true, base + g.ndim + 1, 1, 1);
    }
  transpose_convs(c, c->sten, c->d_tr, f32);
  for (int z = 1; z < c->nzone; z++) {
    ck(cudaMemsetAsync(c->d_zbuf, 0, sizeof(double) * (size_t)g.ncomp * N, c->stream), "memset");
    transpose_convs(c, c->zsten[z], c->d_zbuf, f32);
    tgpu::launch_zone_merge(c->d_zbuf, c->d_tr, g.ncomp, N, c->d_zone, z, c->stream);
    c->stats.kernel_launches++;
  }
}

void red_to_host(Ctx *c, int n);

void ensure_refs(Ctx *c)
{
  if (c->d_rho_ref) return;
  const tgpu::DevGeom &g = c->dg;
  const size_t N = g.N;
  c->d_rho_ref = dalloc<double>(g.ncomp * N);
  c->d_conv_ref = dalloc<double>((g.nrb + g.ncomp) * N);
  c->d_chan_ref = dalloc<double>((size_t)c->nch_max * N);
  c->d_tr_ref = dalloc<double>(g.ncomp * N);
  c->d_drho = dalloc<double>(g.ncomp * N);
  c->d_dchan = dalloc<double>((size_t)c->nch_max * N);
}

void copy_d(Ctx *c, double *dst, const double *src, size_t n)
{
  ck(cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream), "d2d");
}

// Residual fill.  arith: TGPU_FILL_FP64 sums everything in FP64; TGPU_FILL_FP32
// sums in FP32 (inexact residual for early Newton steps); TGPU_FILL_REFINED
// keeps FP64 sums of a reference state and adds FP32 sums of the change since
// then, refreshing the reference in FP64 when the change exceeds tau of the field.
void fill_arith(Ctx *c, const double *d_x, double *d_R, int mode, int arith)
{
  need_final(c);
  if (c->nzone > 1 && arith == TGPU_FILL_REFINED) arith = TGPU_FILL_FP64;   // zone sums are formed whole
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  if (d_x != c->d_x && mode == 0)
    ck(cudaMemcpyAsync(c->d_x, d_x, sizeof(double) * (size_t)g.nunk * N, cudaMemcpyDeviceToDevice, c->stream), "copy x");
  const double *x = mode == 0 ? c->d_x : d_x;
  const double *rho = x + (long)g.first_rho * N;
  const size_t nrho = (size_t)g.ncomp * N, nconv = (size_t)(g.nrb + g.ncomp) * N;
  const size_t nchan = (size_t)g.ncomp * (g.ndim + 2) * N, ntr = (size_t)g.ncomp * N;
  if (!c->d_domain) c->d_domain = dalloc<unsigned>(1);
  ck(cudaMemsetAsync(c->d_domain, 0, sizeof(unsigned), c->stream), "memset");
  if (arith == TGPU_FILL_REFINED) {
    ensure_refs(c);
    tgpu::launch_fmt_local(x, c->d_chan, c->stream, c->d_domain);
    bool refresh = !c->have_ref;
    if (!refresh) {
      const int nb = tgpu::reduce_blocks((long)nchan);
      tgpu::launch_delta_maxabs(rho, c->d_rho_ref, (long)nrho, c->d_drho, c->d_partial, nb, c->d_red, c->stream);
      tgpu::launch_delta_maxabs(c->d_chan, c->d_chan_ref, (long)nchan, c->d_dchan, c->d_partial + 2048, nb,
                                c->d_red + 2, c->stream);
      red_to_host(c, 4);
      const double *m = c->h_red;
      refresh = !(m[0] <= c->refine_tau * m[1]) || !(m[2] <= c->refine_tau * m[3]);
    }
    if (refresh) {
      forward_pass(c, rho, c->pads.rho_res, false);
      transpose_pass(c, c->pads.tr_res, false);
      copy_d(c, c->d_rho_ref, rho, nrho);
      copy_d(c, c->d_conv_ref, c->d_conv, nconv);
      copy_d(c, c->d_chan_ref, c->d_chan, nchan);
      copy_d(c, c->d_tr_ref, c->d_tr, ntr);
      c->have_ref = true;
      c->stats.fp64_refreshes++;
    } else {
      copy_d(c, c->d_conv, c->d_conv_ref, nconv);
      forward_pass(c, c->d_drho, c->pads.rho_jac, true, false);
      copy_d(c, c->d_tr, c->d_tr_ref, ntr);
      transpose_pass(c, c->pads.tr_jac, true, c->d_dchan, false);
      // carry the reference forward: the sums just formed become the reference of the
      // next fill, so each FP32 sum only covers one Newton update (errors add up as
      // 1e-7 of the sum of the updates, which shrink quadratically near the solution)
      copy_d(c, c->d_rho_ref, rho, nrho);
      copy_d(c, c->d_conv_ref, c->d_conv, nconv);
      copy_d(c, c->d_chan_ref, c->d_chan, nchan);
      copy_d(c, c->d_tr_ref, c->d_tr, ntr);
    }
  } else {
    const bool f32 = arith == TGPU_FILL_FP32;
    c->ff_on = arith == TGPU_FILL_FF || arith == TGPU_FILL_FFT;   // FFT: long stencils; float-float: the rest
    c->fft_on = arith == TGPU_FILL_FFT;
    if (c->fft_on) ensure_fft(c);
    forward_pass(c, rho, c->pads.rho_res, f32);
    tgpu::launch_fmt_local(x, c->d_chan, c->stream, c->d_domain);
    transpose_pass(c, c->pads.tr_res, f32);
    c->ff_on = false;
    c->fft_on = false;
  }
  tgpu::launch_assemble(x, c->d_vext, c->d_zero, c->d_conv, c->d_tr, d_R, c->stream, c->d_domain);
  c->stats.kernel_launches += 2;
  if (c->coarse()) {   // the averaged rows of coarsened nodes
    tgpu::launch_coarse_rows(x, d_R, g.nunk, g.first_rho, g.ncomp, N, c->cr, c->d_cbulk, c->stream);
    c->stats.kernel_launches++;
  }
  if (mode == 0) {
    c->have_state = true;
    c->hcoef_form = -1;   // a new state: its Hessian scalars are made at the first product
    c->hcoef32_form = -1;
  }
}

void fill_device(Ctx *c, const double *d_x, double *d_R, int mode)
{
  // outside the Newton solve the mixed policy means the accurate (FP64) residual
  fill_arith(c, d_x, d_R, mode,
             c->fill_mode == TGPU_FILL_MIXED ? TGPU_FILL_FP64
             : c->fill_mode == TGPU_FILL_MIXED_FF ? TGPU_FILL_FF
             : c->fill_mode == TGPU_FILL_MIXED_FFT ? TGPU_FILL_FFT : c->fill_mode);
}

// TGPU_ERR_DOMAIN when the last fill took log(1 - n3) or 1/(1 - n3)^k at n3 >= 1, or log(rho) of rho <= 0 on a
// live Euler-Lagrange row (the reference evaluates them unguarded, calc_FMT_derivatives src/dft_fill_FMT.c:362-366,
// fill_EL_ideal_gas src/dft_fill_EL.c:358, and its Newton fails on the NaN); waits for the stream
void check_domain(Ctx *c)
{
  if (!c->d_domain) return;
  unsigned f = 0;
  ck(cudaMemcpyAsync(&f, c->d_domain, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "d2h");
  ck(cudaStreamSynchronize(c->stream), "sync");
  if (f & tgpu::kDomainN3) throw Error(TGPU_ERR_DOMAIN, "n3 >= 1 at some node: log(1 - n3) and 1/(1 - n3) undefined");
  if (f & tgpu::kDomainRho) throw Error(TGPU_ERR_DOMAIN, "density <= 0 on a live Euler-Lagrange row: log(rho) undefined");
}

void need_state(Ctx *c)
{
  need_final(c);
  if (!c->have_state) throw Error(TGPU_ERR_STATE, "no Jacobian state: call tgpu_fill with mode 0 first");
}

// Arithmetic of the Jacobian / Schur products: TGPU_FP16TC runs the 3-D attraction sums on the tensor cores;
// TGPU_FP64_FFT keeps every sum FP64-accurate but takes the long 3-D ones as FP64 FFT convolutions and the
// short ones in float-float arithmetic (the sums of TGPU_FILL_FFT)
struct TcScope {
  Ctx *c;
  bool prev_tc, prev_ff, prev_fft;
  explicit TcScope(Ctx *c_) : c(c_), prev_tc(c_->tc_on), prev_ff(c_->ff_on), prev_fft(c_->fft_on)
  {
    c->tc_on = c->precision == TGPU_FP16TC && c->tc_ready;
    if (c->precision == TGPU_FP64_FFT) {
      c->ff_on = c->fft_on = true;
      ensure_fft(c);
    }
  }
  ~TcScope()
  {
    c->tc_on = prev_tc;
    c->ff_on = prev_ff;
    c->fft_on = prev_fft;
  }
};

// whether the products' stencil sums run in FP32 arithmetic
bool prod_f32(const Ctx *c) { return c->precision == TGPU_FP32 || c->precision == TGPU_FP16TC; }

// the state's Hessian scalars for the products, made once per state and Jacobian form
const double *hess_coef(Ctx *c)
{
  const int form = c->dg.jac_exact;
  if (c->hcoef_form == form) return c->d_hcoef;
  if (!c->d_hcoef) c->d_hcoef = dalloc<double>((size_t)tgpu::kHessCoef * c->dg.N);
  tgpu::launch_hess_coef(c->d_x, c->d_hcoef, c->stream, c->d_hcoef32);   // with the FP32 table once it exists
  c->stats.kernel_launches++;
  c->hcoef_form = form;
  if (c->d_hcoef32) {
    tgpu::launch_row_info32(c->d_x, c->d_vext, c->d_zero, c->d_inv32, c->d_kind32, c->stream);
    c->stats.kernel_launches++;
    c->hcoef32_form = form;
  }
  return c->d_hcoef;
}

// With coarsened nodes the Schur complement is that of the step on the other nodes: the densities, and
// the block-1 vector between A12 and A21, are interpolated onto the coarsened nodes, whose rows are dropped.
const double *prolonged(Ctx *c, const double *v, int nrows)
{
  if (!c->coarse()) return v;
  copy_d(c, c->d_cscr, v, (size_t)nrows * c->dg.N);
  tgpu::launch_prolong(c->d_cscr, 0, nrows, c->dg.nunk, c->dg.N, c->cr, nullptr, c->stream);
  c->stats.kernel_launches++;
  return c->d_cscr;
}

// The FP32 Schur product with FP32 storage: every stencil sum an FP32 FFT (the choices already made by timing), in
// 3-D, with one quadrature zone, no hard-wall corrections and no coarsened nodes
bool schur_store32_ok(Ctx *c)
{
  const tgpu::DevGeom &g = c->dg;
  if (!prod_f32(c) || !c->spec32_built || g.ndim != 3 || c->nzone != 1 || !c->hw_targets.empty() || c->coarse())
    return false;
  const int nde = 1 + (g.single_size ? 0 : 2) + g.ndim * (g.single_size ? 1 : 2);
  for (int jc = 0; jc < g.ncomp; jc++) {
    const DevStencil &sth = c->sten[TGPU_STEN_THETA][jc], &sde = c->sten[TGPU_STEN_DELTA][jc];
    if (!use_fft32(c, sth, false, 1, 1) || !use_fft32(c, sde, false, 1, nde)) return false;
    if (!use_fft32(c, sde, true, 1 + g.ndim, 1) || !use_fft32(c, sth, true, 1, 1)) return false;
    if (g.attraction)
      for (int ic = 0; ic < g.ncomp; ic++)
        if (!use_fft32(c, c->sten[TGPU_STEN_UATT][ic + g.ncomp * jc], false, 1, 1)) return false;
  }
  return true;
}

// the FP32 storage's buffers, and the state's FP32 Hessian table and row table (made from the FP64 evaluation)
void ensure_store32(Ctx *c)
{
  const tgpu::DevGeom &g = c->dg;
  const size_t N = (size_t)g.N;
  if (!c->d_conv32) {
    c->d_conv32 = dalloc<float>((size_t)(g.nrb + g.ncomp) * N);
    c->d_chan32 = dalloc<float>((size_t)g.ncomp * (g.ndim + 2) * N);
    c->d_tr32 = dalloc<float>((size_t)g.ncomp * N);
    c->d_ymf32 = dalloc<float>((size_t)g.ncomp * N);
    c->d_hcoef32 = dalloc<float>((size_t)(tgpu::kHessCoef + g.nrb) * N);
    c->d_inv32 = dalloc<double>((size_t)g.ncomp * N);
    c->d_kind32 = dalloc<signed char>((size_t)g.ncomp * N);
  }
  if (c->hcoef32_form != g.jac_exact) {
    tgpu::launch_hess_coef32(c->d_x, c->d_hcoef32, c->stream);
    tgpu::launch_row_info32(c->d_x, c->d_vext, c->d_zero, c->d_inv32, c->d_kind32, c->stream);
    c->stats.kernel_launches += 2;
    c->hcoef32_form = g.jac_exact;
  }
}

void schur_device_store32(Ctx *c, const double *d_v2, double *d_y2)
{
  const tgpu::DevGeom &g = c->dg;
  ensure_store32(c);
  c->store32 = true;
  try {
    forward_pass(c, d_v2, c->pads.rho_jac, true);
    tgpu::launch_schur_local32(g.ndim, c->d_conv32, c->d_hcoef32, c->d_chan32, c->d_ymf32, c->stream);
    transpose_pass(c, c->pads.tr_jac, true);
  } catch (...) {
    c->store32 = false;
    c->pad_src32 = nullptr;
    throw;
  }
  c->store32 = false;
  c->pad_src32 = nullptr;
  tgpu::launch_schur_combine32(c->d_inv32, c->d_kind32, d_v2, c->d_tr32, c->d_ymf32, d_y2, c->stream);
  c->stats.kernel_launches += 2;
  c->stats.schur_applies++;
}

void schur_device(Ctx *c, const double *d_v2, double *d_y2)
{
  need_state(c);
  TcScope tcs(c);
  const tgpu::DevGeom &g = c->dg;
  const bool f32 = prod_f32(c);
  if (f32 && schur_store32_ok(c)) {
    schur_device_store32(c, d_v2, d_y2);
    return;
  }
  const double *v2 = prolonged(c, d_v2, g.ncomp);
  forward_pass(c, v2, c->pads.rho_jac, f32);
  if (c->coarse()) tgpu::launch_prolong(c->d_conv, 0, g.nrb + g.ncomp, g.nunk, g.N, c->cr, nullptr, c->stream);
  tgpu::launch_schur_local(c->d_x, c->d_conv, c->d_chan, c->d_ymf, hess_coef(c), c->stream, f32);
  transpose_pass(c, c->pads.tr_jac, f32);
  tgpu::launch_schur_combine(c->d_x, c->d_vext, c->d_zero, v2, c->d_tr, c->d_ymf, d_y2, c->stream);
  if (c->coarse()) tgpu::launch_zero_nodes(d_y2, g.ncomp, g.N, c->cr, c->stream);
  c->stats.kernel_launches += 2;
  c->stats.schur_applies++;
}

void jv_device(Ctx *c, const double *d_v, double *d_out)
{
  need_state(c);
  TcScope tcs(c);
  const long N = c->dg.N;
  const bool f32 = prod_f32(c);
  forward_pass(c, d_v + (long)c->dg.first_rho * N, c->pads.rho_jac, f32);
  tgpu::launch_jv_local(c->d_x, d_v, c->d_chan, hess_coef(c), c->stream, f32);
  transpose_pass(c, c->pads.tr_jac, f32);
  tgpu::launch_jv_combine(c->d_x, c->d_vext, c->d_zero, d_v, c->d_conv, c->d_tr, d_out, c->stream);
  c->stats.kernel_launches += 2;
  if (c->coarse())
    tgpu::launch_coarse_rows(d_v, d_out, c->dg.nunk, c->dg.first_rho, c->dg.ncomp, N, c->cr, nullptr, c->stream);
}

}  // namespace

// ---- kernels used only by the Schur rhs / back-substitution ------------------
namespace tgpu {
void launch_rhs_local(const double *x, const double *b, double *chan, double *ymf, const double *coef, cudaStream_t s);
void launch_rhs_combine(const double *vext, const signed char *zero, const double *b, const double *tr,
                        const double *ymf, double *b2s, cudaStream_t s);
void launch_x1(const double *b, const double *conv, const double *x2, double *dx, cudaStream_t s);
}  // namespace tgpu

namespace {

void schur_rhs_device(Ctx *c, const double *d_b, double *d_b2s)
{
  need_state(c);
  const tgpu::DevGeom &g = c->dg;
  const double *b = d_b;
  if (c->coarse()) {   // block-1 right-hand sides interpolated onto the coarsened nodes
    copy_d(c, c->d_cscr, d_b, (size_t)g.nunk * g.N);
    tgpu::launch_prolong(c->d_cscr, g.first_rb, g.nunk - g.ncomp, g.nunk, g.N, c->cr, nullptr, c->stream);
    b = c->d_cscr;
  }
  TcScope tcs(c);
  if (prod_f32(c) && schur_store32_ok(c)) {   // the FP32 products' right-hand side in FP32 storage
    ensure_store32(c);
    tgpu::launch_rhs_local32(g.ndim, b, c->d_hcoef32, c->d_chan32, c->d_ymf32, c->stream);
    c->store32 = true;
    try {
      transpose_pass(c, c->pads.tr_jac, true);
    } catch (...) {
      c->store32 = false;
      c->pad_src32 = nullptr;
      throw;
    }
    c->store32 = false;
    c->pad_src32 = nullptr;
    tgpu::launch_rhs_combine32(c->d_kind32, b, c->d_tr32, c->d_ymf32, d_b2s, c->stream);
    c->stats.kernel_launches += 2;
    return;
  }
  tgpu::launch_rhs_local(c->d_x, b, c->d_chan, c->d_ymf, hess_coef(c), c->stream);
  transpose_pass(c, c->pads.tr_jac, prod_f32(c));
  tgpu::launch_rhs_combine(c->d_vext, c->d_zero, b, c->d_tr, c->d_ymf, d_b2s, c->stream);
  if (c->coarse()) tgpu::launch_zero_nodes(d_b2s, g.ncomp, g.N, c->cr, c->stream);
  c->stats.kernel_launches += 2;
}

void schur_x1_device(Ctx *c, const double *d_b, const double *d_x2, double *d_dx)
{
  need_state(c);
  TcScope tcs(c);
  const tgpu::DevGeom &g = c->dg;
  const double *x2 = prolonged(c, d_x2, g.ncomp);
  forward_pass(c, x2, c->pads.rho_jac, prod_f32(c));
  tgpu::launch_x1(d_b, c->d_conv, x2, d_dx, c->stream);
  if (c->coarse()) tgpu::launch_prolong(d_dx, 0, g.nunk, g.nunk, g.N, c->cr, nullptr, c->stream);
  c->stats.kernel_launches++;
}

// coarsened nodes' values interpolated from the others (bulk terms included)
void coarse_state(Ctx *c, double *d_x)
{
  if (!c->coarse()) return;
  tgpu::launch_prolong(d_x, 0, c->dg.nunk, c->dg.nunk, c->dg.N, c->cr, c->d_cbulk, c->stream);
  c->stats.kernel_launches++;
}

// ---- GMRES on the Schur complement (src/dft_HardSphereLinProbMgr.cpp:345-428) --

void ensure_krylov(Ctx *c, int kdim)
{
  if (kdim <= c->kdim) return;
  dfree(c->d_V);
  c->d_V = dalloc<double>((size_t)(kdim + 1) * c->n2);
  c->kdim = kdim;
}

void red_to_host(Ctx *c, int n)
{
  ck(cudaMemcpyAsync(c->h_red, c->d_red, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream), "d2h");
  ck(cudaStreamSynchronize(c->stream), "sync");
}

void tc_check(Ctx *c);
void schur_t_device(Ctx *c, const double *d_v2, double *d_y2);

int gmres(Ctx *c, const double *d_rhs, double *d_x2, double tol, int maxit, int *iters, double *relres)
{
  const long n = c->n2;
  const int nb = tgpu::reduce_blocks(n);
  const int kdim = std::max(1, std::min(maxit, 500));
  ensure_krylov(c, kdim);
  double *V = c->d_V;
  ck(cudaMemsetAsync(d_x2, 0, sizeof(double) * n, c->stream), "memset");
  // r0 = M^-1 b
  tgpu::launch_precond(c->d_x, c->d_vext, c->d_zero, d_rhs, c->d_gt, c->stream);
  tgpu::launch_norm2(c->d_gt, n, c->d_partial, nb, c->d_red, c->stream);
  red_to_host(c, 1);
  const double r0 = std::sqrt(c->h_red[0]);
  *iters = 0;
  *relres = 0.0;
  if (!(r0 > 0.0)) {
    if (!std::isfinite(r0)) throw Error(TGPU_ERR_NONFINITE, "non-finite right-hand side in the Schur solve");
    return TGPU_OK;
  }
  int it = 0;
  double rel = 1.0;
  std::vector<double> H((size_t)(kdim + 1) * kdim), cs(kdim), sn(kdim), gv(kdim + 1), y(kdim);
  bool first = true;
  while (it < maxit) {
    double beta;
    if (first) {
      beta = r0;
      tgpu::launch_scale(V, c->d_gt, 1.0 / beta, n, c->stream);
      first = false;
    } else {
      // r = M^-1 (b - S x)
      if (c->gmres_transpose) schur_t_device(c, d_x2, c->d_gw);
      else schur_device(c, d_x2, c->d_gw);
      tgpu::launch_axpby(c->d_gw, 1.0, d_rhs, -1.0, n, c->stream);
      tgpu::launch_precond(c->d_x, c->d_vext, c->d_zero, c->d_gw, c->d_gt, c->stream);
      tgpu::launch_norm2(c->d_gt, n, c->d_partial, nb, c->d_red, c->stream);
      red_to_host(c, 1);
      beta = std::sqrt(c->h_red[0]);
      rel = beta / r0;
      if (rel < tol) break;
      tgpu::launch_scale(V, c->d_gt, 1.0 / beta, n, c->stream);
    }
    const int m = std::min(kdim, maxit - it);
    std::fill(H.begin(), H.end(), 0.0);
    std::fill(gv.begin(), gv.end(), 0.0);
    gv[0] = beta;
    int k = 0;
    for (; k < m; k++) {
      if (c->gmres_transpose) schur_t_device(c, V + (long)k * n, c->d_gw);
      else schur_device(c, V + (long)k * n, c->d_gw);
      tgpu::launch_precond(c->d_x, c->d_vext, c->d_zero, c->d_gw, c->d_gt, c->stream);
      // classical Gram-Schmidt, two passes; h and the norm stay on the device
      // until one copy per iteration
      double *d_h1 = c->d_red, *d_h2 = c->d_red + (kdim + 1), *d_nrm = c->d_red + 2 * (kdim + 1);
      tgpu::launch_multidot(V, n, k + 1, c->d_gt, n, c->d_partial, nb, d_h1, c->stream);
      tgpu::launch_multiaxpy(c->d_gt, V, n, k + 1, d_h1, n, c->stream);
      tgpu::launch_multidot(V, n, k + 1, c->d_gt, n, c->d_partial, nb, d_h2, c->stream);
      tgpu::launch_multiaxpy(c->d_gt, V, n, k + 1, d_h2, n, c->stream);
      tgpu::launch_norm2(c->d_gt, n, c->d_partial, nb, d_nrm, c->stream);
      c->stats.kernel_launches += 6;
      red_to_host(c, 2 * (kdim + 1) + 1);
      const double hn = std::sqrt(c->h_red[2 * (kdim + 1)]);
      if (!std::isfinite(hn)) throw Error(TGPU_ERR_NONFINITE, "non-finite Krylov vector in the Schur solve");
      for (int j = 0; j <= k; j++) H[(size_t)j * kdim + k] = c->h_red[j] + c->h_red[kdim + 1 + j];
      H[(size_t)(k + 1) * kdim + k] = hn;
      if (hn > 0.0) tgpu::launch_scale(V + (long)(k + 1) * n, c->d_gt, 1.0 / hn, n, c->stream);
      for (int j = 0; j < k; j++) {
        const double a = H[(size_t)j * kdim + k], b = H[(size_t)(j + 1) * kdim + k];
        H[(size_t)j * kdim + k] = cs[j] * a + sn[j] * b;
        H[(size_t)(j + 1) * kdim + k] = -sn[j] * a + cs[j] * b;
      }
      const double a = H[(size_t)k * kdim + k], b = H[(size_t)(k + 1) * kdim + k];
      const double den = std::sqrt(a * a + b * b);
      cs[k] = den == 0.0 ? 1.0 : a / den;
      sn[k] = den == 0.0 ? 0.0 : b / den;
      H[(size_t)k * kdim + k] = den;
      H[(size_t)(k + 1) * kdim + k] = 0.0;
      gv[k + 1] = -sn[k] * gv[k];
      gv[k] = cs[k] * gv[k];
      it++;
      rel = std::fabs(gv[k + 1]) / r0;
      if (rel < tol || hn == 0.0) {
        k++;
        break;
      }
    }
    for (int i = k - 1; i >= 0; i--) {
      double s = gv[i];
      for (int j = i + 1; j < k; j++) s -= H[(size_t)i * kdim + j] * y[j];
      y[i] = s / H[(size_t)i * kdim + i];
    }
    // x -= sum_j (-y_j) V_j
    for (int j = 0; j < k; j++) c->h_red[j] = -y[j];
    ck(cudaMemcpyAsync(c->d_red, c->h_red, sizeof(double) * k, cudaMemcpyHostToDevice, c->stream), "h2d");
    tgpu::launch_multiaxpy(d_x2, V, n, k, c->d_red, n, c->stream);
    ck(cudaStreamSynchronize(c->stream), "sync");
    if (rel < tol) break;
  }
  *iters = it;
  *relres = rel;
  return rel < tol ? TGPU_OK : TGPU_ERR_NOCONV;
}

int solve_device(Ctx *c, const double *d_b, double *d_dx, double tol, int maxit, int *iters, double *relres)
{
  need_state(c);
  schur_rhs_device(c, d_b, c->d_b2s);
  const int st = gmres(c, c->d_b2s, c->d_gx, tol, maxit, iters, relres);
  schur_x1_device(c, d_b, c->d_gx, d_dx);
  return st;
}

int newton_device(Ctx *c, double *d_x, double rel_tol, double abs_tol, double update_floor, int max_iter,
                  double lin_tol, int lin_max_iter, int *iters, double *final_resid)
{
  need_final(c);
  const tgpu::DevGeom &g = c->dg;
  const long n = (long)g.nunk * g.N;
  const int nb = tgpu::reduce_blocks(n);
  double *d_R = c->d_work, *d_dx = c->d_work2;
  int it = 0;
  bool converged = false;
  double rnorm = 0.0;
  int st = TGPU_OK;
  // With the refined residual, iterations far from the solution use FP32 sums;
  // once ||R|| falls below refine_switch the residual is FP64-accurate.
  double rprev = 1e300;
  coarse_state(c, d_x);
  while (it < max_iter && !converged) {
    it++;
    int arith = c->fill_mode;
    if (arith == TGPU_FILL_REFINED && rprev > c->refine_switch) arith = TGPU_FILL_FP32;
    fill_arith(c, d_x, d_R, 0, arith);
    tgpu::launch_norm2(d_R, n, c->d_partial, nb, c->d_red, c->stream);
    red_to_host(c, 1);
    check_domain(c);
    rnorm = std::sqrt(c->h_red[0]);
    rprev = rnorm;
    if (!std::isfinite(rnorm)) throw Error(TGPU_ERR_NONFINITE, "non-finite residual in Newton");
    // b = -R (the reference's rhs)
    tgpu::launch_scale(d_R, d_R, -1.0, n, c->stream);
    int li = 0;
    double lr = 0.0;
    st = solve_device(c, d_R, d_dx, lin_tol, lin_max_iter, &li, &lr);
    // update_solution (src/dft_newton.c:266-381): positivity fraction, clamps, weighted norm
    tgpu::launch_newton_frac(d_x, d_dx, update_floor, c->d_partial, nb, c->d_red, c->stream);
    red_to_host(c, 1);
    const double frac = c->h_red[0];
    tgpu::launch_newton_update(d_x, d_dx, frac, rel_tol, abs_tol, c->d_partial, nb, c->d_red, c->stream);
    coarse_state(c, d_x);
    red_to_host(c, 1);
    const double upd = std::sqrt(c->h_red[0]);
    if (!std::isfinite(upd)) throw Error(TGPU_ERR_NONFINITE, "non-finite Newton update");
    converged = upd <= 1.0;
    c->stats.kernel_launches += 5;
  }
  *iters = it;
  if (final_resid) {
    // residual of the returned state, with the accurate arithmetic of the handle
    fill_arith(c, d_x, d_R, 1, c->fill_mode == TGPU_FILL_FP32 ? TGPU_FILL_FP32 : c->fill_mode);
    tgpu::launch_norm2(d_R, n, c->d_partial, nb, c->d_red, c->stream);
    red_to_host(c, 1);
    rnorm = std::sqrt(c->h_red[0]);
    *final_resid = rnorm;
  }
  (void)st;
  return converged ? TGPU_OK : TGPU_ERR_NOCONV;
}

// Residual-targeted Newton: iterate until ||R||_2 <= resid_tol with R taken in
// FP64-accurate arithmetic.  The inexact-Newton linear tolerance follows
// Eisenstat and Walker's second choice, eta_k = 0.9 (||R_k|| / ||R_k-1||)^2,
// kept in [lin_tol, 0.1] and not below 0.9 eta_k-1^2 when that exceeds 0.1.
// Under TGPU_FILL_MIXED (and TGPU_FILL_REFINED) the residual is summed in FP32
// while ||R||_2 > refine_switch; below it the final iterations use FP64
// (respectively refined) sums, so the returned residual is FP64-accurate.
int newton_solve_device(Ctx *c, double *d_x, double resid_tol, int max_iter, double lin_tol, int lin_max_iter,
                        double update_floor, int *iters, double *final_resid, int *lin_iters_total)
{
  need_final(c);
  const tgpu::DevGeom &g = c->dg;
  const long n = (long)g.nunk * g.N;
  const int nb = tgpu::reduce_blocks(n);
  double *d_R = c->d_work, *d_dx = c->d_work2;
  int it = 0, lin_total = 0;
  double rprev = 1e300, eta = 0.1, rnorm = 1e300;
  bool converged = false;
  coarse_state(c, d_x);
  for (;;) {
    int arith = c->fill_mode;
    const bool inexact = (arith == TGPU_FILL_MIXED || arith == TGPU_FILL_MIXED_FF || arith == TGPU_FILL_MIXED_FFT ||
                          arith == TGPU_FILL_REFINED) &&
                         rprev > c->refine_switch;
    if (inexact) arith = TGPU_FILL_FP32;
    else if (arith == TGPU_FILL_MIXED) arith = TGPU_FILL_FP64;
    else if (arith == TGPU_FILL_MIXED_FF) arith = TGPU_FILL_FF;
    else if (arith == TGPU_FILL_MIXED_FFT) arith = TGPU_FILL_FFT;
    fill_arith(c, d_x, d_R, 0, arith);
    tgpu::launch_norm2(d_R, n, c->d_partial, nb, c->d_red, c->stream);
    red_to_host(c, 1);
    check_domain(c);
    rnorm = std::sqrt(c->h_red[0]);
    if (!std::isfinite(rnorm)) throw Error(TGPU_ERR_NONFINITE, "non-finite residual in Newton");
    if (inexact && rnorm <= c->refine_switch) {
      rprev = rnorm;   // close enough: redo this residual in the accurate arithmetic
      continue;
    }
    if (!inexact && rnorm <= resid_tol) {
      converged = true;
      break;
    }
    if (it >= max_iter) break;
    if (it > 0 && rprev < 1e299) {
      const double r = rnorm / rprev;
      double e = 0.9 * r * r;
      const double safe = 0.9 * eta * eta;
      if (safe > 0.1) e = std::max(e, safe);
      eta = std::min(0.1, std::max(e, lin_tol));
    }
    it++;
    rprev = rnorm;
    tgpu::launch_scale(d_R, d_R, -1.0, n, c->stream);
    int li = 0;
    double lr = 0.0;
    solve_device(c, d_R, d_dx, eta, lin_max_iter, &li, &lr);
    lin_total += li;
    tgpu::launch_newton_frac(d_x, d_dx, update_floor, c->d_partial, nb, c->d_red, c->stream);
    red_to_host(c, 1);
    const double frac = c->h_red[0];
    // no update norm here (the stopping test is the next residual, whose norm also catches a non-finite update)
    tgpu::launch_newton_update(d_x, d_dx, frac, 1.0, 1.0, nullptr, nb, nullptr, c->stream);
    coarse_state(c, d_x);
    c->stats.kernel_launches += 5;
  }
  *iters = it;
  if (final_resid) *final_resid = rnorm;
  if (lin_iters_total) *lin_iters_total = lin_total;
  tc_check(c);
  return converged ? TGPU_OK : TGPU_ERR_NOCONV;
}

// ---- adjoint: J^T w and J^T lambda = g ------------------------------------

void ensure_adjoint(Ctx *c)
{
  if (c->d_adj_chan) return;
  const tgpu::DevGeom &g = c->dg;
  const size_t N = g.N;
  const int nch = g.ncomp * (g.ndim + 3);
  c->d_adj_chan = dalloc<double>((size_t)nch * N);
  c->d_adj_pad = dalloc<double>((size_t)nch * g.NP);
  c->d_adj_g = dalloc<double>((size_t)g.ncomp * (g.ndim + 2) * N);
  c->d_adj_v = dalloc<double>((size_t)g.nunk * N);
  c->d_adj_t = dalloc<double>((size_t)g.nunk * N);
}

// transposed stencil sum (FP64): out[j] (+)= sum_k coef[k] . in(j - offset_k), coefficient rows of shape (nin, nout)
bool has_reflect(const Ctx *c)
{
  for (int d = 0; d < c->g.ndim; d++)
    if (c->g.bc[d][0] == TGPU_BC_REFLECT || c->g.bc[d][1] == TGPU_BC_REFLECT) return true;
  return false;
}

// Transposed sums of the padded adjoint channels ch0.. into outs; with reflecting boundaries also the
// fold of the mirrored positions (vecdim[o] >= 0: output o is the vector component along that dimension).
void adj_conv(Ctx *c, int ch0, int nin, const DevStencil &st, const double *coef, double *const *outs, int nout,
              const int *vecdim = nullptr)
{
  tgpu::launch_conv<double>(c->d_adj_pad + (long)ch0 * c->dg.NP, c->dg.NP, nin, st.d_loff_neg, coef, st.L, outs, nout,
                            true, c->dg.N, c->stream);
  c->stats.conv_launches++;
  c->stats.kernel_launches++;
  if (has_reflect(c)) {
    int sm[tgpu::kMaxRb] = {0};
    for (int o = 0; o < nout; o++) sm[o] = (vecdim && vecdim[o] >= 0) ? 1 << vecdim[o] : 0;
    tgpu::launch_reflect_fold(c->d_adj_pad + (long)ch0 * c->dg.NP, c->dg.NP, nin, st.d_off, coef, st.L, outs, sm,
                              nout, c->stream);
    c->stats.kernel_launches++;
  }
}

void adj_pad(Ctx *c, int nch)
{
  tgpu::launch_pad<double>(c->d_adj_chan, c->d_adj_pad, nch, c->pads.zero_ext.bulk, c->pads.zero_ext.sign,
                           c->pads.zero_ext.zc, c->d_zero, has_reflect(c), c->stream);
  c->stats.kernel_launches++;
}

void jtv_device(Ctx *c, const double *d_w_in, double *d_out)
{
  need_state(c);
  const tgpu::DevGeom &g = c->dg;
  ensure_adjoint(c);
  const long N = g.N;
  const int nd = g.ndim;
  const int cpc = nd + 2;   // channels per component: A, B[d], C
  ck(cudaMemsetAsync(d_out, 0, sizeof(double) * (size_t)g.nunk * N, c->stream), "memset");
  // the averaged rows of coarsened nodes are transposed apart (at the end); the stencil rows of each
  // quadrature zone with that zone's stencils
  const double *d_w = d_w_in;
  if (c->coarse()) {
    copy_d(c, c->d_cscr, d_w_in, (size_t)g.nunk * N);
    tgpu::launch_zero_nodes(c->d_cscr, g.nunk, N, c->cr, c->stream);
    d_w = c->d_cscr;
  }
  // (a) density columns <- transposed weighted-density sums of the rb rows and mean-field sums of the MF rows
  {
    const int nch = g.ncomp * cpc + (g.attraction ? g.ncomp : 0);
    for (int z = 0; z < c->nzone; z++) {
      const std::vector<DevStencil> *sten = z == 0 ? c->sten : c->zsten[z];
      tgpu::launch_adj_rb_channels(d_w, c->d_adj_chan, c->stream);
      if (c->nzone > 1) tgpu::launch_zone_mask(c->d_adj_chan, nch, N, c->d_zone, z, c->stream);
      adj_pad(c, nch);
      for (int jc = 0; jc < g.ncomp; jc++) {
        double *o[1] = {d_out + (long)(g.first_rho + jc) * N};
        const DevStencil &sd = sten[TGPU_STEN_DELTA][jc], &st = sten[TGPU_STEN_THETA][jc];
        adj_conv(c, jc * cpc, 1 + nd, sd, sd.d_coef_adj, o, 1);
        adj_conv(c, jc * cpc + nd + 1, 1, st, st.d_coef_fwd, o, 1);
        if (g.attraction)
          for (int ic = 0; ic < g.ncomp; ic++) {
            const DevStencil &su = sten[TGPU_STEN_UATT][ic + g.ncomp * jc];
            adj_conv(c, g.ncomp * cpc + ic, 1, su, su.d_coef_fwd, o, 1);
          }
      }
    }
    // hard-wall boundary weights: the transpose of the forward correction
    if (g.hard_surf && !c->hw_targets.empty()) {
      tgpu::launch_hw_correct_t(d_w, g.attraction ? d_w + (long)g.first_mf * N : nullptr,
                                c->sten[TGPU_STEN_THETA].data(), c->sten[TGPU_STEN_DELTA].data(),
                                g.attraction ? c->sten[TGPU_STEN_UATT].data() : nullptr, g.ncomp, true,
                                g.attraction != 0, c->d_hw_targets, (int)c->hw_targets.size(), c->d_zero,
                                c->d_bnodes, c->d_fmask, d_out, c->stream);
      c->stats.kernel_launches++;
    }
    // density columns exist only off zero-density nodes
    tgpu::launch_mask_rows(d_out + (long)g.first_rho * N, nullptr, c->d_vext, c->d_zero, 0, g.ncomp, 1, c->stream);
  }
  // (b) rb columns <- H(n) g with g gathered from the EL rows of w by the transposed delta/theta sums
  {
    const int gst = nd + 2;   // per component: delta outputs (scalar, vector[d]) then theta
    ck(cudaMemsetAsync(c->d_adj_g, 0, sizeof(double) * (size_t)g.ncomp * gst * N, c->stream), "memset");
    for (int z = 0; z < c->nzone; z++) {
      const std::vector<DevStencil> *sten = z == 0 ? c->sten : c->zsten[z];
      tgpu::launch_mask_rows(c->d_adj_chan, d_w, c->d_vext, c->d_zero, g.first_rho, g.ncomp, 0, c->stream);
      if (c->nzone > 1) tgpu::launch_zone_mask(c->d_adj_chan, g.ncomp, N, c->d_zone, z, c->stream);
      adj_pad(c, g.ncomp);
      for (int ic = 0; ic < g.ncomp; ic++) {
        double *o[tgpu::kMaxRb];
        for (int q = 0; q < gst; q++) o[q] = c->d_adj_g + ((long)ic * gst + q) * N;
        const DevStencil &sd = sten[TGPU_STEN_DELTA][ic], &st = sten[TGPU_STEN_THETA][ic];
        const int vd[tgpu::kMaxRb] = {-1, 0, 1, 2};   // outputs: the scalar sum, then one per dimension
        adj_conv(c, ic, 1, sd, sd.d_coef_adj, o, 1 + nd, vd);
        adj_conv(c, ic, 1, st, st.d_coef_fwd, o + nd + 1, 1);
      }
    }
    tgpu::launch_jtv_local(c->d_x, c->d_vext, c->d_zero, d_w, c->d_adj_g, gst, 1, d_out, c->stream);
    c->stats.kernel_launches += 4;
  }
  if (c->coarse()) {
    tgpu::launch_coarse_rows_t(d_w_in, d_out, g.nunk, g.first_rho, g.ncomp, N, c->cr, c->stream);
    c->stats.kernel_launches++;
  }
}

// The transpose of the step on the other nodes (coarsened meshes): J_r = R J E with E the prolongation
// onto coarsened nodes and R the restriction to the other rows, so J_r^T w = E^T J^T (w, zero on
// coarsened rows); E^T folds the coarsened columns onto the nodes they are interpolated from.
void jtv_reduced(Ctx *c, const double *d_w, double *d_out)
{
  jtv_device(c, d_w, d_out);   // coarsened rows of w do not enter J_r
  if (c->coarse()) {
    tgpu::launch_prolong_t(d_out, 0, c->dg.nunk, c->dg.N, c->cr, c->stream);
    c->stats.kernel_launches++;
  }
}

// J^T lambda = g by GMRES on the transposed Schur complement
//   S^T = A22^T - A12^T A11^-T A21^T,  right-hand side g2 - A12^T A11^-T g1,
//   lambda1 = A11^-T (g1 - A21^T lambda2),
// with every block product taken from J^T on masked full vectors and
// A11^-T [u_ind; u_dep] = [-u_ind - B^T u_dep; -u_dep].
// S^T v2: t = J^T [0; v2]; y1 = A11^-T (t_block1); S^T v2 = t_rho - (J^T [y1; 0])_rho
void schur_t_device(Ctx *c, const double *d_v2, double *d_y2)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  const size_t n = (size_t)g.nunk * N;
  double *full = c->d_adj_v, *t = c->d_adj_t;
  ck(cudaMemsetAsync(full, 0, n * sizeof(double), c->stream), "memset");
  copy_d(c, full + (long)g.first_rho * N, d_v2, (size_t)g.ncomp * N);
  jtv_reduced(c, full, t);
  copy_d(c, d_y2, t + (long)g.first_rho * N, (size_t)g.ncomp * N);   // A22^T v2 - nothing else yet
  tgpu::launch_a11inv_t(t, full, c->stream);                           // y1 in block-1 rows, density rows 0
  jtv_reduced(c, full, t);                                             // t_rho = A12^T y1
  tgpu::launch_axpby(d_y2, -1.0, t + (long)g.first_rho * N, 1.0, (long)g.ncomp * N, c->stream);
  c->stats.schur_applies++;
}

int adjoint_solve_device(Ctx *c, const double *d_g_in, double *d_lam, double tol, int maxit, int *iters,
                         double *relres)
{
  need_state(c);
  ensure_adjoint(c);
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  const size_t n = (size_t)g.nunk * N;
  double *full = c->d_adj_v, *t = c->d_adj_t;
  // coarsened meshes: the adjoint of the step on the other nodes, right-hand side E^T g
  const double *d_g = d_g_in;
  if (c->coarse()) {
    if (!c->d_cscr2) c->d_cscr2 = dalloc<double>(n);
    copy_d(c, c->d_cscr2, d_g_in, n);
    tgpu::launch_prolong_t(c->d_cscr2, 0, g.nunk, N, c->cr, c->stream);
    d_g = c->d_cscr2;
  }
  // rhs2 = g2 - A12^T A11^-T g1
  tgpu::launch_a11inv_t(d_g, full, c->stream);
  jtv_reduced(c, full, t);
  copy_d(c, c->d_b2s, d_g + (long)g.first_rho * N, (size_t)g.ncomp * N);
  tgpu::launch_axpby(c->d_b2s, -1.0, t + (long)g.first_rho * N, 1.0, (long)g.ncomp * N, c->stream);
  c->gmres_transpose = true;
  int st;
  try {
    st = gmres(c, c->d_b2s, c->d_gx, tol, maxit, iters, relres);
  } catch (...) {
    c->gmres_transpose = false;
    throw;
  }
  c->gmres_transpose = false;
  // lambda1 = A11^-T (g1 - A21^T lambda2)
  ck(cudaMemsetAsync(full, 0, n * sizeof(double), c->stream), "memset");
  copy_d(c, full + (long)g.first_rho * N, c->d_gx, (size_t)g.ncomp * N);
  jtv_reduced(c, full, t);                                  // block-1 rows: A21^T lambda2
  tgpu::launch_axpby(t, 1.0, d_g, -1.0, (long)n, c->stream);  // t = g - J^T[0; lambda2] (block-1 rows used)
  tgpu::launch_a11inv_t(t, d_lam, c->stream);
  copy_d(c, d_lam + (long)g.first_rho * N, c->d_gx, (size_t)g.ncomp * N);
  return st;
}

// ---- objectives: Omega_s and Gamma_ex, their gradients, sensitivities to V_ext ----

void need_integ(Ctx *c)
{
  need_final(c);
  if (!c->have_integ) throw Error(TGPU_ERR_STATE, "no integration weights: call tgpu_set_integration first");
}

// mean-field sums S_ic = sum_jc sum_o u_ic,jc(o) rho_jc(i+o) of the densities of d_x into d_conv rows nrb..
const double *attraction_sums(Ctx *c, const double *d_x)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  if (!g.attraction) return c->d_conv;   // unused
  double *S = c->d_conv + (long)g.nrb * N;
  ck(cudaMemsetAsync(S, 0, sizeof(double) * (size_t)g.ncomp * N, c->stream), "memset");
  pad(c, d_x + (long)g.first_rho * N, c->pads.rho_res, false);
  for (int jc = 0; jc < g.ncomp; jc++)
    for (int ic = 0; ic < g.ncomp; ic++) {
      double *o[1] = {S + (long)ic * N};
      conv(c, jc, 1, c->sten[TGPU_STEN_UATT][ic + g.ncomp * jc], false, o, 1, false);
    }
  // hard-wall boundary weights of the mean-field stencils (int_stencil, src/dft_energy_CLSintsten.c:73-129)
  if (g.hard_surf && !c->hw_targets.empty()) {
    tgpu::launch_hw_correct(d_x + (long)g.first_rho * N, N, 0, nullptr, nullptr, c->sten[TGPU_STEN_UATT].data(),
                            g.ncomp, false, true, c->d_hw_targets, (int)c->hw_targets.size(), c->d_zero,
                            c->d_bnodes, c->d_fmask, c->d_conv, c->stream);
    c->stats.kernel_launches++;
  }
  return S;
}

// ATTInA22Block = 1 (the mean field summed into the Euler-Lagrange rows, src/dft_fill_EL.c:143-161,
// linsolver_setup_HSTYPE's A22 block, src/dft_linsolver_setup.c:234-236): the caller's vectors have no
// mean-field rows.  Inside, the mean field stays an unknown of its own, so every kernel is shared with
// ATTInA22Block = 0.  With J = [[J_ee, C], [B, -I]] (C: the mean field in the EL rows, B: its stencil sums)
// the caller's Jacobian is J_ee + C B, and at the boundary
//   states and perturbations v  -> [v; B v]        (mean-field rows equal to their attraction sums)
//   right-hand sides b of J, J^T -> [b; 0]
//   arguments w of J^T          -> [w; C^T w]      (mean-field rows equal to the EL rows off zero-density rows)
// and results drop the mean-field rows.  The density block of the Schur complement is the same in both forms.
void a22_mf_sums(Ctx *c, const double *x, bool jac, double *mf)
{
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  ck(cudaMemsetAsync(mf, 0, sizeof(double) * (size_t)g.ncomp * N, c->stream), "memset");
  pad(c, x + (long)g.first_rho * N, jac ? c->pads.rho_jac : c->pads.rho_res, false);
  for (int jc = 0; jc < g.ncomp; jc++)
    for (int ic = 0; ic < g.ncomp; ic++) {
      double *o[1] = {mf + (long)ic * N};
      conv(c, jc, 1, c->sten[TGPU_STEN_UATT][ic + g.ncomp * jc], false, o, 1, false);
    }
  // nodes of the coarser quadrature zones take their own zone's sums (load_mean_field with the node's
  // zone, src/dft_fill_EL.c:156-159)
  for (int z = 1; z < c->nzone; z++) {
    ck(cudaMemsetAsync(c->d_zbuf, 0, sizeof(double) * (size_t)g.ncomp * N, c->stream), "memset");
    for (int jc = 0; jc < g.ncomp; jc++)
      for (int ic = 0; ic < g.ncomp; ic++) {
        double *o[1] = {c->d_zbuf + (long)ic * N};
        conv(c, jc, 1, c->zsten[z][TGPU_STEN_UATT][ic + g.ncomp * jc], false, o, 1, false);
      }
    tgpu::launch_zone_merge(c->d_zbuf, mf, g.ncomp, N, c->d_zone, z, c->stream);
    c->stats.kernel_launches++;
  }
  if (g.hard_surf && !c->hw_targets.empty()) {
    tgpu::launch_hw_correct(x + (long)g.first_rho * N, N, 0, nullptr, nullptr, c->sten[TGPU_STEN_UATT].data(),
                            g.ncomp, false, true, c->d_hw_targets, (int)c->hw_targets.size(), c->d_zero,
                            c->d_bnodes, c->d_fmask, mf - (long)g.nrb * N, c->stream);
    c->stats.kernel_launches++;
  }
}

enum { A22_SUMS = 0, A22_JAC_SUMS = 1, A22_ZERO = 2, A22_EL = 3 };

// the internal-layout copy of a caller vector in scratch slot (the caller's own vector without ATTInA22Block)
const double *a22_in(Ctx *c, const double *ext, int how, int slot)
{
  if (!c->a22) return ext;
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  double *in = c->d_a22[slot];
  copy_d(c, in, ext, (size_t)c->nunk_ext * N);
  double *mf = in + (long)g.first_mf * N;
  if (how == A22_ZERO) ck(cudaMemsetAsync(mf, 0, sizeof(double) * (size_t)g.ncomp * N, c->stream), "memset");
  else if (how == A22_EL) {  // C^T w: the EL rows, except rows that hold no mean field (zero-density rows,
                            // averaged rows of coarsened nodes)
    tgpu::launch_mask_rows(mf, ext, c->d_vext, c->d_zero, g.first_rho, g.ncomp, 0, c->stream);
    if (c->coarse()) tgpu::launch_zero_nodes(mf, g.ncomp, N, c->cr, c->stream);
  } else {
    a22_mf_sums(c, in, how == A22_JAC_SUMS, mf);
  }
  return in;
}

// where an internal-layout result goes (scratch slot, or the caller's vector), and its copy back
double *a22_out_buf(Ctx *c, double *ext, int slot) { return c->a22 ? c->d_a22[slot] : ext; }
void a22_out(Ctx *c, const double *in, double *ext)
{
  if (c->a22) copy_d(c, ext, in, (size_t)c->nunk_ext * c->dg.N);
}

void objectives_device(Ctx *c, const double *d_x, double *omega_s, double *gamma_ex)
{
  need_integ(c);
  const tgpu::DevGeom &g = c->dg;
  const double *S = attraction_sums(c, d_x);
  const int nb = tgpu::reduce_blocks(g.N);
  tgpu::launch_objectives(d_x, c->d_vext, S, c->d_wf, c->d_wb, c->oc, g.ncomp, c->d_partial, nb, c->d_red, c->stream);
  c->stats.kernel_launches += 2;
  red_to_host(c, 1 + g.ncomp);
  if (omega_s) *omega_s = c->h_red[0];
  if (gamma_ex)
    for (int ic = 0; ic < g.ncomp; ic++) gamma_ex[ic] = c->h_red[1 + ic];
}

// dF/dx ([nunk][N]) and the explicit dF/dV_ext ([ncomp][N]) of F = Omega_s (kind 0) or Gamma_ex[icomp] (kind 1)
void objective_grad_device(Ctx *c, const double *d_x, int kind, int icomp, double *d_gx, double *d_gv)
{
  need_integ(c);
  const tgpu::DevGeom &g = c->dg;
  const long N = g.N;
  if (kind != TGPU_OBJ_OMEGA && kind != TGPU_OBJ_GAMMA) throw Error(TGPU_ERR_ARG, "objective kind");
  if (kind == TGPU_OBJ_GAMMA && (icomp < 0 || icomp >= g.ncomp)) throw Error(TGPU_ERR_ARG, "component index");
  const bool att = kind == TGPU_OBJ_OMEGA && g.attraction;
  if (att) ensure_adjoint(c);
  const double *S = att ? attraction_sums(c, d_x) : c->d_conv;
  tgpu::launch_objective_grad(d_x, c->d_vext, S, c->d_wf, c->d_wb, c->oc, kind, icomp, d_gx, d_gv,
                              att ? c->d_adj_chan : nullptr, c->stream);
  c->stats.kernel_launches++;
  if (att) {
    // the other nodes' mean-field terms: d/drho_jc(j) sum_i wf_ic rho_ic(i) S_ic(i) / 2 =
    // transposed attraction sums of wf rho / 2 (the kernel stored wf rho on rho > 0 nodes)
    tgpu::launch_scale(c->d_adj_chan, c->d_adj_chan, 0.5, (long)g.ncomp * N, c->stream);
    adj_pad(c, g.ncomp);
    for (int jc = 0; jc < g.ncomp; jc++) {
      double *o[1] = {d_gx + (long)(g.first_rho + jc) * N};
      for (int ic = 0; ic < g.ncomp; ic++) {
        const DevStencil &su = c->sten[TGPU_STEN_UATT][ic + g.ncomp * jc];
        adj_conv(c, ic, 1, su, su.d_coef_fwd, o, 1);
      }
    }
    if (g.hard_surf && !c->hw_targets.empty()) {
      tgpu::launch_hw_correct_t(nullptr, c->d_adj_chan, nullptr, nullptr, c->sten[TGPU_STEN_UATT].data(), g.ncomp,
                                false, true, c->d_hw_targets, (int)c->hw_targets.size(), c->d_zero, c->d_bnodes,
                                c->d_fmask, d_gx, c->stream);
      c->stats.kernel_launches++;
    }
    // densities at zero-density nodes are not unknowns of the sums (int_stencil skips them)
    tgpu::launch_mask_rows(d_gx + (long)g.first_rho * N, nullptr, c->d_vext, c->d_zero, 0, g.ncomp, 1, c->stream);
    c->stats.kernel_launches += 2;
  }
}

void ensure_obj(Ctx *c)
{
  if (c->d_obj_gx) return;
  const size_t N = c->dg.N, U = c->dg.nunk;
  c->d_obj_gx = dalloc<double>(U * N);
  c->d_obj_lam = dalloc<double>(U * N);
  c->d_obj_R = dalloc<double>(U * N);
  c->d_obj_gv = dalloc<double>((size_t)c->dg.ncomp * N);
}

// dF/dV_ext at the state d_x: Jacobian at d_x (FP64 fill), J^T lambda = dF/dx, dF/dV = dF/dV|_x - lambda_EL
// The sensitivities need the derivative of the residual itself: the exact FMT second
// derivatives for the duration of a gradient, whatever tgpu_set_jacobian_form chose.
struct ExactJacScope {
  Ctx *c;
  int saved;
  explicit ExactJacScope(Ctx *c_) : c(c_), saved(c_->dg.jac_exact)
  {
    if (!saved) {
      c->dg.jac_exact = 1;
      tgpu::upload_geom(c->dg, c->stream);
    }
  }
  ~ExactJacScope()
  {
    if (!saved) {
      c->dg.jac_exact = 0;
      tgpu::upload_geom(c->dg, c->stream);
    }
  }
};

int grad_vext_device(Ctx *c, const double *d_x, int kind, int icomp, double tol, int maxit, double *d_out, int *iters)
{
  ExactJacScope exact(c);
  need_integ(c);
  ensure_obj(c);
  fill_arith(c, d_x, c->d_obj_R, 0, TGPU_FILL_FP64);
  objective_grad_device(c, c->d_x, kind, icomp, c->d_obj_gx, c->d_obj_gv);
  double rr = 0.0;
  const int st = adjoint_solve_device(c, c->d_obj_gx, c->d_obj_lam, tol, maxit, iters, &rr);
  tgpu::launch_vext_sens(c->d_obj_lam, c->d_obj_gv, c->d_vext, c->d_zero, d_out, c->stream);
  c->stats.kernel_launches++;
  return st;
}

// A bounded wait of the tensor-core kernel that ran out leaves a flag on the device.
void tc_check(Ctx *c)
{
  if (!c->tc_ready) return;
  int err = 0;
  ck(cudaMemcpyAsync(&err, c->tcslab.d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "d2h");
  ck(cudaStreamSynchronize(c->stream), "sync");
  if (err) {
    ck(cudaMemsetAsync(c->tcslab.d_err, 0, sizeof(int), c->stream), "memset");
    throw Error(TGPU_ERR_CUDA, "tensor-core stencil sum: a bounded wait ran out (code " + std::to_string(err) + ")");
  }
}

// Host-pointer wrappers: copy in, run on the device, copy out, synchronise.
void h2d(Ctx *c, double *d, const double *h, size_t n)
{
  ck(cudaMemcpyAsync(d, h, n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "h2d");
}
void d2h(Ctx *c, double *h, const double *d, size_t n)
{
  ck(cudaMemcpyAsync(h, d, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "d2h");
  ck(cudaStreamSynchronize(c->stream), "sync");
  tc_check(c);
}

// Regroup a 3-D stencil by z offset into x-lines of constant oy for the FP32
// slab kernel: per plane {first line, count, first weight, weight count} and
// {oz, oy_lo, oy_hi, 0}; per line {oy - oy_lo, ox_min + h0, blocks of 8, weight offset}.
DevStencil::Lines build_lines(const DevStencil &st, const std::vector<double> &coef, const tgpu::DevGeom &dg,
                              cudaStream_t s, int ncoef = 1, int nin = 1)
{
  // per point: its x offset and the index of its coefficient row
  std::map<int, std::map<int, std::vector<std::pair<int, int>>>> planes;
  for (int k = 0; k < st.L; k++) {
    const short *o = &st.off[(size_t)k * 3];
    planes[o[2]][o[1]].push_back({o[0], k});
  }
  std::vector<int4> pd, lines;
  std::vector<float> w, w_lo;
  DevStencil::Lines L;
  for (auto &pkv : planes) {
    const int oz = pkv.first;
    const int oy_lo = pkv.second.begin()->first, oy_hi = pkv.second.rbegin()->first;
    const int first_line = (int)lines.size(), first_w = (int)w.size();
    for (auto &ykv : pkv.second) {
      int xmin = 1 << 30, xmax = -(1 << 30);
      for (auto &e : ykv.second) { xmin = std::min(xmin, e.first); xmax = std::max(xmax, e.first); }
      const int nb = (xmax - xmin + 1 + 7) / 8;
      lines.push_back({ykv.first - oy_lo, xmin + dg.h[0], nb, (int)w.size()});
      const size_t base = w.size();
      w.resize(base + (size_t)nb * 8, 0.0f);
      w_lo.resize(base + (size_t)nb * 8, 0.0f);
      for (auto &e : ykv.second) {
        const double v = coef[(size_t)e.second * ncoef];
        const float hi = (float)v;
        w[base + (e.first - xmin)] = hi;
        w_lo[base + (e.first - xmin)] = (float)(v - (double)hi);
      }
    }
    const int nl = (int)lines.size() - first_line, nw = (int)w.size() - first_w;
    pd.push_back({first_line, nl, first_w, nw});
    pd.push_back({oz, oy_lo, oy_hi, 0});
    L.max_rows = std::max(L.max_rows, tgpu::kSlabTileY + oy_hi - oy_lo);
    L.max_lines = std::max(L.max_lines, nl);
    L.max_w = std::max(L.max_w, nw);
  }
  // columns: 128 outputs + 2 h0 halo + 16 for the window overrun of the last block of 8
  L.ncols = tgpu::kSlabTileX + 2 * dg.h[0] + 16;
  int pitch = L.ncols + (L.ncols >> 3) + 1;
  while (pitch % 32 != 16) pitch++;
  L.pitch = pitch;
  L.nplanes = (int)planes.size();
  L.d_planes = upload(pd, s);
  L.d_lines = upload(lines, s);
  L.ncoef = ncoef;
  L.wstride = (int)w.size();
  if (ncoef == 1) {
    const size_t smem = sizeof(float) * ((size_t)L.max_rows * pitch + L.max_w) + sizeof(int4) * L.max_lines;
    if (smem > 200 * 1024) throw Error(TGPU_ERR_UNSUPPORTED, "stencil plane too large for the shared-memory slab");
    L.d_w = upload(w, s);
    L.d_w_lo = upload(w_lo, s);
    L.ff_ok = tgpu::conv_slab_ff_smem(L.pitch, L.max_rows, L.max_lines, L.max_w) <= 220 * 1024;
  } else {
    // coefficient c of every point at w + c * wstride, in the line layout of coefficient 0
    std::vector<float> wall((size_t)ncoef * w.size(), 0.0f);
    size_t pos = 0;
    for (auto &pkv : planes)
      for (auto &ykv : pkv.second) {
        int xmin = 1 << 30, xmax = -(1 << 30);
        for (auto &e : ykv.second) { xmin = std::min(xmin, e.first); xmax = std::max(xmax, e.first); }
        const int nb = (xmax - xmin + 1 + 7) / 8;
        for (auto &e : ykv.second)
          for (int cc = 0; cc < ncoef; cc++)
            wall[(size_t)cc * w.size() + pos + (e.first - xmin)] = (float)coef[(size_t)e.second * ncoef + cc];
        pos += (size_t)nb * 8;
      }
    L.d_w = upload(wall, s);
    L.mc_ok = tgpu::conv_slab_mc_smem(nin, ncoef, L.pitch, L.max_rows, L.max_lines, L.max_w) <= 200 * 1024;
  }
  return L;
}

// ---- mesh coarsening: averaged rows and the prolongation onto coarsened nodes ----

// One step along dimension d (s = +1 or -1) from a node under the boundary conditions: a node index,
// -1 beyond an IN_BULK boundary (-3 beyond the high one of a phase interface, the RTF state) or -2 inside
// a wall (offset_to_node_box, src/dft_mesh_lib.c:203-297, for unit offsets).
long step_node(const Ctx *c, long node, int d, int s)
{
  const long bulk_hi = c->g.interface == 2 ? tgpu::kSentBulkHi : tgpu::kSentBulk;
  const tgpu::DevGeom &dg = c->dg;
  long ijk[3] = {node % dg.nx[0], (node / dg.nx[0]) % dg.nx[1], node / ((long)dg.nx[0] * dg.nx[1])};
  const long n = dg.nx[d];
  long q = ijk[d] + s;
  const int bl = c->g.bc[d][0], br = c->g.bc[d][1];
  if (q < 0) {
    if (bl == TGPU_BC_IN_BULK) return -1;
    if (bl == TGPU_BC_IN_WALL) return -2;
    q = bl == TGPU_BC_REFLECT ? -q : q + n;
  } else if (q >= n) {
    if (br == TGPU_BC_IN_BULK) return bulk_hi;
    if (br == TGPU_BC_IN_WALL) return -2;
    q = br == TGPU_BC_REFLECT ? 2 * (n - 1) - q : q - n;
  }
  if (q < 0 || q >= n) throw Error(TGPU_ERR_UNSUPPORTED, "mesh too small for its coarsening");
  ijk[d] = q;
  return ijk[0] + dg.nx[0] * (ijk[1] + (long)dg.nx[1] * ijk[2]);
}

// Flags of Mesh_coarsen_flag beyond zones and averaging axes (src/dft_mesh.c:2788-2850)
constexpr int kFlagPB = TGPU_FLAG_PB, kFlagBulk = TGPU_FLAG_BULK, kFlag1dbc = TGPU_FLAG_1DBC;

// a node whose rows are not filled but follow other nodes: averaged along an axis, or the 1-D boundary copy
inline bool coarse_flag(int f) { return f == kFlag1dbc || (f < 0 && f >= -3); }

// the node on the line through the origin along dim_1dbc with the same coordinate along it
// (load_coarse_node_1dim, src/dft_fill_coarse.c:43-45)
long line_node(const Ctx *c, long node)
{
  const tgpu::DevGeom &dg = c->dg;
  const long ijk[3] = {node % dg.nx[0], (node / dg.nx[0]) % dg.nx[1], node / ((long)dg.nx[0] * dg.nx[1])};
  long jk[3] = {0, 0, 0};
  jk[c->dim_1dbc] = ijk[c->dim_1dbc];
  return jk[0] + dg.nx[0] * (jk[1] + (long)dg.nx[1] * jk[2]);
}

// locate_neighbor_unks (src/dft_fill_coarse.c:103-123): the averaged row's terms (column, weight a) of a
// coarsened node; with two zones a coarsened neighbour gives way to its own neighbours.  Wall columns
// (value 0, no Jacobian entry) are left out.  With two zones the reference recurses into a neighbour with
// a 1-D boundary, BULK_ZONE or PB_ZONE flag as if the flag were an axis (reading past its offset table), so
// that pattern is refused.
void coarse_row_terms(const Ctx *c, long node, double a, int depth, std::vector<std::pair<long, double>> &out)
{
  if (depth > 8) throw Error(TGPU_ERR_UNSUPPORTED, "coarsening pattern");
  const int d = -c->h_zone[node] - 1;
  for (int s : {1, -1}) {
    const long j = step_node(c, node, d, s);
    if (j >= 0 && c->h_zone[j] < 0 && c->nzone == 2) {
      if (c->h_zone[j] < -3)
        throw Error(TGPU_ERR_UNSUPPORTED, "with two zones, an averaged node next to a 1-D boundary, BULK_ZONE or "
                                          "PB_ZONE node");
      coarse_row_terms(c, j, 0.5 * a, depth + 1, out);
    } else if (j != -2) {
      out.push_back({j, a});
    }
  }
}

// Values beyond the low and the high IN_BULK boundary per unknown (constant_boundary, src/dft_utils.c:
// 89-110): the bulk densities (Rho_b, or Rho_b_LBB / _RTF of a phase interface) and Rhobar_b; mean-field
// unknowns 0 (the reference leaves them undefined there).  Called again when the bulk state moves.
void upload_cbulk(Ctx *c)
{
  const tgpu::DevGeom &dg = c->dg;
  const tgpu_geometry &g = c->g;
  const int nrb = dg.nrb;
  std::vector<double> cb(2 * (size_t)dg.nunk, 0.0);
  for (int side = 0; side < 2; side++) {
    double *o = cb.data() + (size_t)side * dg.nunk;
    for (int ic = 0; ic < dg.ncomp; ic++)
      o[dg.first_rho + ic] = g.interface == 2 ? (side ? g.rho_b_rtf[ic] : g.rho_b_lbb[ic]) : g.rho_b[ic];
    const size_t off = c->h_rb_bulk.size() >= 2 * (size_t)nrb ? (size_t)side * nrb : 0;
    for (int k = 0; k < nrb && off + k < c->h_rb_bulk.size(); k++) o[dg.first_rb + k] = c->h_rb_bulk[off + k];
  }
  if (!c->d_cbulk) c->d_cbulk = dalloc<double>(cb.size());
  ck(cudaMemcpyAsync(c->d_cbulk, cb.data(), cb.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream), "h2d");
  ck(cudaStreamSynchronize(c->stream), "sync");
}

// The values at coarsened nodes that satisfy every averaged row, as weights on the other nodes (and on the
// bulk, column -1).  Coarsened nodes with one flag form runs along their averaging axis; each run is a
// small linear system in its own nodes, given its outside neighbours, and runs are solved after the runs
// they lean on (a cyclic dependence is rejected).
void build_coarse(Ctx *c)
{
  const tgpu::DevGeom &dg = c->dg;
  const long N = dg.N;
  std::vector<int> cnode, pos(N, -1);
  for (long i = 0; i < N; i++)
    if (coarse_flag(c->h_zone[i])) {
      pos[i] = (int)cnode.size();
      cnode.push_back((int)i);
    }
  const int nc = (int)cnode.size();
  c->cr.ncoarse = nc;
  if (nc == 0) return;
  // averaged rows fac (x_c - sum_k a_k x_k), and the 1-D boundary rows x_c - x_line (fac 1 on every unknown)
  std::vector<int> rptr(1, 0);
  std::vector<long> rcol;
  std::vector<double> ra;
  std::vector<signed char> ckind(nc, 0);
  for (int k = 0; k < nc; k++) {
    std::vector<std::pair<long, double>> t;
    if (c->h_zone[cnode[k]] == kFlag1dbc) {
      const long ln = line_node(c, cnode[k]);
      if (c->h_zone[ln] == kFlag1dbc) throw Error(TGPU_ERR_ARG, "a 1-D boundary node on its own line");
      t.push_back({ln, 1.0});
      ckind[k] = 1;
    } else {
      coarse_row_terms(c, cnode[k], 0.5, 0, t);
    }
    for (auto &e : t) {
      rcol.push_back(e.first);
      ra.push_back(e.second);
    }
    rptr.push_back((int)rcol.size());
  }
  // prolongation by runs
  typedef std::vector<std::pair<long, double>> Expr;
  std::vector<Expr> expr(nc);
  std::vector<char> state(nc, 0);
  std::function<void(int)> solve = [&](int k0) {
    if (state[k0] == 2) return;
    if (state[k0] == 1) throw Error(TGPU_ERR_UNSUPPORTED, "cyclic coarsening pattern");
    if (c->h_zone[cnode[k0]] == kFlag1dbc) {   // the line node's value (its own prolongation when averaged)
      const long ln = line_node(c, cnode[k0]);
      state[k0] = 1;
      if (coarse_flag(c->h_zone[ln])) {
        solve(pos[ln]);
        expr[k0] = expr[pos[ln]];
      } else {
        expr[k0].assign(1, {ln, 1.0});
      }
      state[k0] = 2;
      return;
    }
    const int flag = c->h_zone[cnode[k0]], d = -flag - 1;
    std::vector<int> run(1, k0);
    std::map<int, int> in_run{{k0, 0}};
    for (size_t q = 0; q < run.size(); q++)
      for (int s : {1, -1}) {
        const long j = step_node(c, cnode[run[q]], d, s);
        if (j >= 0 && c->h_zone[j] == flag && !in_run.count(pos[j])) {
          in_run[pos[j]] = (int)run.size();
          run.push_back(pos[j]);
        }
      }
    const int m = (int)run.size();
    if (m > 4096) throw Error(TGPU_ERR_UNSUPPORTED, "coarsening pattern");
    for (int k : run) state[k] = 1;
    std::vector<double> A((size_t)m * m, 0.0);
    std::vector<long> ext;
    std::map<long, int> ext_idx;
    std::vector<std::vector<std::pair<int, double>>> brow(m);
    for (int r = 0; r < m; r++) {
      A[(size_t)r * m + r] += 1.0;
      for (int s : {1, -1}) {
        const long j = step_node(c, cnode[run[r]], d, s);
        if (j == -2) continue;
        if (j >= 0 && c->h_zone[j] == flag) {
          A[(size_t)r * m + in_run.at(pos[j])] -= 0.5;
          continue;
        }
        if (j >= 0 && coarse_flag(c->h_zone[j])) solve(pos[j]);
        auto it = ext_idx.find(j);
        int e;
        if (it == ext_idx.end()) {
          e = (int)ext.size();
          ext_idx[j] = e;
          ext.push_back(j);
        } else {
          e = it->second;
        }
        brow[r].push_back({e, 0.5});
      }
    }
    const int E = (int)ext.size();
    std::vector<double> X((size_t)m * E, 0.0);
    for (int r = 0; r < m; r++)
      for (auto &b : brow[r]) X[(size_t)r * E + b.first] += b.second;
    // Gaussian elimination with partial pivoting on [A | X]
    for (int col = 0; col < m; col++) {
      int piv = col;
      for (int r = col + 1; r < m; r++)
        if (std::fabs(A[(size_t)r * m + col]) > std::fabs(A[(size_t)piv * m + col])) piv = r;
      if (std::fabs(A[(size_t)piv * m + col]) < 1e-12) throw Error(TGPU_ERR_UNSUPPORTED, "singular coarsening run");
      if (piv != col) {
        for (int q = 0; q < m; q++) std::swap(A[(size_t)piv * m + q], A[(size_t)col * m + q]);
        for (int q = 0; q < E; q++) std::swap(X[(size_t)piv * E + q], X[(size_t)col * E + q]);
      }
      for (int r = 0; r < m; r++) {
        if (r == col) continue;
        const double f = A[(size_t)r * m + col] / A[(size_t)col * m + col];
        if (f == 0.0) continue;
        for (int q = col; q < m; q++) A[(size_t)r * m + q] -= f * A[(size_t)col * m + q];
        for (int q = 0; q < E; q++) X[(size_t)r * E + q] -= f * X[(size_t)col * E + q];
      }
    }
    for (int r = 0; r < m; r++) {
      std::map<long, double> acc;
      const double inv = 1.0 / A[(size_t)r * m + r];
      for (int e = 0; e < E; e++) {
        const double w = X[(size_t)r * E + e] * inv;
        if (w == 0.0) continue;
        const long j = ext[e];
        if (j >= 0 && coarse_flag(c->h_zone[j]))
          for (auto &t : expr[pos[j]]) acc[t.first] += w * t.second;
        else
          acc[j] += w;
      }
      expr[run[r]].assign(acc.begin(), acc.end());
    }
    for (int k : run) state[k] = 2;
  };
  for (int k = 0; k < nc; k++) solve(k);
  std::vector<int> pptr(1, 0);
  std::vector<long> pcol;
  std::vector<double> pw;
  for (int k = 0; k < nc; k++) {
    for (auto &t : expr[k]) {
      pcol.push_back(t.first);
      pw.push_back(t.second);
    }
    pptr.push_back((int)pcol.size());
  }
  c->cr.d_node = upload(cnode, c->stream);
  c->cr.d_rptr = upload(rptr, c->stream);
  c->cr.d_rcol = upload(rcol, c->stream);
  c->cr.d_ra = upload(ra, c->stream);
  c->cr.d_pptr = upload(pptr, c->stream);
  c->cr.d_pcol = upload(pcol, c->stream);
  c->cr.d_pw = upload(pw, c->stream);
  c->cr.d_kind = upload(ckind, c->stream);
  upload_cbulk(c);
  c->d_cscr = dalloc<double>((size_t)dg.nunk * N);
}

void build_device_tables(Ctx *c)
{
  tgpu_geometry &g = c->g;
  tgpu::DevGeom &dg = c->dg;
  const int nd = g.ndim;
  // halo = largest stencil reach per dimension
  int h[3] = {0, 0, 0};
  for (int z = 0; z < c->nzone; z++)
    for (int t = 0; t < 3; t++)
      for (auto &st : (z == 0 ? c->sten[t] : c->zsten[z][t]))
        for (int k = 0; k < st.L; k++)
          for (int d = 0; d < nd; d++) h[d] = std::max(h[d], std::abs((int)st.off[(size_t)k * nd + d]));
  long NP = 1;
  for (int d = 0; d < 3; d++) {
    dg.nx[d] = d < nd ? g.nx[d] : 1;
    dg.h[d] = d < nd ? h[d] : 0;
    dg.P[d] = dg.nx[d] + 2 * dg.h[d];
    dg.esize[d] = d < nd ? g.esize[d] : 0.0;
  }
  dg.pstride[0] = 1;
  dg.pstride[1] = dg.P[0];
  dg.pstride[2] = (long)dg.P[0] * dg.P[1];
  NP = (long)dg.P[0] * dg.P[1] * dg.P[2];
  dg.NP = NP;
  for (int d = 0; d < 3; d++) {
    std::vector<int> m = d < nd ? build_map(dg.nx[d], dg.h[d], g.bc[d][0], g.bc[d][1], g.interface == 2)
                                : std::vector<int>{0};
    c->d_map[d] = upload(m, c->stream);
    dg.map[d] = c->d_map[d];
  }
  // stencil tables; the coarser zones' stencils get the generic tables only
  auto prep = [&](DevStencil &st, int t, int idx, bool fast) {
      if (st.L == 0) return;
      std::vector<int> loff(st.L);
      std::vector<short> off3((size_t)st.L * 3, 0);
      for (int k = 0; k < st.L; k++) {
        long o = 0;
        for (int d = 0; d < nd; d++) {
          o += (long)st.off[(size_t)k * nd + d] * dg.pstride[d];
          off3[(size_t)k * 3 + d] = st.off[(size_t)k * nd + d];
        }
        loff[k] = (int)o;
      }
      st.d_loff = upload(loff, c->stream);
      std::vector<int> lneg(loff.size());
      for (size_t k = 0; k < loff.size(); k++) lneg[k] = -loff[k];
      st.d_loff_neg = upload(lneg, c->stream);
      st.d_off = upload(off3, c->stream);
      st.d_w = upload(st.w, c->stream);
      if (!st.hw.empty()) st.d_hw = upload(st.hw, c->stream);
      std::vector<double> fwd, tr;
      if (t == TGPU_STEN_THETA) {
        const int jc = idx;
        st.nout_fwd = 1;
        for (int k = 0; k < st.L; k++) fwd.push_back(g.fac_overlap[jc] * st.w[k]);
        st.nin_tr = 1;
        tr = st.w;
      } else if (t == TGPU_STEN_DELTA) {
        const int jc = idx;
        const double f = g.fac_overlap[jc];
        st.nout_fwd = g.single_size ? 1 + nd : 3 + 2 * nd;  // n2 [n1 n0] V2[d] [V1[d]]
        for (int k = 0; k < st.L; k++) {
          const double w = st.w[k];
          fwd.push_back(f * w);
          if (!g.single_size) {
            fwd.push_back(f * g.inv_4pir[jc] * w);
            fwd.push_back(f * g.inv_4pirsq[jc] * w);
          }
          for (int d = 0; d < nd; d++) fwd.push_back(f * ((double)st.off[(size_t)k * nd + d] * g.esize[d] * g.inv_rad[jc]) * w);
          if (!g.single_size)
            for (int d = 0; d < nd; d++)
              fwd.push_back(f * g.inv_4pir[jc] * ((double)st.off[(size_t)k * nd + d] * g.esize[d] * g.inv_rad[jc]) * w);
        }
        st.nin_tr = 1 + nd;
        std::vector<double> adj;   // [L][1+nd]: fac (w, e_d w), the forward scalar and vector rows
        for (int k = 0; k < st.L; k++) {
          adj.push_back(f * st.w[k]);
          for (int d = 0; d < nd; d++) adj.push_back(f * ((double)st.off[(size_t)k * nd + d] * g.esize[d] * g.inv_rad[jc]) * st.w[k]);
        }
        st.d_coef_adj = upload(adj, c->stream);
        for (int k = 0; k < st.L; k++) {
          tr.push_back(st.w[k]);
          for (int d = 0; d < nd; d++) tr.push_back(-st.w[k] * (double)st.off[(size_t)k * nd + d] * g.esize[d] * g.inv_rad[idx]);
        }
      } else {
        st.nout_fwd = 1;
        fwd = st.w;
      }
      st.d_coef_fwd = upload(fwd, c->stream);
      std::vector<float> f32(fwd.begin(), fwd.end());
      st.d_coef_fwd32 = upload(f32, c->stream);
      if (!tr.empty()) {
        st.d_coef_tr = upload(tr, c->stream);
        std::vector<float> t32(tr.begin(), tr.end());
        st.d_coef_tr32 = upload(t32, c->stream);
      }
      if (fast && nd == 3 && (t == TGPU_STEN_THETA || t == TGPU_STEN_UATT)) {
        st.lines_fwd = build_lines(st, fwd, dg, c->stream);
        if (t == TGPU_STEN_THETA) st.lines_tr = build_lines(st, tr, dg, c->stream);
      }
      if (fast && nd == 3 && t == TGPU_STEN_DELTA && g.single_size) {
        // the forward table is [L][1 + nd] (one input), the transpose table [L][1 + nd] (one output)
        st.lines_fwd = build_lines(st, fwd, dg, c->stream, st.nout_fwd, 1);
        st.lines_tr = build_lines(st, tr, dg, c->stream, st.nin_tr, st.nin_tr);
        // one table per coefficient for the float-float sums
        for (int q = 0; q < st.nout_fwd; q++) {
          std::vector<double> col(st.L);
          for (int k = 0; k < st.L; k++) col[k] = fwd[(size_t)k * st.nout_fwd + q];
          st.ff_fwd.push_back(build_lines(st, col, dg, c->stream));
        }
        for (int q = 0; q < st.nin_tr; q++) {
          std::vector<double> col(st.L);
          for (int k = 0; k < st.L; k++) col[k] = tr[(size_t)k * st.nin_tr + q];
          st.ff_tr.push_back(build_lines(st, col, dg, c->stream));
        }
      }
      if (fast && nd == 3 && t == TGPU_STEN_UATT) tgpu::tc_build_tables(st.off, fwd, st.L, dg.h[1], st.tc, c->stream);
  };
  for (int t = 0; t < 3; t++)
    for (int idx = 0; idx < (int)c->sten[t].size(); idx++) prep(c->sten[t][idx], t, idx, true);
  for (int z = 1; z < c->nzone; z++)
    for (int t = 0; t < 3; t++)
      for (int idx = 0; idx < (int)c->zsten[z][t].size(); idx++) prep(c->zsten[z][t][idx], t, idx, false);
  const long N = dg.N;
  // fields
  if (c->h_vext.empty()) c->h_vext.assign((size_t)g.ncomp * N, 0.0);
  if (c->h_zero.empty()) c->h_zero.assign((size_t)g.ncomp * N, 0);
  c->d_vext = upload(c->h_vext, c->stream);
  c->d_zero = upload(c->h_zero, c->stream);
  if (g.hard_surf) {
    c->d_bnodes = upload(c->h_bnodes, c->stream);
    c->d_fmask = upload(c->h_fmask, c->stream);
    // target nodes: within the largest stencil reach of a boundary node (box dilation)
    std::vector<char> mark(N, 0);
    for (int l = 0; l < g.nlists_hw; l++)
      for (long i = 0; i < N; i++)
        if (c->h_bnodes[(size_t)l * N + i] != -1) mark[i] = 1;
    for (int d = 0; d < nd; d++) {
      std::vector<char> nm(N, 0);
      const long stride = d == 0 ? 1 : (d == 1 ? dg.nx[0] : (long)dg.nx[0] * dg.nx[1]);
      for (long i = 0; i < N; i++) {
        if (!mark[i]) continue;
        const int coord = (int)((i / stride) % dg.nx[d]);
        for (int s = -dg.h[d]; s <= dg.h[d]; s++) {
          int q = coord + s;
          if (q < 0 || q >= dg.nx[d]) {
            if (g.bc[d][0] == TGPU_BC_PERIODIC) q = (q % dg.nx[d] + dg.nx[d]) % dg.nx[d];
            else if (q < 0 && g.bc[d][0] == TGPU_BC_REFLECT) q = std::min(-q, dg.nx[d] - 1);
            else if (q >= dg.nx[d] && g.bc[d][1] == TGPU_BC_REFLECT) q = std::max(2 * (dg.nx[d] - 1) - q, 0);
            else continue;
          }
          nm[i + (long)(q - coord) * stride] = 1;
        }
      }
      mark.swap(nm);
    }
    for (long i = 0; i < N; i++)
      if (mark[i]) c->hw_targets.push_back((int)i);
    c->d_hw_targets = upload(c->hw_targets, c->stream);
  }
  // padding parameter sets
  {
    std::vector<double> b_res = bulk_values_rho(g), b_jac;
    std::vector<int> sg, zc;
    for (int jc = 0; jc < g.ncomp; jc++) {
      b_jac.push_back(0.0);
      sg.push_back(0);
      zc.push_back(jc);
    }
    c->pads.rho_res = make_pad(b_res, sg, zc, c->stream);
    c->pads.rho_jac = make_pad(b_jac, sg, zc, c->stream);
  }
  {
    std::vector<double> b_res = bulk_values_tr(g), b_jac;
    std::vector<int> sg, zc;
    for (int ic = 0; ic < g.ncomp; ic++) {
      b_jac.push_back(0.0);
      sg.push_back(0);
      zc.push_back(-1);
      for (int d = 0; d < nd; d++) {
        b_jac.push_back(0.0);
        sg.push_back(1 << d);
        zc.push_back(-1);
      }
      b_jac.push_back(0.0);
      sg.push_back(0);
      zc.push_back(-1);
    }
    c->pads.tr_res = make_pad(b_res, sg, zc, c->stream);
    c->pads.tr_jac = make_pad(b_jac, sg, zc, c->stream);
  }
  {
    const int nz = TGPU_MAXC * 6;   // adjoint channels: per component A, B[d], C and the mean-field row
    c->pads.zero_ext = make_pad(std::vector<double>(nz, 0.0), std::vector<int>(nz, 0), std::vector<int>(nz, -1), c->stream);
  }
  // work buffers
  c->nch_max = std::max(g.ncomp, g.ncomp * (nd + 2));
  const size_t U = (size_t)dg.nunk;
  c->d_x = dalloc<double>(U * N);
  c->d_work = dalloc<double>(U * N);
  c->d_work2 = dalloc<double>(U * N);
  c->d_pad = dalloc<double>((size_t)c->nch_max * NP);
  // FP32 padded channels with slack: the line kernel reads up to 2*kLineTX past a row end
  c->d_pad32 = dalloc<float>((size_t)c->nch_max * NP + 64);
  ck(cudaMemsetAsync(c->d_pad32, 0, sizeof(float) * ((size_t)c->nch_max * NP + 64), c->stream), "memset");
  c->d_chan = dalloc<double>((size_t)c->nch_max * N);
  c->d_conv = dalloc<double>((size_t)(dg.nrb + dg.ncomp) * N);
  c->d_tr = dalloc<double>((size_t)dg.ncomp * N);
  c->d_ymf = dalloc<double>((size_t)dg.ncomp * N);
  c->n2 = (long)dg.ncomp * N;
  c->d_newton_x = dalloc<double>(U * N);
  if (c->a22)
    for (auto &b : c->d_a22) b = dalloc<double>(U * N);
  c->d_b2s = dalloc<double>(c->n2);
  c->d_gw = dalloc<double>(c->n2);
  c->d_gt = dalloc<double>(c->n2);
  c->d_gx = dalloc<double>(c->n2);
  c->d_gb = dalloc<double>(c->n2);
  c->d_partial = dalloc<double>((size_t)tgpu::kPartialWords);
  ck(cudaMemsetAsync(c->d_partial + tgpu::kPartialWords - 1, 0, sizeof(double), c->stream), "memset");
  c->d_red = dalloc<double>(4096);
  ck(cudaMallocHost(&c->h_red, 4096 * sizeof(double)), "cudaMallocHost");
  tgpu::upload_geom(dg, c->stream);
  g_geom_owner = c;
  ck(cudaStreamSynchronize(c->stream), "sync");
}

}  // namespace

namespace tgpu {
void set_last_error(const std::string &text) { g_last_error = text; }
}  // namespace tgpu

extern "C" {

const char *tgpu_last_error(void) { return g_last_error.c_str(); }

int tgpu_create(const tgpu_geometry *geom, int device, tgpu_handle *out)
{
  return guard([&] {
    if (!geom || !out) throw Error(TGPU_ERR_ARG, "null argument");
    const tgpu_geometry &g = *geom;
    if (g.ndim < 1 || g.ndim > 3) throw Error(TGPU_ERR_ARG, "ndim must be 1, 2 or 3");
    if (g.ncomp < 1 || g.ncomp > TGPU_MAXC) throw Error(TGPU_ERR_ARG, "ncomp out of range");
    for (int d = 0; d < g.ndim; d++) {
      if (g.nx[d] < 1) throw Error(TGPU_ERR_ARG, "nx must be positive");
      for (int k = 0; k < 2; k++)
        if (g.bc[d][k] < TGPU_BC_IN_WALL || g.bc[d][k] > TGPU_BC_REFLECT)
          throw Error(TGPU_ERR_UNSUPPORTED, "boundary condition outside IN_WALL/IN_BULK/PERIODIC/REFLECT");
      if ((g.bc[d][0] == TGPU_BC_PERIODIC) != (g.bc[d][1] == TGPU_BC_PERIODIC))
        throw Error(TGPU_ERR_ARG, "periodic boundaries must be periodic on both sides");
    }
    if (g.interface != 0 && g.interface != 2) throw Error(TGPU_ERR_UNSUPPORTED, "interface type (0 or 2)");
    if (g.pin && g.interface != 2) throw Error(TGPU_ERR_ARG, "a pinned density needs a phase interface");
    if (g.functional < TGPU_FMT1 || g.functional > TGPU_FMT4)
      throw Error(TGPU_ERR_UNSUPPORTED, "functional outside FMT1..FMT4");
    const long N = nnodes(g);
    if (N > (1L << 31) / 4) throw Error(TGPU_ERR_ARG, "mesh too large for 32-bit stencil offsets");
    ck(cudaSetDevice(device), "cudaSetDevice");
    Ctx *c = new Ctx;
    c->g = g;
    c->device = device;
    tgpu::DevGeom &dg = c->dg;
    std::memset(&dg, 0, sizeof(dg));
    dg.ndim = g.ndim;
    dg.N = N;
    dg.ncomp = g.ncomp;
    dg.nrb = 4 + 2 * g.ndim;
    dg.first_rho = 0;
    dg.first_rb = g.ncomp;
    dg.first_mf = g.attraction ? g.ncomp + dg.nrb : -1;
    dg.nunk = g.ncomp + dg.nrb + (g.attraction ? g.ncomp : 0);
    c->a22 = g.attraction && g.att_in_a22;
    dg.interface = g.interface;
    for (int i = 0; i < TGPU_MAXC; i++) dg.betamu_if[i] = g.betamu[i];
    dg.pin_node = g.pin ? g.pin_node : -1;
    dg.pin_value = g.pin_value;
    if (g.pin && (g.pin_node < 0 || g.pin_node >= N)) throw Error(TGPU_ERR_ARG, "pinned node outside the mesh");
    c->nunk_ext = c->a22 ? dg.nunk - g.ncomp : dg.nunk;
    dg.functional = g.functional;
    dg.attraction = g.attraction;
    dg.single_size = g.single_size;
    dg.hard_surf = g.hard_surf;
    dg.nlists = g.nlists_hw;
    for (int i = 0; i < TGPU_MAXC; i++) {
      dg.rho_b[i] = g.rho_b[i];
      dg.betamu_hs_ex[i] = g.betamu_hs_ex[i];
      dg.betamu_att[i] = g.betamu_att[i];
      dg.inv_rad[i] = g.inv_rad[i];
      dg.inv_4pir[i] = g.inv_4pir[i];
      dg.inv_4pirsq[i] = g.inv_4pirsq[i];
      dg.fac[i] = g.fac_overlap[i];
    }
    for (int i = 0; i < 4; i++) dg.dphi_bulk[i] = g.dphi_bulk[i];
    dg.vext_max = g.vext_max;
    for (int t = 0; t < 3; t++) c->sten[t].resize((size_t)g.ncomp * g.ncomp);
    ck(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    c->own_stream = true;
    *out = c;
    return TGPU_OK;
  });
}

int tgpu_destroy(tgpu_handle h)
{
  return guard([&] {
    Ctx *c = C(h);
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (int t = 0; t < 3; t++)
      for (auto &st : c->sten[t]) {
        dfree(st.d_loff); dfree(st.d_loff_neg); dfree(st.d_off); dfree(st.d_w); dfree(st.d_hw);
        dfree(st.d_coef_fwd); dfree(st.d_coef_fwd32); dfree(st.d_coef_tr); dfree(st.d_coef_tr32); dfree(st.d_coef_adj);
        for (auto *L : {&st.lines_fwd, &st.lines_tr}) {
          dfree(L->d_planes); dfree(L->d_lines); dfree(L->d_w); dfree(L->d_w_lo);
        }
        for (auto *V : {&st.ff_fwd, &st.ff_tr})
          for (auto &L : *V) {
            dfree(L.d_planes); dfree(L.d_lines); dfree(L.d_w); dfree(L.d_w_lo);
          }
        tgpu::tc_free_tables(st.tc);
        for (auto *V : {&st.spec_fwd, &st.spec_tr})
          for (auto &k : *V) dfree(k);
        for (auto *V : {&st.spec_fwd32, &st.spec_tr32})
          for (auto &k : *V) dfree(k);
      }
    for (auto &b : c->d_fbox) dfree(b);
    dfree(c->d_dscr);
    for (auto &b : c->d_fbox32) dfree(b);
    for (auto &b : c->d_trbox) dfree(b);
    for (auto &b : c->d_trbox32) dfree(b);
    tgpu::fft_free_plan(c->fft);
    for (int z = 1; z < tgpu::kMaxZone; z++)
      for (int t = 0; t < 3; t++)
        for (auto &st : c->zsten[z][t]) {
          dfree(st.d_loff); dfree(st.d_loff_neg); dfree(st.d_off); dfree(st.d_w); dfree(st.d_hw);
          dfree(st.d_coef_fwd); dfree(st.d_coef_fwd32); dfree(st.d_coef_tr); dfree(st.d_coef_tr32); dfree(st.d_coef_adj);
        }
    dfree(c->d_zone); dfree(c->d_zbuf); dfree(c->d_cbulk); dfree(c->d_cscr); dfree(c->d_cscr2); dfree(c->d_hcoef); dfree(c->d_domain);
    dfree(c->cr.d_node); dfree(c->cr.d_rptr); dfree(c->cr.d_rcol); dfree(c->cr.d_ra);
    dfree(c->cr.d_pptr); dfree(c->cr.d_pcol); dfree(c->cr.d_pw); dfree(c->cr.d_kind); dfree(c->d_rowkind);
    dfree(c->d_conv32); dfree(c->d_chan32); dfree(c->d_tr32); dfree(c->d_ymf32); dfree(c->d_hcoef32);
    dfree(c->d_inv32); dfree(c->d_kind32);
    for (int d = 0; d < 3; d++) dfree(c->d_map[d]);
    tgpu::tc_free_slab(c->tcslab);
    dfree(c->d_vext); dfree(c->d_zero); dfree(c->d_bnodes); dfree(c->d_fmask); dfree(c->d_hw_targets);
    dfree(c->d_x); dfree(c->d_work); dfree(c->d_work2); dfree(c->d_pad); dfree(c->d_pad32); dfree(c->d_chan);
    dfree(c->d_conv); dfree(c->d_tr); dfree(c->d_ymf); dfree(c->d_b2s); dfree(c->d_V); dfree(c->d_partial);
    dfree(c->d_red); dfree(c->d_gw); dfree(c->d_gt); dfree(c->d_gx); dfree(c->d_gb);
    dfree(c->d_rho_ref); dfree(c->d_conv_ref); dfree(c->d_chan_ref); dfree(c->d_tr_ref);
    dfree(c->d_drho); dfree(c->d_dchan); dfree(c->d_newton_x);
    for (auto &b : c->d_a22) dfree(b);
    if (c->h_red) cudaFreeHost(c->h_red);
    free_pad(c->pads.rho_res); free_pad(c->pads.rho_jac); free_pad(c->pads.tr_res); free_pad(c->pads.tr_jac);
    free_pad(c->pads.zero_ext);
    dfree(c->d_adj_chan); dfree(c->d_adj_pad); dfree(c->d_adj_g); dfree(c->d_adj_v); dfree(c->d_adj_t);
    dfree(c->d_wf); dfree(c->d_wb); dfree(c->d_obj_gx); dfree(c->d_obj_gv); dfree(c->d_obj_lam); dfree(c->d_obj_R);
    if (c->own_stream) cudaStreamDestroy(c->stream);
    if (g_geom_owner == c) g_geom_owner = nullptr;
    delete c;
    return TGPU_OK;
  });
}

int tgpu_set_stencil(tgpu_handle h, int type, int index, int length, const short *offsets, const double *weights,
                     const double *hw)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) throw Error(TGPU_ERR_STATE, "stencils are fixed after tgpu_finalize");
    if (type < 0 || type > 2) throw Error(TGPU_ERR_ARG, "stencil type");
    const int nidx = type == TGPU_STEN_UATT ? c->g.ncomp * c->g.ncomp : c->g.ncomp;
    if (index < 0 || index >= nidx) throw Error(TGPU_ERR_ARG, "stencil index");
    if (length < 0 || (length > 0 && (!offsets || !weights))) throw Error(TGPU_ERR_ARG, "stencil arrays");
    DevStencil &st = c->sten[type][index];
    const int nd = c->g.ndim;
    st.L = length;
    st.off.assign(offsets, offsets + (size_t)length * nd);
    st.w.assign(weights, weights + length);
    if (hw) st.hw.assign(hw, hw + (size_t)length * (1 << nd));
    else st.hw.clear();
    return TGPU_OK;
  });
}

int tgpu_set_zones(tgpu_handle h, int nzone, const int *flag, const double *rb_bulk)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) throw Error(TGPU_ERR_STATE, "zones are fixed after tgpu_finalize");
    if (nzone < 1 || nzone > tgpu::kMaxZone) throw Error(TGPU_ERR_ARG, "number of zones");
    if (!flag || !rb_bulk) throw Error(TGPU_ERR_ARG, "null zone arrays");
    const long N = c->dg.N;
    for (long i = 0; i < N; i++) {
      const int f = flag[i];
      if (!((f >= -c->g.ndim && f < nzone) || f == kFlag1dbc || f == kFlagBulk || f == kFlagPB))
        throw Error(TGPU_ERR_ARG, "zone flag");
    }
    c->nzone = nzone;
    c->h_zone.assign(flag, flag + N);
    const int nrb = 4 + 2 * c->g.ndim;
    c->h_rb_bulk.assign(rb_bulk, rb_bulk + (c->g.interface == 2 ? 2 : 1) * nrb);
    for (int z = 1; z < nzone; z++)
      for (int t = 0; t < 3; t++) c->zsten[z][t].resize(c->sten[t].size());
    return TGPU_OK;
  });
}

int tgpu_set_1d_boundary(tgpu_handle h, int dim)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) throw Error(TGPU_ERR_STATE, "zones are fixed after tgpu_finalize");
    if (dim < 0 || dim >= c->g.ndim) throw Error(TGPU_ERR_ARG, "dimension");
    c->dim_1dbc = dim;
    return TGPU_OK;
  });
}

int tgpu_set_zone_stencil(tgpu_handle h, int zone, int type, int index, int length, const short *offsets,
                          const double *weights, const double *hw)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) throw Error(TGPU_ERR_STATE, "stencils are fixed after tgpu_finalize");
    if (zone < 1 || zone >= c->nzone) throw Error(TGPU_ERR_ARG, "zone (set the zones first)");
    if (type < 0 || type > 2) throw Error(TGPU_ERR_ARG, "stencil type");
    const int nidx = type == TGPU_STEN_UATT ? c->g.ncomp * c->g.ncomp : c->g.ncomp;
    if (index < 0 || index >= nidx) throw Error(TGPU_ERR_ARG, "stencil index");
    if (length <= 0 || !offsets || !weights) throw Error(TGPU_ERR_ARG, "stencil arrays");
    DevStencil &st = c->zsten[zone][type][index];
    const int nd = c->g.ndim;
    st.L = length;
    st.off.assign(offsets, offsets + (size_t)length * nd);
    st.w.assign(weights, weights + length);
    if (hw) st.hw.assign(hw, hw + (size_t)length * (1 << nd));
    else st.hw.clear();
    return TGPU_OK;
  });
}

int tgpu_set_vext(tgpu_handle h, const double *vext)
{
  return guard([&] {
    Ctx *c = C(h);
    if (!vext) throw Error(TGPU_ERR_ARG, "null vext");
    const size_t n = (size_t)c->g.ncomp * c->dg.N;
    for (size_t i = 0; i < n; i++)
      if (std::isnan(vext[i])) throw Error(TGPU_ERR_NONFINITE, "NaN in the external field");
    c->h_vext.assign(vext, vext + n);
    c->hcoef32_form = -1;   // the FP32 products' row kinds follow V_ext (vext_max rows)
    if (c->finalized) ck(cudaMemcpyAsync(c->d_vext, vext, n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "h2d");
    ck(cudaStreamSynchronize(c->stream), "sync");
    return TGPU_OK;
  });
}

int tgpu_set_bulk_state(tgpu_handle h, const double *rho_b, const double *betamu_hs_ex, const double *betamu_att,
                        const double *dphi_bulk)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if (!rho_b || !betamu_hs_ex || !betamu_att || !dphi_bulk) throw Error(TGPU_ERR_ARG, "null argument");
    tgpu_geometry &g = c->g;
    tgpu::DevGeom &dg = c->dg;
    for (int ic = 0; ic < g.ncomp; ic++) {
      if (!(rho_b[ic] > 0.0)) throw Error(TGPU_ERR_ARG, "bulk densities must be positive");
      g.rho_b[ic] = dg.rho_b[ic] = rho_b[ic];
      g.betamu_hs_ex[ic] = dg.betamu_hs_ex[ic] = betamu_hs_ex[ic];
      g.betamu_att[ic] = dg.betamu_att[ic] = betamu_att[ic];
    }
    for (int k = 0; k < 4; k++) g.dphi_bulk[k] = dg.dphi_bulk[k] = dphi_bulk[k];
    if (c->coarse() && g.interface != 2) {
      // Rhobar_b of the new bulk state for the averaged rows next to IN_BULK boundaries (rhobar_icomp,
      // src/dft_thermo_hs.c:292-311; the diameter from 1/R)
      std::fill(c->h_rb_bulk.begin(), c->h_rb_bulk.end(), 0.0);
      for (int ic = 0; ic < g.ncomp; ic++) {
        const double d = 2.0 / g.inv_rad[ic], vol = M_PI * d * d * d / 6.0, area = M_PI * d * d;
        const double f = g.fac_overlap[ic] * g.rho_b[ic];
        c->h_rb_bulk[0] += f * vol;
        c->h_rb_bulk[1] += f * area;
        c->h_rb_bulk[2] += f * area * g.inv_4pir[ic];
        c->h_rb_bulk[3] += f * area * g.inv_4pirsq[ic];
      }
      upload_cbulk(c);
    }
    const std::vector<double> br = bulk_values_rho(g), bt = bulk_values_tr(g);
    ck(cudaMemcpyAsync(c->pads.rho_res.bulk, br.data(), br.size() * sizeof(double), cudaMemcpyHostToDevice,
                       c->stream), "h2d");
    ck(cudaMemcpyAsync(c->pads.tr_res.bulk, bt.data(), bt.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream),
       "h2d");
    c->pads.rho_res.h_bulk = br;   // the host copies the FFT sums read the boundary values from
    c->pads.tr_res.h_bulk = bt;
    tgpu::upload_geom(dg, c->stream);
    g_geom_owner = c;
    c->have_state = false;
    c->have_ref = false;
    ck(cudaStreamSynchronize(c->stream), "sync");
    return TGPU_OK;
  });
}

int tgpu_set_zero_density(tgpu_handle h, const signed char *flags)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) throw Error(TGPU_ERR_STATE, "zero-density flags are fixed after tgpu_finalize");
    if (!flags) throw Error(TGPU_ERR_ARG, "null flags");
    c->h_zero.assign(flags, flags + (size_t)c->g.ncomp * c->dg.N);
    return TGPU_OK;
  });
}

int tgpu_set_hard_wall(tgpu_handle h, const int *bnodes, const short *fmask)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) throw Error(TGPU_ERR_STATE, "hard-wall data is fixed after tgpu_finalize");
    if (!c->g.hard_surf) throw Error(TGPU_ERR_ARG, "geometry has no hard surfaces");
    if (!bnodes || !fmask) throw Error(TGPU_ERR_ARG, "null hard-wall arrays");
    const size_t N = c->dg.N;
    const size_t L = c->g.nlists_hw;
    c->h_bnodes.assign(bnodes, bnodes + L * N);
    c->h_fmask.assign(fmask, fmask + L * ((size_t)1 << c->g.ndim) * N);
    return TGPU_OK;
  });
}

int tgpu_finalize(tgpu_handle h)
{
  return guard([&] {
    Ctx *c = C(h);
    if (c->finalized) return TGPU_OK;
    const tgpu_geometry &g = c->g;
    for (int ic = 0; ic < g.ncomp; ic++) {
      if (c->sten[TGPU_STEN_DELTA][ic].L == 0 || c->sten[TGPU_STEN_THETA][ic].L == 0)
        throw Error(TGPU_ERR_STATE, "missing delta or theta stencil");
      if (g.hard_surf && (c->sten[TGPU_STEN_DELTA][ic].hw.empty() || c->sten[TGPU_STEN_THETA][ic].hw.empty()))
        throw Error(TGPU_ERR_STATE, "hard surfaces need the stencils' corner weights");
    }
    if (g.attraction)
      for (int k = 0; k < g.ncomp * g.ncomp; k++)
        if (c->sten[TGPU_STEN_UATT][k].L == 0) throw Error(TGPU_ERR_STATE, "missing attraction stencil");
        else if (g.hard_surf && c->sten[TGPU_STEN_UATT][k].hw.empty())
          throw Error(TGPU_ERR_STATE, "hard surfaces need the attraction stencils' corner weights");
    if (g.hard_surf && c->h_bnodes.empty()) throw Error(TGPU_ERR_STATE, "hard surfaces need tgpu_set_hard_wall");
    if (c->nzone > 1) {
      for (int z = 1; z < c->nzone; z++)
        for (int t = 0; t < 3; t++) {
          if (t == TGPU_STEN_UATT && !g.attraction) continue;
          const int nidx = t == TGPU_STEN_UATT ? g.ncomp * g.ncomp : g.ncomp;
          for (int k = 0; k < nidx; k++)
            if (c->zsten[z][t][k].L == 0) throw Error(TGPU_ERR_STATE, "missing stencil of a coarser zone");
        }
    }
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    build_device_tables(c);
    if (!c->h_zone.empty()) {
      for (int t : c->hw_targets)
        if (c->h_zone[t] > 0)
          throw Error(TGPU_ERR_UNSUPPORTED, "hard-wall boundary nodes within reach of a coarser zone's stencils");
      // stencil zone per node: BULK_ZONE / PB_ZONE nodes fill their other rows with zone 0's stencils (the
      // reference indexes its stencil table with the negative flag there); their Euler-Lagrange rows by kind
      std::vector<int> zone(c->h_zone);
      std::vector<signed char> kind(zone.size(), 0);
      bool any_kind = false;
      for (size_t i = 0; i < zone.size(); i++)
        if (zone[i] == kFlagBulk || zone[i] == kFlagPB) {
          kind[i] = zone[i] == kFlagBulk ? 1 : 2;
          zone[i] = 0;
          any_kind = true;
        }
      c->d_zone = upload(zone, c->stream);
      if (any_kind) {
        c->d_rowkind = upload(kind, c->stream);
        c->dg.rowkind = c->d_rowkind;
        tgpu::upload_geom(c->dg, c->stream);
      }
      if (c->nzone > 1) c->d_zbuf = dalloc<double>((size_t)(c->dg.nrb + c->dg.ncomp) * c->dg.N);
      build_coarse(c);
      ck(cudaStreamSynchronize(c->stream), "sync");
    }
    bool any_tc = false;
    for (auto &st : c->sten[TGPU_STEN_UATT]) any_tc = any_tc || st.tc.nplanes > 0;
    if (any_tc) c->tc_ready = tgpu::tc_make_slab(c->tcslab, c->dg, c->tc_why);
    else c->tc_why = "no 3-D attraction stencil";
    c->finalized = true;
    return TGPU_OK;
  });
}

int tgpu_set_precision(tgpu_handle h, int precision)
{
  return guard([&] {
    Ctx *c = C(h);
    if (precision != TGPU_FP64 && precision != TGPU_FP32 && precision != TGPU_FP16TC && precision != TGPU_FP64_FFT)
      throw Error(TGPU_ERR_UNSUPPORTED, "precision");
    if (precision == TGPU_FP16TC && !c->tc_ready)
      throw Error(TGPU_ERR_UNSUPPORTED, "tensor-core sums unavailable: " + c->tc_why);
    c->precision = precision;
    return TGPU_OK;
  });
}

int tgpu_set_jacobian_form(tgpu_handle h, int form)
{
  return guard([&] {
    Ctx *c = C(h);
    if (form != TGPU_JAC_REFERENCE && form != TGPU_JAC_EXACT) throw Error(TGPU_ERR_ARG, "jacobian form");
    c->dg.jac_exact = form == TGPU_JAC_EXACT ? 1 : 0;
    tgpu::upload_geom(c->dg, c->stream);
    ck(cudaStreamSynchronize(c->stream), "sync");
    return TGPU_OK;
  });
}

int tgpu_set_fft32_policy(tgpu_handle h, int policy)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if (policy < -1 || policy > 1) throw Error(TGPU_ERR_ARG, "policy");
    int v = 0;
    if (policy != -1) {
      v = policy == 1 ? 1 : -1;
      if (v == 1 && !prepare_spec32(c)) throw Error(TGPU_ERR_UNSUPPORTED, "FP32 FFT sums unavailable for this problem");
    }
    c->fft32_tc = c->fft32_slab = v;
    for (int t = 0; t < 3; t++)
      for (auto &st : c->sten[t]) st.fft32_fwd = st.fft32_tr = v;
    return TGPU_OK;
  });
}

int tgpu_set_fft_threshold(tgpu_handle h, int min_points)
{
  return guard([&] {
    Ctx *c = C(h);
    c->fft_min_points = min_points < 0 ? -1 : min_points;
    if (c->fft_state != 0) {   // spectra are rebuilt for the new choice at the next FFT fill
      ck(cudaStreamSynchronize(c->stream), "sync");
      for (int t = 0; t < 3; t++)
        for (auto &st : c->sten[t]) {
          for (auto *V : {&st.spec_fwd, &st.spec_tr}) {
            for (auto &k : *V) dfree(k);
            V->clear();
          }
        }
      for (auto &b : c->d_fbox) dfree(b);
      for (int t = 0; t < 3; t++)
        for (auto &st : c->sten[t]) {
          for (auto *V : {&st.spec_fwd32, &st.spec_tr32}) {
            for (auto &k : *V) dfree(k);
            V->clear();
          }
          st.fft32_fwd = st.fft32_tr = 0;
        }
      for (auto &b : c->d_fbox32) dfree(b);
      for (auto &b : c->d_trbox) dfree(b);
      for (auto &b : c->d_trbox32) dfree(b);
      c->d_trbox.clear();
      c->d_trbox32.clear();
      tgpu::fft_free_plan(c->fft);
      c->fft_state = 0;
      c->fft_gen = -1;
      c->fft_plan_ok = false;
      c->spec32_built = false;
      c->fft32_tc = c->fft32_slab = 0;
      c->fft32_gen = -1;
    }
    return TGPU_OK;
  });
}

int tgpu_fft32_choice(tgpu_handle h, int type, int index, int *choice, double *ms)
{
  return guard([&] {
    Ctx *c = C(h);
    if (type < 0 || type > 2 || index < 0 || index >= (int)c->sten[type].size() || !choice || !ms)
      throw Error(TGPU_ERR_ARG, "no such stencil");
    const DevStencil &st = c->sten[type][index];
    if (type == TGPU_STEN_UATT) {
      const int ctx = c->precision == TGPU_FP16TC ? 1 : 0;
      choice[0] = ctx ? c->fft32_tc : c->fft32_slab;
      choice[1] = 0;
      ms[0] = c->t32_att[ctx][0];
      ms[1] = c->t32_att[ctx][1];
      ms[2] = ms[3] = 0.0;
    } else {
      choice[0] = st.fft32_fwd;
      choice[1] = st.fft32_tr;
      for (int k = 0; k < 4; k++) ms[k] = st.t32[k / 2][k % 2];
    }
    return TGPU_OK;
  });
}

int tgpu_set_fill_arithmetic(tgpu_handle h, int arith, double tau, double switch_norm)
{
  return guard([&] {
    Ctx *c = C(h);
    if (arith != TGPU_FILL_FP64 && arith != TGPU_FILL_FP32 && arith != TGPU_FILL_REFINED && arith != TGPU_FILL_MIXED &&
        arith != TGPU_FILL_FF && arith != TGPU_FILL_MIXED_FF && arith != TGPU_FILL_FFT && arith != TGPU_FILL_MIXED_FFT)
      throw Error(TGPU_ERR_ARG, "fill arithmetic");
    if (tau > 0) c->refine_tau = tau;
    if (switch_norm > 0) c->refine_switch = switch_norm;
    c->fill_mode = arith;
    c->have_ref = false;
    return TGPU_OK;
  });
}

int tgpu_set_stream(tgpu_handle h, void *stream)
{
  return guard([&] {
    Ctx *c = C(h);
    ck(cudaStreamSynchronize(c->stream), "sync");
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->own_stream = false;
    c->stream = static_cast<cudaStream_t>(stream);
    return TGPU_OK;
  });
}

int tgpu_sizes(tgpu_handle h, long *nn, int *nunk, int *ncomp)
{
  return guard([&] {
    Ctx *c = C(h);
    if (nn) *nn = c->dg.N;
    if (nunk) *nunk = c->nunk_ext;
    if (ncomp) *ncomp = c->dg.ncomp;
    return TGPU_OK;
  });
}

int tgpu_fill_device(tgpu_handle h, const double *d_x, double *d_R, int mode)
{
  return guard([&] {
    if (mode != 0 && mode != 1) throw Error(TGPU_ERR_ARG, "mode must be 0 or 1");
    Ctx *c = C(h);
    need_final(c);
    double *R = a22_out_buf(c, d_R, 1);
    fill_device(c, a22_in(c, d_x, A22_SUMS, 0), R, mode);
    a22_out(c, R, d_R);
    ck(cudaGetLastError(), "fill launch");
    check_domain(c);
    return TGPU_OK;
  });
}

int tgpu_fill(tgpu_handle h, const double *x, double *R, int mode)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if (mode != 0 && mode != 1) throw Error(TGPU_ERR_ARG, "mode must be 0 or 1");
    const size_t n = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_work, x, n);
    double *Rd = a22_out_buf(c, c->d_work2, 1);
    fill_device(c, a22_in(c, c->d_work, A22_SUMS, 0), Rd, mode);
    a22_out(c, Rd, c->d_work2);
    d2h(c, R, c->d_work2, n);
    ck(cudaGetLastError(), "fill launch");
    check_domain(c);
    return TGPU_OK;
  });
}

int tgpu_jv_device(tgpu_handle h, const double *d_v, double *d_out)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    double *o = a22_out_buf(c, d_out, 1);
    jv_device(c, a22_in(c, d_v, A22_JAC_SUMS, 0), o);
    a22_out(c, o, d_out);
    ck(cudaGetLastError(), "jv");
    return TGPU_OK;
  });
}

int tgpu_jv(tgpu_handle h, const double *v, double *out)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    const size_t n = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_work, v, n);
    double *o = a22_out_buf(c, c->d_work2, 1);
    jv_device(c, a22_in(c, c->d_work, A22_JAC_SUMS, 0), o);
    a22_out(c, o, c->d_work2);
    d2h(c, out, c->d_work2, n);
    return TGPU_OK;
  });
}

int tgpu_schur_apply_device(tgpu_handle h, const double *d_v2, double *d_y2)
{
  return guard([&] { schur_device(C(h), d_v2, d_y2); ck(cudaGetLastError(), "schur"); return TGPU_OK; });
}

int tgpu_schur_apply(tgpu_handle h, const double *v2, double *y2)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    h2d(c, c->d_work, v2, c->n2);
    schur_device(c, c->d_work, c->d_work2);
    d2h(c, y2, c->d_work2, c->n2);
    return TGPU_OK;
  });
}

int tgpu_schur_rhs_device(tgpu_handle h, const double *d_b, double *d_b2s)
{
  return guard([&] {
    Ctx *c = C(h);
    schur_rhs_device(c, a22_in(c, d_b, A22_ZERO, 0), d_b2s);
    return TGPU_OK;
  });
}

int tgpu_schur_x1_device(tgpu_handle h, const double *d_b, const double *d_x2, double *d_x)
{
  return guard([&] {
    Ctx *c = C(h);
    double *o = a22_out_buf(c, d_x, 1);
    schur_x1_device(c, a22_in(c, d_b, A22_ZERO, 0), d_x2, o);
    a22_out(c, o, d_x);
    return TGPU_OK;
  });
}

int tgpu_solve_device(tgpu_handle h, const double *d_b, double *d_dx, double tol, int maxit, int *iters,
                      double *relres)
{
  return guard([&] {
    int it = 0;
    double rr = 0.0;
    Ctx *c = C(h);
    double *o = a22_out_buf(c, d_dx, 1);
    const int st = solve_device(c, a22_in(c, d_b, A22_ZERO, 0), o, tol, maxit, &it, &rr);
    a22_out(c, o, d_dx);
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st;
  });
}

int tgpu_solve(tgpu_handle h, const double *b, double *dx, double tol, int maxit, int *iters, double *relres)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    const size_t n = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_work, b, n);
    int it = 0;
    double rr = 0.0;
    double *o = a22_out_buf(c, c->d_work2, 1);
    const int st = solve_device(c, a22_in(c, c->d_work, A22_ZERO, 0), o, tol, maxit, &it, &rr);
    a22_out(c, o, c->d_work2);
    d2h(c, dx, c->d_work2, n);
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st;
  });
}

int tgpu_newton_device(tgpu_handle h, double *d_x, double rel_tol, double abs_tol, double update_floor, int max_iter,
                       double lin_tol, int lin_max_iter, int *iters, double *final_resid)
{
  return guard([&] {
    int it = 0;
    Ctx *c = C(h);
    need_final(c);
    double *x = c->a22 ? const_cast<double *>(a22_in(c, d_x, A22_SUMS, 2)) : d_x;
    const int st = newton_device(c, x, rel_tol, abs_tol, update_floor, max_iter, lin_tol, lin_max_iter, &it,
                                 final_resid);
    a22_out(c, x, d_x);
    if (iters) *iters = it;
    return st;
  });
}

int tgpu_newton(tgpu_handle h, double *x, double rel_tol, double abs_tol, double update_floor, int max_iter,
                double lin_tol, int lin_max_iter, int *iters, double *final_resid)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    const size_t n = (size_t)c->dg.nunk * c->dg.N, ne = (size_t)c->nunk_ext * c->dg.N;
    double *d_xs = dalloc<double>(n);
    int st = TGPU_OK;
    try {
      h2d(c, d_xs, x, ne);
      if (c->a22) copy_d(c, d_xs, a22_in(c, d_xs, A22_SUMS, 2), n);
      int it = 0;
      st = newton_device(c, d_xs, rel_tol, abs_tol, update_floor, max_iter, lin_tol, lin_max_iter, &it, final_resid);
      if (iters) *iters = it;
      d2h(c, x, d_xs, ne);
    } catch (...) {
      dfree(d_xs);
      throw;
    }
    dfree(d_xs);
    return st;
  });
}

int tgpu_newton_solve_device(tgpu_handle h, double *d_x, double resid_tol, int max_iter, double lin_tol,
                             int lin_max_iter, double update_floor, int *iters, double *final_resid,
                             int *lin_iters_total)
{
  return guard([&] {
    int it = 0, lt = 0;
    double fr = 0.0;
    Ctx *c = C(h);
    need_final(c);
    double *x = c->a22 ? const_cast<double *>(a22_in(c, d_x, A22_SUMS, 2)) : d_x;
    const int st = newton_solve_device(c, x, resid_tol, max_iter, lin_tol, lin_max_iter, update_floor, &it, &fr, &lt);
    a22_out(c, x, d_x);
    if (iters) *iters = it;
    if (final_resid) *final_resid = fr;
    if (lin_iters_total) *lin_iters_total = lt;
    return st;
  });
}

int tgpu_newton_solve(tgpu_handle h, double *x, double resid_tol, int max_iter, double lin_tol, int lin_max_iter,
                      double update_floor, int *iters, double *final_resid, int *lin_iters_total)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    const size_t n = (size_t)c->dg.nunk * c->dg.N, ne = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_newton_x, x, ne);
    if (c->a22) copy_d(c, c->d_newton_x, a22_in(c, c->d_newton_x, A22_SUMS, 2), n);
    int it = 0, lt = 0;
    double fr = 0.0;
    const int st = newton_solve_device(c, c->d_newton_x, resid_tol, max_iter, lin_tol, lin_max_iter, update_floor,
                                       &it, &fr, &lt);
    d2h(c, x, c->d_newton_x, ne);
    if (iters) *iters = it;
    if (final_resid) *final_resid = fr;
    if (lin_iters_total) *lin_iters_total = lt;
    return st;
  });
}

int tgpu_time_stencil_sum(tgpu_handle h, int type, int index, int precision, int reps, double *ms_per_sum)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if (type < 0 || type > 2 || index < 0 || index >= (int)c->sten[type].size() || c->sten[type][index].L == 0)
      throw Error(TGPU_ERR_ARG, "no such stencil");
    if (reps < 1) throw Error(TGPU_ERR_ARG, "reps");
    if (precision != TGPU_FP64 && precision != TGPU_FP32 && precision != TGPU_FP16TC && precision != TGPU_FILL_FF &&
        precision != TGPU_FILL_FFT && precision != TGPU_TIME_FFT32)
      throw Error(TGPU_ERR_ARG, "precision");
    if (precision == TGPU_TIME_FFT32 && (type != TGPU_STEN_UATT || !prepare_spec32(c) ||
                                         c->sten[type][index].spec_fwd32.empty()))
      throw Error(TGPU_ERR_UNSUPPORTED, "FP32 FFT sums exist for 3-D attraction stencils only");
    if (precision == TGPU_FILL_FFT) {
      ensure_fft(c);
      if (c->fft_state != 1) throw Error(TGPU_ERR_UNSUPPORTED, "FFT sums unavailable for this problem");
    }
    const bool f32 = precision == TGPU_FP32 || precision == TGPU_FP16TC || precision == TGPU_TIME_FFT32;
    if (precision == TGPU_FP16TC && !c->tc_ready)
      throw Error(TGPU_ERR_UNSUPPORTED, "tensor-core sums unavailable: " + c->tc_why);
    const bool tc_prev = c->tc_on, ff_prev = c->ff_on, fft_prev = c->fft_on;
    const int fft32_prev[2] = {c->fft32_tc, c->fft32_slab};
    // the direct kernels of each arithmetic (tensor core, FP32 slab), or the FP32 FFT
    c->fft32_tc = c->fft32_slab = precision == TGPU_TIME_FFT32 ? 1 : -1;
    c->tc_on = precision == TGPU_FP16TC;
    c->ff_on = precision == TGPU_FILL_FF || precision == TGPU_FILL_FFT;
    c->fft_on = precision == TGPU_FILL_FFT;
    const DevStencil &st = c->sten[type][index];
    const int jc = type == TGPU_STEN_UATT ? index / c->dg.ncomp : index;
    const long N = c->dg.N;
    // density of the handle's state (or zeros before any fill) as the field
    pad(c, c->d_x + (long)c->dg.first_rho * N, c->pads.rho_res, f32);
    double *out[1] = {c->d_tr};
    ck(cudaEventCreate(&c->ev0), "event");
    ck(cudaEventCreate(&c->ev1), "event");
    conv(c, jc, 1, st, false, out, 1, f32);   // warm-up
    ck(cudaEventRecord(c->ev0, c->stream), "event");
    for (int r = 0; r < reps; r++) {
      c->fft_gen = c->fft32_gen = -1;   // each FFT sum transforms its field afresh
      conv(c, jc, 1, st, false, out, 1, f32);
    }
    ck(cudaEventRecord(c->ev1, c->stream), "event");
    ck(cudaEventSynchronize(c->ev1), "event");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "event");
    cudaEventDestroy(c->ev0);
    cudaEventDestroy(c->ev1);
    c->ev0 = c->ev1 = nullptr;
    c->tc_on = tc_prev;
    c->ff_on = ff_prev;
    c->fft_on = fft_prev;
    c->fft32_tc = fft32_prev[0];
    c->fft32_slab = fft32_prev[1];
    tc_check(c);
    *ms_per_sum = ms / reps;
    return TGPU_OK;
  });
}

int tgpu_set_tc_wait_limit(tgpu_handle h, long spins)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if (!c->tc_ready) throw Error(TGPU_ERR_UNSUPPORTED, "tensor-core sums unavailable: " + c->tc_why);
    c->tcslab.spin = spins > 0 ? spins : 0;
    return TGPU_OK;
  });
}

int tgpu_time_fft_pass(tgpu_handle h, int precision, int axis, int reps, double *ms_per_pass, long *box_points,
                       long *real_points)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if ((precision != TGPU_FP32 && precision != TGPU_FP64) || axis < 1 || axis > 2 || reps < 1 || !ms_per_pass)
      throw Error(TGPU_ERR_ARG, "precision, axis or reps");
    if (precision == TGPU_FP32 ? !prepare_spec32(c) : (ensure_fft(c), c->fft_state != 1))
      throw Error(TGPU_ERR_UNSUPPORTED, "FFT sums unavailable for this problem");
    if (c->fft.F[axis] == 1) throw Error(TGPU_ERR_UNSUPPORTED, "no transform along that axis");
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    auto run = [&] {
      if (precision == TGPU_FP32) tgpu::fft_pass(c->d_fbox32[1], c->fft, axis, false, c->stream);
      else tgpu::fft_pass(c->d_fbox[1], c->fft, axis, false, c->stream);
    };
    run();   // warm-up (the work spectrum's contents do not matter)
    ck(cudaEventRecord(e0, c->stream), "event");
    for (int r = 0; r < reps; r++) run();
    ck(cudaEventRecord(e1, c->stream), "event");
    ck(cudaEventSynchronize(e1), "event");
    float ms = 0.f;
    ck(cudaEventElapsedTime(&ms, e0, e1), "event");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms_per_pass = ms / reps;
    if (box_points) *box_points = c->fft.NH;
    if (real_points) *real_points = c->fft.NR;
    return TGPU_OK;
  });
}

int tgpu_pass_timer_begin(tgpu_handle h)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    long nl = 0;
    tgpu::pass_timer_collect(&nl, nullptr, nullptr, nullptr);   // drop an earlier unread window
    tgpu::pass_timer_enable(true);
    return TGPU_OK;
  });
}

int tgpu_pass_timer_end(tgpu_handle h, long *launches, double *ms_total, double *bytes_total, long *transforms)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    tgpu::pass_timer_enable(false);
    ck(cudaStreamSynchronize(c->stream), "sync");
    tgpu::pass_timer_collect(launches, ms_total, bytes_total, transforms);
    return TGPU_OK;
  });
}

int tgpu_get_stats(tgpu_handle h, tgpu_stats *out)
{
  return guard([&] { *out = C(h)->stats; return TGPU_OK; });
}

int tgpu_reset_stats(tgpu_handle h)
{
  return guard([&] { std::memset(&C(h)->stats, 0, sizeof(tgpu_stats)); return TGPU_OK; });
}

int tgpu_jtv_device(tgpu_handle h, const double *d_w, double *d_out)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    double *o = a22_out_buf(c, d_out, 1);
    jtv_device(c, a22_in(c, d_w, A22_EL, 0), o);
    a22_out(c, o, d_out);
    ck(cudaGetLastError(), "jtv");
    return TGPU_OK;
  });
}

int tgpu_jtv(tgpu_handle h, const double *w, double *out)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    const size_t n = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_work, w, n);
    double *o = a22_out_buf(c, c->d_work2, 1);
    jtv_device(c, a22_in(c, c->d_work, A22_EL, 0), o);
    a22_out(c, o, c->d_work2);
    d2h(c, out, c->d_work2, n);
    return TGPU_OK;
  });
}

int tgpu_adjoint_solve_device(tgpu_handle h, const double *d_g, double *d_lambda, double tol, int max_iter,
                              int *iters, double *relres)
{
  return guard([&] {
    int it = 0;
    double rr = 0.0;
    Ctx *c = C(h);
    double *o = a22_out_buf(c, d_lambda, 1);
    const int st = adjoint_solve_device(c, a22_in(c, d_g, A22_ZERO, 0), o, tol, max_iter, &it, &rr);
    a22_out(c, o, d_lambda);
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st;
  });
}

int tgpu_adjoint_solve(tgpu_handle h, const double *g, double *lambda, double tol, int max_iter, int *iters,
                       double *relres)
{
  return guard([&] {
    Ctx *c = C(h);
    need_state(c);
    const size_t n = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_work, g, n);
    int it = 0;
    double rr = 0.0;
    double *o = a22_out_buf(c, c->d_work2, 1);
    const int st = adjoint_solve_device(c, a22_in(c, c->d_work, A22_ZERO, 0), o, tol, max_iter, &it, &rr);
    a22_out(c, o, c->d_work2);
    d2h(c, lambda, c->d_work2, n);
    if (iters) *iters = it;
    if (relres) *relres = rr;
    return st;
  });
}

int tgpu_set_integration(tgpu_handle h, const double *w_fluid, const double *w_bulk, const double *rhobar_b,
                         const double *betamu)
{
  return guard([&] {
    Ctx *c = C(h);
    need_final(c);
    if (!w_fluid || !w_bulk || !rhobar_b || !betamu) throw Error(TGPU_ERR_ARG, "null argument");
    const tgpu::DevGeom &g = c->dg;
    const size_t n = (size_t)g.ncomp * g.N;
    if (!c->d_wf) {
      c->d_wf = dalloc<double>(n);
      c->d_wb = dalloc<double>(n);
    }
    ck(cudaMemcpyAsync(c->d_wf, w_fluid, n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "h2d");
    ck(cudaMemcpyAsync(c->d_wb, w_bulk, n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "h2d");
    tgpu::ObjConst oc{};
    for (int ic = 0; ic < g.ncomp; ic++) {
      const double rb = g.rho_b[ic];
      oc.betamu[ic] = betamu[ic];
      oc.bulk[ic] = rb * (std::log(rb) - 1.0) - rb * betamu[ic] + (g.attraction ? 0.5 * rb * g.betamu_att[ic] : 0.0);
    }
    // bulk weighted densities (n3 n2 n1 n0 in solution-vector order), vectors zero
    double nb[tgpu::kMaxRb] = {0.0};
    nb[0] = rhobar_b[3];
    nb[1] = rhobar_b[2];
    nb[2] = rhobar_b[1];
    nb[3] = rhobar_b[0];
    oc.phi_b = tgpu::fmt_phi(nb, g.ndim, g.functional);
    c->oc = oc;
    c->have_integ = true;
    ck(cudaStreamSynchronize(c->stream), "sync");
    return TGPU_OK;
  });
}

int tgpu_objectives_device(tgpu_handle h, const double *d_x, double *omega_s, double *gamma_ex)
{
  return guard([&] {
    Ctx *c = C(h);
    need_integ(c);
    objectives_device(c, a22_in(c, d_x, A22_SUMS, 0), omega_s, gamma_ex);
    return TGPU_OK;
  });
}

int tgpu_objectives(tgpu_handle h, const double *x, double *omega_s, double *gamma_ex)
{
  return guard([&] {
    Ctx *c = C(h);
    need_integ(c);
    h2d(c, c->d_work, x, (size_t)c->nunk_ext * c->dg.N);
    objectives_device(c, a22_in(c, c->d_work, A22_SUMS, 0), omega_s, gamma_ex);
    return TGPU_OK;
  });
}

int tgpu_objective_grad_device(tgpu_handle h, const double *d_x, int kind, int icomp, double *d_gx, double *d_gv)
{
  return guard([&] {
    Ctx *c = C(h);
    need_integ(c);
    double *o = a22_out_buf(c, d_gx, 1);
    objective_grad_device(c, a22_in(c, d_x, A22_SUMS, 0), kind, icomp, o, d_gv);
    a22_out(c, o, d_gx);
    ck(cudaGetLastError(), "objective gradient");
    return TGPU_OK;
  });
}

int tgpu_grad_vext_device(tgpu_handle h, const double *d_x, int kind, int icomp, double tol, int max_iter,
                          double *d_dF_dV, int *iters)
{
  return guard([&] {
    int it = 0;
    Ctx *c = C(h);
    need_integ(c);
    const int st = grad_vext_device(c, a22_in(c, d_x, A22_SUMS, 2), kind, icomp, tol, max_iter, d_dF_dV, &it);
    if (iters) *iters = it;
    return st;
  });
}

namespace {
int grad_vext_host(tgpu_handle h, const double *x, int kind, int icomp, double tol, int max_iter, double *dF_dV,
                   int *iters)
{
  return guard([&] {
    Ctx *c = C(h);
    need_integ(c);
    const size_t n = (size_t)c->nunk_ext * c->dg.N;
    h2d(c, c->d_work, x, n);
    int it = 0;
    const int st = grad_vext_device(c, a22_in(c, c->d_work, A22_SUMS, 2), kind, icomp, tol, max_iter, c->d_work2, &it);
    d2h(c, dF_dV, c->d_work2, (size_t)c->dg.ncomp * c->dg.N);
    if (iters) *iters = it;
    return st;
  });
}
}  // namespace

int tgpu_grad_omega_vext(tgpu_handle h, const double *x, double tol, int max_iter, double *dOmega_dV, int *iters)
{
  return grad_vext_host(h, x, TGPU_OBJ_OMEGA, 0, tol, max_iter, dOmega_dV, iters);
}

int tgpu_grad_gamma_vext(tgpu_handle h, const double *x, int icomp, double tol, int max_iter, double *dGamma_dV,
                         int *iters)
{
  return grad_vext_host(h, x, TGPU_OBJ_GAMMA, icomp, tol, max_iter, dGamma_dV, iters);
}

int tgpu_grad_epsw(tgpu_handle h, const double *x, int kind, int icomp, const double *dvext_deps, double tol,
                   int max_iter, double *dF_deps, int *iters)
{
  if (!dvext_deps || !dF_deps) return guard([&]() -> int { throw Error(TGPU_ERR_ARG, "null argument"); });
  Ctx *c = nullptr;
  const int st0 = guard([&] { c = C(h); need_integ(c); return TGPU_OK; });
  if (st0 != TGPU_OK) return st0;
  const size_t n = (size_t)c->dg.ncomp * c->dg.N;
  std::vector<double> s(n);
  const int st = grad_vext_host(h, x, kind, icomp, tol, max_iter, s.data(), iters);
  if (st != TGPU_OK && st != TGPU_ERR_NOCONV) return st;
  double acc = 0.0;
  for (size_t k = 0; k < n; k++) acc += s[k] * dvext_deps[k];
  *dF_deps = acc;
  return st;
}

}  // extern "C"
