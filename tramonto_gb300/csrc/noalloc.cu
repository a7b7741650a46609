// Allocation-free stencil sum: tgpu_stencil_sum_noalloc (see include/tramonto_gpu.h).
//
// Some callers cannot call cudaMalloc at the point where they need this sum:
// code running inside a framework that owns all device memory (a custom
// operator whose buffers come from the framework's allocator), or code that
// must not allocate between two phases of a larger computation.  This entry
// point takes the field and the output as device pointers from the caller and
// keeps its own scratch - the padded copy of the field, the boundary maps and
// the stencil table - in fixed-size arrays that live in this file for as long
// as the library is loaded.  It calls no cudaMalloc, cudaFree or allocating
// library routine.
//
// The arrays are shared by every call on a device and keep the last call's
// contents; every call rewrites all of the scratch it reads, so nothing has to
// start at zero.  Two calls whose work overlaps on the GPU (different streams,
// or the same arrays in flight) race on the scratch.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/tramonto_gpu.h"

namespace {

constexpr long kPadMax = TGPU_NOALLOC_MAX_PADDED;     // padded-box points
constexpr int kStenMax = TGPU_NOALLOC_MAX_STENCIL;    // stencil points
constexpr int kMapMax = 4096;                         // padded extent per dimension

static __device__ __align__(256) double g_pad[kPadMax];
static __device__ __align__(256) double g_w[kStenMax];
static __device__ __align__(256) int g_loff[kStenMax];
static __device__ __align__(256) int g_map[3 * kMapMax];

struct DevPtrs {
  double *pad = nullptr, *w = nullptr;
  int *loff = nullptr, *map = nullptr;
  bool ready = false;
};

constexpr int kMaxDevices = 64;
DevPtrs g_dev[kMaxDevices];
std::mutex g_mu;
thread_local char g_msg[256];

constexpr int kSentBulk = -1, kSentWall = -2, kSentBad = -9;
constexpr int kReflBit = 1 << 30;

struct Geo {
  int ndim, nx[3], h[3], P[3];
  long N, NP, pstride[3];
};

__global__ void k_na_pad(const double *__restrict__ field, double bulk, Geo g, const int *__restrict__ map,
                         double *__restrict__ pad)
{
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < g.NP; p += (long)gridDim.x * blockDim.x) {
    const int q[3] = {(int)(p % g.P[0]), (int)((p / g.P[0]) % g.P[1]), (int)(p / ((long)g.P[0] * g.P[1]))};
    int sent = 0, idx[3] = {0, 0, 0};
    for (int d = 0; d < g.ndim; d++) {
      const int m = map[d * kMapMax + q[d]];
      if (m < 0) { sent = m; break; }
      idx[d] = m & ~kReflBit;
    }
    double v;
    if (sent == kSentBulk) v = bulk;
    else if (sent == kSentWall) v = 0.0;
    else v = field[idx[0] + (long)g.nx[0] * (idx[1] + (long)g.nx[1] * idx[2])];
    pad[p] = v;
  }
}

__global__ void k_na_sum(const double *__restrict__ pad, const int *__restrict__ loff,
                         const double *__restrict__ w, int L, Geo g, double *__restrict__ out)
{
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.N) return;
  const int ix = (int)(i % g.nx[0]);
  const long r = i / g.nx[0];
  const int iy = (int)(r % g.nx[1]), iz = (int)(r / g.nx[1]);
  const long ip = (ix + g.h[0]) + g.pstride[1] * (iy + g.h[1]) + g.pstride[2] * (iz + g.h[2]);
  double acc = 0.0;
  for (int k = 0; k < L; k++) acc = fma(w[k], pad[ip + loff[k]], acc);
  out[i] = acc;
}

int fail(int code, const char *msg)
{
  std::snprintf(g_msg, sizeof(g_msg), "%s", msg);
  return code;
}

// Resolve the device addresses of the static arrays once per device, with
// that device current (the host-side names of __device__ arrays are not
// device addresses).
int device_ptrs(int dev, DevPtrs **out)
{
  if (dev < 0 || dev >= kMaxDevices) return fail(TGPU_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_mu);
  DevPtrs &d = g_dev[dev];
  if (!d.ready) {
    void *p = nullptr;
    cudaError_t e;
    if ((e = cudaGetSymbolAddress(&p, g_pad)) != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
    d.pad = static_cast<double *>(p);
    if ((e = cudaGetSymbolAddress(&p, g_w)) != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
    d.w = static_cast<double *>(p);
    if ((e = cudaGetSymbolAddress(&p, g_loff)) != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
    d.loff = static_cast<int *>(p);
    if ((e = cudaGetSymbolAddress(&p, g_map)) != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
    d.map = static_cast<int *>(p);
    d.ready = true;
  }
  *out = &d;
  return TGPU_OK;
}

// one padded dimension: q -> node (with reflect bit) or sentinel, as offset_to_node_box; false when a
// padded position has no node to read: a periodic reach longer than the box, or a mirrored position that
// falls past the far side without a bulk or wall rule there
bool fill_map(int n, int h, int bcl, int bcr, int *m)
{
  for (int q = 0; q < n + 2 * h; q++) {
    int s = q - h, v;
    if (s < 0) {
      if (bcl == TGPU_BC_IN_BULK) v = kSentBulk;
      else if (bcl == TGPU_BC_IN_WALL) v = kSentWall;
      else if (bcl == TGPU_BC_REFLECT) {
        s = -s;
        v = s < n ? (s | kReflBit) : (bcr == TGPU_BC_IN_BULK ? kSentBulk : bcr == TGPU_BC_IN_WALL ? kSentWall : kSentBad);
      } else { s += n; v = s >= 0 ? s : kSentBad; }
    } else if (s >= n) {
      if (bcr == TGPU_BC_IN_BULK) v = kSentBulk;
      else if (bcr == TGPU_BC_IN_WALL) v = kSentWall;
      else if (bcr == TGPU_BC_REFLECT) {
        s = 2 * (n - 1) - s;
        v = s >= 0 ? (s | kReflBit) : (bcl == TGPU_BC_IN_BULK ? kSentBulk : bcl == TGPU_BC_IN_WALL ? kSentWall : kSentBad);
      } else { s -= n; v = s < n ? s : kSentBad; }
    } else {
      v = s;
    }
    if (v == kSentBad) return false;
    m[q] = v;
  }
  return true;
}

}  // namespace

extern "C" {

const char *tgpu_noalloc_last_error(void) { return g_msg; }

int tgpu_stencil_sum_noalloc(int ndim, const int *nx, const int *bc, double bulk_value, int length,
                             const short *offsets, const double *weights, const double *d_field, double *d_out,
                             void *stream)
{
  if (ndim < 1 || ndim > 3 || !nx || !bc || !d_field || !d_out) return fail(TGPU_ERR_ARG, "null or bad argument");
  if (length < 0 || length > kStenMax) return fail(TGPU_ERR_ARG, "stencil longer than TGPU_NOALLOC_MAX_STENCIL");
  if (length > 0 && (!offsets || !weights)) return fail(TGPU_ERR_ARG, "null stencil arrays");
  for (int d = 0; d < ndim; d++)
    for (int k = 0; k < 2; k++)
      if (bc[2 * d + k] < TGPU_BC_IN_WALL || bc[2 * d + k] > TGPU_BC_REFLECT)
        return fail(TGPU_ERR_UNSUPPORTED, "boundary condition");
  Geo g{};
  g.ndim = ndim;
  int h[3] = {0, 0, 0};
  for (int k = 0; k < length; k++)
    for (int d = 0; d < ndim; d++) {
      const int o = offsets[(long)k * ndim + d];
      h[d] = o < 0 ? (h[d] > -o ? h[d] : -o) : (h[d] > o ? h[d] : o);
    }
  g.N = 1;
  long NP = 1;
  for (int d = 0; d < 3; d++) {
    g.nx[d] = d < ndim ? nx[d] : 1;
    if (g.nx[d] < 1) return fail(TGPU_ERR_ARG, "nx must be positive");
    if (g.nx[d] > kMapMax) return fail(TGPU_ERR_ARG, "padded extent above 4096 in a dimension");
    g.h[d] = d < ndim ? h[d] : 0;
    const long P = (long)g.nx[d] + 2L * g.h[d];
    if (P > kMapMax) return fail(TGPU_ERR_ARG, "padded extent above 4096 in a dimension");
    g.P[d] = (int)P;
    NP *= P;
    g.N *= g.nx[d];
  }
  if (NP > kPadMax) return fail(TGPU_ERR_ARG, "padded box larger than TGPU_NOALLOC_MAX_PADDED points");
  g.NP = NP;
  g.pstride[0] = 1;
  g.pstride[1] = g.P[0];
  g.pstride[2] = (long)g.P[0] * g.P[1];
  // host-side staging of the maps and offsets (host memory, reused per thread); the maps are checked before
  // any device work, so a rejected call leaves the device untouched
  static thread_local int h_map[3 * kMapMax];
  static thread_local int h_loff[kStenMax];
  for (int d = 0; d < 3; d++) {
    if (d >= ndim) {
      h_map[d * kMapMax] = 0;
    } else if (!fill_map(g.nx[d], g.h[d], bc[2 * d], bc[2 * d + 1], h_map + d * kMapMax)) {
      return fail(TGPU_ERR_UNSUPPORTED,
                  "stencil reaches past the box: a periodic reach longer than the box, or a mirrored point beyond "
                  "the far side without a bulk or wall boundary there");
    }
  }
  for (int k = 0; k < length; k++) {
    long o = 0;
    for (int d = 0; d < ndim; d++) o += (long)offsets[(long)k * ndim + d] * g.pstride[d];
    h_loff[k] = (int)o;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
  DevPtrs *dp = nullptr;
  int st = device_ptrs(dev, &dp);
  if (st != TGPU_OK) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if ((e = cudaMemcpyAsync(dp->map, h_map, sizeof(int) * 3 * kMapMax, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
      (length > 0 && (e = cudaMemcpyAsync(dp->loff, h_loff, sizeof(int) * length, cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
      (length > 0 && (e = cudaMemcpyAsync(dp->w, weights, sizeof(double) * length, cudaMemcpyHostToDevice, s)) != cudaSuccess))
    return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
  k_na_pad<<<592, 256, 0, s>>>(d_field, bulk_value, g, dp->map, dp->pad);
  k_na_sum<<<(unsigned)((g.N + 255) / 256), 256, 0, s>>>(dp->pad, dp->loff, dp->w, length, g, d_out);
  // a launch that could not start reports here, before the wait
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
  // the host tables above are reused by the next call: wait for the copies to land
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail(TGPU_ERR_CUDA, cudaGetErrorString(e));
  return TGPU_OK;
}

}  // extern "C"
