// FP64 three-dimensional FFTs for the stencil sums of the accurate fills.
//
// A stencil sum out(i) = sum_o c(o) f(i + h + o) over the padded box is a correlation; with the kernel
// g[(-o) mod F] = c(o) it is the circular convolution (f * g)(i + h), exact for interior outputs when
// every F_d >= P_d (the padded extent: i + h + o stays inside [0, P)).  So one forward transform of the
// padded channel, a pointwise product with the kernel's spectrum (computed once per stencil coefficient)
// and one inverse transform give a sum whose cost does not depend on the stencil's length: for the
// 71 831-point attraction stencil at 128^3 that is ~2 transforms of 180^3 against 1.5e11 terms.
// Rounding: FP64 FFTs with tabulated twiddles keep the error near eps log2(NF) of the sum's scale.
//
// Each axis is a batch of 1-D transforms.  A CTA loads kFftLines lines and the twiddle table into shared
// memory (coalesced:
// consecutive lines along x for the y and z axes, whole contiguous lines for x), runs the stages of a
// mixed-radix Stockham autosort FFT there (radices 2, 3, 4, 5; the iteration of Govindaraju, Lloyd,
// Dotsenko, Smith and Manferdelli, "High performance discrete Fourier transforms on graphics
// processors", SC 2008: butterfly j reads j + r n/R, multiplies by W_{Ns R}^{r (j mod Ns)}, takes an
// R-point DFT and writes (j / Ns) Ns R + (j mod Ns) + r Ns), and writes the lines back in place.
// The inverse uses conjugate twiddles; its 1/NF goes into the extraction.
#include <cmath>
#include <vector>

#include "tgpu_internal.h"

namespace tgpu {

namespace {

constexpr int kFftLines = 8;
constexpr int kFftThreads = 256;
constexpr int kFftMaxN = 432;   // two ping-pong tiles of kFftLines lines and the twiddles fit in shared memory

struct Stages {
  int nst;
  int rad[16];
};

// complex arithmetic on double2 (FP64 sums of the accurate fills) and float2 (FP32 sums of the products)
template <class C>
__device__ __forceinline__ C cmul(C a, C b)
{
  return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <class C>
__device__ __forceinline__ C cadd(C a, C b)
{
  return C{a.x + b.x, a.y + b.y};
}
template <class C>
__device__ __forceinline__ C csub(C a, C b)
{
  return C{a.x - b.x, a.y - b.y};
}

// tw points at the axis's table in shared memory
template <class C>
__device__ __forceinline__ C twiddle(const C *tw, int k, int inv)
{
  C w = tw[k];
  if (inv) w.y = -w.y;
  return w;
}

// R-point DFT of v in place (forward: exp(-2 pi i r k / R); inverse: conjugate); R known at compile time so
// that v stays in registers
template <int R, class C>
__device__ __forceinline__ void dft_small(C *v, const C *tw, int n, int inv)
{
  if (R == 2) {
    const C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (R == 4) {
    const C y0 = cadd(v[0], v[2]), y1 = csub(v[0], v[2]), y2 = cadd(v[1], v[3]);
    C y3 = csub(v[1], v[3]);
    y3 = inv ? C{-y3.y, y3.x} : C{y3.y, -y3.x};   // times +i (inverse) or -i
    v[0] = cadd(y0, y2);
    v[2] = csub(y0, y2);
    v[1] = cadd(y1, y3);
    v[3] = csub(y1, y3);
  } else {
    C w[R];   // W_R^m from the table: W_n^(m n / R)
#pragma unroll
    for (int m = 0; m < R; m++) w[m] = twiddle(tw, m * (n / R), inv);
    C o[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
      C s = v[0];
#pragma unroll
      for (int r = 1; r < R; r++) s = cadd(s, cmul(v[r], w[(r * k) % R]));
      o[k] = s;
    }
#pragma unroll
    for (int k = 0; k < R; k++) v[k] = o[k];
  }
}

// one Stockham stage of radix R over nlines lines of line stride ls
template <int R, class C>
__device__ __forceinline__ void fft_stage(const C *in, C *out, int n, int ls, int nlines, int Ns, const C *tw, int inv)
{
  const int nb = n / R, step = n / (Ns * R);
  for (int t = threadIdx.x; t < nlines * nb; t += blockDim.x) {
    const int line = t / nb, j = t - line * nb;
    const C *src = in + line * ls;
    C *dst = out + line * ls;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * nb];
    const int k = j % Ns;
#pragma unroll
    for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tw, r * k * step, inv));
    dft_small<R, C>(v, tw, n, inv);
    const int idx = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) dst[idx + r * Ns] = v[r];
  }
}

// stages of one tile of kFftLines lines (line stride ls) from buf0; returns the buffer holding the result
template <class C>
__device__ C *fft_tile(C *buf0, C *buf1, int n, int ls, int nlines, const Stages &st, const C *tw, int inv)
{
  C *in = buf0, *out = buf1;
  int Ns = 1;
  for (int s = 0; s < st.nst; s++) {
    const int R = st.rad[s];
    switch (R) {
      case 2: fft_stage<2, C>(in, out, n, ls, nlines, Ns, tw, inv); break;
      case 3: fft_stage<3, C>(in, out, n, ls, nlines, Ns, tw, inv); break;
      case 4: fft_stage<4, C>(in, out, n, ls, nlines, Ns, tw, inv); break;
      default: fft_stage<5, C>(in, out, n, ls, nlines, Ns, tw, inv); break;
    }
    __syncthreads();
    C *t = in;
    in = out;
    out = t;
    Ns *= R;
  }
  return in;
}

// axis 0: lines along x (contiguous), kFftLines consecutive lines per CTA
template <class C>
__global__ void __launch_bounds__(kFftThreads) k_fft_x(C *box, int F0, long nlines_total, Stages st,
                                                     const C *__restrict__ tw_g, int inv)
{
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int n = F0, ls = n + 1;
  C *b0 = sm, *b1 = sm + kFftLines * ls, *tw = b1 + kFftLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  const long l0 = (long)blockIdx.x * kFftLines;
  const int nl = (int)min((long)kFftLines, nlines_total - l0);
  for (int q = threadIdx.x; q < nl * n; q += blockDim.x) {
    const int l = q / n, e = q - l * n;
    b0[l * ls + e] = box[(l0 + l) * n + e];
  }
  __syncthreads();
  const C *res = fft_tile<C>(b0, b1, n, ls, nl, st, tw, inv);
  for (int q = threadIdx.x; q < nl * n; q += blockDim.x) {
    const int l = q / n, e = q - l * n;
    box[(l0 + l) * n + e] = res[l * ls + e];
  }
}

// axes 1 and 2: lines of element stride es; a CTA takes kFftLines consecutive x at one (outer) index
template <class C>
__global__ void __launch_bounds__(kFftThreads) k_fft_strided(C *box, int F0, int n, long es, long outer_stride,
                                                           Stages st, const C *__restrict__ tw_g, int inv)
{
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int ls = n + 1;
  C *b0 = sm, *b1 = sm + kFftLines * ls, *tw = b1 + kFftLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  const int xblocks = (F0 + kFftLines - 1) / kFftLines;
  const int x0 = (blockIdx.x % xblocks) * kFftLines;
  const long base = (long)(blockIdx.x / xblocks) * outer_stride + x0;
  const int nl = min(kFftLines, F0 - x0);
  for (int q = threadIdx.x; q < kFftLines * n; q += blockDim.x) {
    const int e = q / kFftLines, l = q - e * kFftLines;
    if (l < nl) b0[l * ls + e] = box[base + e * es + l];
  }
  __syncthreads();
  const C *res = fft_tile<C>(b0, b1, n, ls, nl, st, tw, inv);
  for (int q = threadIdx.x; q < kFftLines * n; q += blockDim.x) {
    const int e = q / kFftLines, l = q - e * kFftLines;
    if (l < nl) box[base + e * es + l] = res[l * ls + e];
  }
}

template <class T, class C>
__global__ void k_fft_load(const T *__restrict__ pad, int P0, int P1, int P2, C *__restrict__ box, int F0, int F1,
                           long NF)
{
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < NF; q += (long)gridDim.x * blockDim.x) {
    const int x = (int)(q % F0);
    const long r = q / F0;
    const int y = (int)(r % F1), z = (int)(r / F1);
    T v = 0;
    if (x < P0 && y < P1 && z < P2) v = pad[((long)z * P1 + y) * P0 + x];
    box[q] = C{v, 0};
  }
}

__global__ void k_fft_kernel_box(const short *__restrict__ off3, const double *__restrict__ coef, int L, int ncoef,
                                 int q, double2 *__restrict__ box, int F0, int F1, int F2)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= L) return;
  const int x = ((-(int)off3[3 * k]) % F0 + F0) % F0;
  const int y = ((-(int)off3[3 * k + 1]) % F1 + F1) % F1;
  const int z = ((-(int)off3[3 * k + 2]) % F2 + F2) % F2;
  box[((long)z * F1 + y) * F0 + x] = make_double2(coef[(long)k * ncoef + q], 0.0);
}

template <class C>
__global__ void k_spec_mul(const C *__restrict__ a, const C *__restrict__ k, C *__restrict__ out, long n, int accumulate)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const C p = cmul(a[i], k[i]);
    out[i] = accumulate ? cadd(out[i], p) : p;
  }
}

template <class C>
__global__ void k_fft_extract(const C *__restrict__ box, int F0, int F1, int h0, int h1, int h2, int nx0, int nx1,
                              long N, double scale, double *__restrict__ out)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx0);
    const long r = i / nx0;
    const int y = (int)(r % nx1), z = (int)(r / nx1);
    out[i] += (double)box[((long)(z + h2) * F1 + (y + h1)) * F0 + (x + h0)].x * scale;
  }
}

__global__ void k_to_float2(const double2 *__restrict__ in, float2 *__restrict__ out, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

int grid_for(long n) { return (int)std::min<long>((n + 255) / 256, 152L * 16); }

// smallest F >= P that is a product of 2, 3, 5, and its radix list (4s first)
bool choose(int P, int &F, Stages &st)
{
  for (F = std::max(P, 1); F <= kFftMaxN; F++) {
    int m = F;
    for (int r : {2, 3, 5})
      while (m % r == 0) m /= r;
    if (m == 1) break;
  }
  if (F > kFftMaxN) return false;
  int m = F;
  st.nst = 0;
  while (m % 4 == 0) { st.rad[st.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { st.rad[st.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { st.rad[st.nst++] = 3; m /= 3; }
  while (m % 5 == 0) { st.rad[st.nst++] = 5; m /= 5; }
  return st.nst <= 16;
}

template <class C>
size_t tile_smem(int n)
{
  return sizeof(C) * (2 * (size_t)kFftLines * (n + 1) + n);
}

template <class C>
void set_smem_limits(const FftPlan &p, int ndim)
{
  size_t sx = tile_smem<C>(p.F[0]), ss = 0;
  for (int d = 1; d < ndim; d++) ss = std::max(ss, tile_smem<C>(p.F[d]));
  cudaFuncSetAttribute(k_fft_x<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sx);
  if (ss) cudaFuncSetAttribute(k_fft_strided<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ss);
}

template <class C>
void fft3d_impl(C *box, const FftPlan &p, int ndim, bool inverse, const C *const *tw, cudaStream_t s)
{
  const int F0 = p.F[0], F1 = p.F[1], F2 = p.F[2];
  for (int d = 0; d < ndim; d++) {
    const FftAxis &a = p.ax[d];
    Stages st{};
    st.nst = a.nst;
    for (int k = 0; k < a.nst; k++) st.rad[k] = a.rad[k];
    const size_t sm = tile_smem<C>(a.n);
    if (d == 0) {
      const long nl = (long)F1 * F2;
      k_fft_x<C><<<(unsigned)((nl + kFftLines - 1) / kFftLines), kFftThreads, sm, s>>>(box, F0, nl, st, tw[d],
                                                                                       inverse ? 1 : 0);
    } else {
      const int xblocks = (F0 + kFftLines - 1) / kFftLines;
      const long es = d == 1 ? (long)F0 : (long)F0 * F1;
      const long outer = d == 1 ? (long)F0 * F1 : (long)F0;   // axis 1: outer index z; axis 2: outer index y
      const long nouter = d == 1 ? F2 : F1;
      k_fft_strided<C><<<(unsigned)(xblocks * nouter), kFftThreads, sm, s>>>(box, F0, a.n, es, outer, st, tw[d],
                                                                             inverse ? 1 : 0);
    }
  }
}

}  // namespace

bool fft_make_plan(FftPlan &p, const int P[3], int ndim, cudaStream_t s)
{
  p.NF = 1;
  for (int d = 0; d < 3; d++) {
    FftAxis &a = p.ax[d];
    if (d >= ndim) {
      p.F[d] = 1;
      a.n = 1;
      a.nst = 0;
      continue;
    }
    Stages st{};
    if (!choose(P[d], p.F[d], st)) return false;
    a.n = p.F[d];
    a.nst = st.nst;
    for (int k = 0; k < st.nst; k++) a.rad[k] = st.rad[k];
    std::vector<double2> tw(a.n);
    std::vector<float2> tw32(a.n);
    for (int k = 0; k < a.n; k++) {
      // exp(-2 pi i k / n) from the host library in extended precision, rounded once
      const long double ang = -2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)a.n;
      tw[k] = make_double2((double)std::cos(ang), (double)std::sin(ang));
      tw32[k] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    if (cudaMalloc(&a.d_tw, sizeof(double2) * a.n) != cudaSuccess) return false;
    if (cudaMalloc(&a.d_tw32, sizeof(float2) * a.n) != cudaSuccess) return false;
    cudaMemcpyAsync(a.d_tw, tw.data(), sizeof(double2) * a.n, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(a.d_tw32, tw32.data(), sizeof(float2) * a.n, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);   // the host tables go out of scope
    p.NF *= p.F[d];
  }
  set_smem_limits<double2>(p, ndim);
  set_smem_limits<float2>(p, ndim);
  return true;
}

void fft_free_plan(FftPlan &p)
{
  for (auto &a : p.ax) {
    if (a.d_tw) cudaFree(a.d_tw);
    if (a.d_tw32) cudaFree(a.d_tw32);
    a.d_tw = nullptr;
    a.d_tw32 = nullptr;
  }
}

void fft3d(double2 *box, const FftPlan &p, int ndim, bool inverse, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  fft3d_impl<double2>(box, p, ndim, inverse, tw, s);
}

void fft3d(float2 *box, const FftPlan &p, int ndim, bool inverse, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  fft3d_impl<float2>(box, p, ndim, inverse, tw, s);
}

void launch_fft_load(const double *pad, const int P[3], double2 *box, const FftPlan &p, cudaStream_t s)
{
  k_fft_load<double, double2><<<grid_for(p.NF), 256, 0, s>>>(pad, P[0], P[1], P[2], box, p.F[0], p.F[1], p.NF);
}

void launch_fft_load(const float *pad, const int P[3], float2 *box, const FftPlan &p, cudaStream_t s)
{
  k_fft_load<float, float2><<<grid_for(p.NF), 256, 0, s>>>(pad, P[0], P[1], P[2], box, p.F[0], p.F[1], p.NF);
}

void launch_fft_kernel_box(const short *off3, const double *coef, int L, int ncoef, int q, double2 *box,
                           const FftPlan &p, cudaStream_t s)
{
  cudaMemsetAsync(box, 0, sizeof(double2) * p.NF, s);
  if (L > 0) k_fft_kernel_box<<<(L + 255) / 256, 256, 0, s>>>(off3, coef, L, ncoef, q, box, p.F[0], p.F[1], p.F[2]);
}

void launch_to_float2(const double2 *in, float2 *out, long n, cudaStream_t s)
{
  k_to_float2<<<grid_for(n), 256, 0, s>>>(in, out, n);
}

void launch_spec_mul(const double2 *a, const double2 *k, double2 *out, long n, bool accumulate, cudaStream_t s)
{
  k_spec_mul<double2><<<grid_for(n), 256, 0, s>>>(a, k, out, n, accumulate ? 1 : 0);
}

void launch_spec_mul(const float2 *a, const float2 *k, float2 *out, long n, bool accumulate, cudaStream_t s)
{
  k_spec_mul<float2><<<grid_for(n), 256, 0, s>>>(a, k, out, n, accumulate ? 1 : 0);
}

void launch_fft_extract(const double2 *box, const FftPlan &p, const int h[3], const int nx[3], double scale,
                        double *out, cudaStream_t s)
{
  const long N = (long)nx[0] * nx[1] * nx[2];
  k_fft_extract<double2><<<grid_for(N), 256, 0, s>>>(box, p.F[0], p.F[1], h[0], h[1], h[2], nx[0], nx[1], N, scale,
                                                     out);
}

void launch_fft_extract(const float2 *box, const FftPlan &p, const int h[3], const int nx[3], double scale,
                        double *out, cudaStream_t s)
{
  const long N = (long)nx[0] * nx[1] * nx[2];
  k_fft_extract<float2><<<grid_for(N), 256, 0, s>>>(box, p.F[0], p.F[1], h[0], h[1], h[2], nx[0], nx[1], N, scale,
                                                    out);
}

}  // namespace tgpu
