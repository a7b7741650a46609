// Device kernels of the nonlocal-density path (FP64 and FP32 stencil sums,
// local FMT physics, residual assembly, Schur-operator local steps, Krylov
// and Newton vector kernels).
//
// Reference correspondence (file:line in the reference tree):
//   k_fmt_local      calc_FMT_derivatives + FMT1/FMT3_1stderiv  src/dft_fill_FMT.c:349-385,
//                    src/dft_physics_FMT1.c:59-77, src/dft_physics_FMT3.c:61-96
//   k_pad            offset_to_node_box boundary rules          src/dft_mesh_lib.c:203-297
//                    constant_boundary                          src/dft_utils.c:90-150
//   k_conv           the stencil loops of resid_and_Jac_sten_fill_sum_Ncomp
//                    (src/dft_fill_CLSmf.c:129-169) and load_nonlocal_hs_rosen_rb
//                    (src/dft_fill_FMT.c:77-133)
//   k_hw_correct     HW_boundary_weight                         src/dft_utils.c:41-62
//   k_assemble       load_euler_lagrange / load_rho_bar_s/v / load_mean_field
//                    src/dft_fill_EL.c:38-196, src/dft_fill_FMT.c:195-347, src/dft_fill_mf.c:38-63
//   k_schur_local    A11^-1 (src/dft_HardSphereA11_Epetra_Operator.cpp:176-192) and the
//                    local Hessian that the reference spreads over d2phi_drb2_* per stencil
//                    point (src/dft_physics_FMT1.c:79-168, src/dft_physics_FMT3.c:101-265)
//   k_newton_*       update_solution                            src/dft_newton.c:266-381
#include <cstdio>
#include <cstdlib>

#include "tgpu_internal.h"

namespace tgpu {

__constant__ DevGeom c_g;

void upload_geom(const DevGeom &g, cudaStream_t s)
{
  cudaMemcpyToSymbolAsync(c_g, &g, sizeof(DevGeom), 0, cudaMemcpyHostToDevice, s);
}

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr int kThreads = 256;

__device__ __forceinline__ void node_ijk(long i, int *ijk)
{
  ijk[0] = (int)(i % c_g.nx[0]);
  long r = i / c_g.nx[0];
  ijk[1] = (int)(r % c_g.nx[1]);
  ijk[2] = (int)(r / c_g.nx[1]);
}

__device__ __forceinline__ long pad_center(long i)
{
  int ijk[3];
  node_ijk(i, ijk);
  return (long)(ijk[0] + c_g.h[0]) + c_g.pstride[1] * (ijk[1] + c_g.h[1]) + c_g.pstride[2] * (ijk[2] + c_g.h[2]);
}

// ---------------------------------------------------------------------------
// Padding: resolve each padded position to a source node or a sentinel with
// the reference's dimension order (the first out-of-range dimension decides).
// With no_mirror, mirrored positions read 0: the zero extension of a field that the transposed sums of a
// problem with reflecting boundaries start from (their mirrored contributions are folded back separately).
template <typename T>
__global__ void k_pad(const double *__restrict__ src, T *__restrict__ dst, int nch, const double *__restrict__ bulk,
                      const int *__restrict__ signmask, const int *__restrict__ zcomp,
                      const signed char *__restrict__ zero, int no_mirror)
{
  const long NP = c_g.NP;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < NP; p += (long)gridDim.x * blockDim.x) {
    const int q0 = (int)(p % c_g.P[0]);
    const long r = p / c_g.P[0];
    const int q1 = (int)(r % c_g.P[1]);
    const int q2 = (int)(r / c_g.P[1]);
    const int q[3] = {q0, q1, q2};
    int sent = 0, refl = 0;
    int idx[3] = {0, 0, 0};
    for (int d = 0; d < c_g.ndim; d++) {
      const int m = c_g.map[d][q[d]];
      if (m < 0) { sent = m; break; }
      if (m & kReflBit) refl |= 1 << d;
      idx[d] = m & ~kReflBit;
    }
    const long node = idx[0] + (long)c_g.nx[0] * (idx[1] + (long)c_g.nx[1] * idx[2]);
    for (int ch = 0; ch < nch; ch++) {
      double v;
      if (sent == kSentBulk) v = bulk[ch];
      else if (sent == kSentBulkHi) v = bulk[nch + ch];   // the high side's bulk (phase interfaces)
      else if (sent == kSentWall) v = 0.0;
      else if (sent != 0) v = __longlong_as_double(0x7ff8000000000000ULL);
      else if (no_mirror && refl) v = 0.0;
      else {
        v = src[(long)ch * c_g.N + node];
        const int zc = zcomp[ch];
        if (zc >= 0 && zero[(long)zc * c_g.N + node]) v = 0.0;
        if (__popc(refl & signmask[ch]) & 1) v = -v;
      }
      dst[(long)ch * NP + p] = (T)v;
    }
  }
}

template <typename T>
void launch_pad(const double *src, T *dst, int nch, const double *bulk, const int *signmask, const int *zcomp,
                const signed char *zero, bool no_mirror, cudaStream_t s)
{
  // bulk/signmask/zcomp live in device memory (small arrays set up by the caller)
  k_pad<T><<<1184, kThreads, 0, s>>>(src, dst, nch, bulk, signmask, zcomp, zero, no_mirror ? 1 : 0);
}
template void launch_pad<double>(const double *, double *, int, const double *, const int *, const int *,
                                 const signed char *, bool, cudaStream_t);
template void launch_pad<float>(const double *, float *, int, const double *, const int *, const int *,
                                const signed char *, bool, cudaStream_t);

// ---------------------------------------------------------------------------
// Stencil sums.  One thread per output node; the stencil's linear offsets and
// coefficient rows stream through shared memory in chunks that every thread
// of the block reads in the same order (broadcast), the inputs are gathered
// from the padded box (neighbouring threads read neighbouring addresses).
struct OutPtrs {
  double *p[kMaxRb];
};

constexpr int kChunk = 256;

template <typename T, typename Acc, int NIN, int NOUT>
__global__ void __launch_bounds__(kThreads) k_conv(const T *__restrict__ in, long cstride,
                                                    const int *__restrict__ loff, const T *__restrict__ coef, int L,
                                                    OutPtrs out, int accumulate)
{
  __shared__ int s_off[kChunk];
  __shared__ T s_coef[kChunk * NIN * NOUT];
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool active = i < c_g.N;
  const long ip = active ? pad_center(i) : 0;
  Acc acc[NOUT];
#pragma unroll
  for (int o = 0; o < NOUT; o++) acc[o] = 0;
  for (int k0 = 0; k0 < L; k0 += kChunk) {
    const int n = min(kChunk, L - k0);
    __syncthreads();
    for (int t = threadIdx.x; t < n; t += blockDim.x) s_off[t] = loff[k0 + t];
    for (int t = threadIdx.x; t < n * NIN * NOUT; t += blockDim.x) s_coef[t] = coef[(long)k0 * NIN * NOUT + t];
    __syncthreads();
    if (active) {
      for (int k = 0; k < n; k++) {
        const long j = ip + s_off[k];
        T v[NIN];
#pragma unroll
        for (int c = 0; c < NIN; c++) v[c] = __ldg(in + c * cstride + j);
#pragma unroll
        for (int o = 0; o < NOUT; o++)
#pragma unroll
          for (int c = 0; c < NIN; c++) acc[o] = fma((Acc)s_coef[(k * NOUT + o) * NIN + c], (Acc)v[c], acc[o]);
      }
    }
  }
  if (active) {
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
      double *dst = out.p[o];
      if (accumulate) dst[i] += (double)acc[o];
      else dst[i] = (double)acc[o];
    }
  }
}

template <typename T, typename Acc, int NIN, int NOUT>
static void conv_dispatch(const T *in, long cstride, const int *loff, const T *coef, int L, const OutPtrs &out,
                          bool acc, cudaStream_t s, long N)
{
  const int grid = (int)((N + kThreads - 1) / kThreads);
  k_conv<T, Acc, NIN, NOUT><<<grid, kThreads, 0, s>>>(in, cstride, loff, coef, L, out, acc ? 1 : 0);
}

// Coefficient rows: `coef` is the table for the shape (nin, nout) this call uses.
template <>
void launch_conv<double>(const double *in, long cstride, int nin, const int *loff, const double *coef, int L,
                         double *const *out, int nout, bool acc, long N, cudaStream_t s)
{
  OutPtrs o{};
  for (int k = 0; k < nout; k++) o.p[k] = out[k];
#define TGPU_CONV(NI, NO) \
  if (nin == NI && nout == NO) { conv_dispatch<double, double, NI, NO>(in, cstride, loff, coef, L, o, acc, s, N); return; }
  TGPU_CONV(1, 1) TGPU_CONV(1, 2) TGPU_CONV(1, 3) TGPU_CONV(1, 4) TGPU_CONV(1, 5) TGPU_CONV(1, 6) TGPU_CONV(1, 7)
  TGPU_CONV(1, 8) TGPU_CONV(1, 9) TGPU_CONV(2, 1) TGPU_CONV(3, 1) TGPU_CONV(4, 1)
#undef TGPU_CONV
  fprintf(stderr, "tgpu: no FP64 convolution for nin=%d nout=%d\n", nin, nout);
  abort();
}

template <>
void launch_conv<float>(const float *in, long cstride, int nin, const int *loff, const float *coef, int L,
                        double *const *out, int nout, bool acc, long N, cudaStream_t s)
{
  OutPtrs o{};
  for (int k = 0; k < nout; k++) o.p[k] = out[k];
#define TGPU_CONV(NI, NO) \
  if (nin == NI && nout == NO) { conv_dispatch<float, float, NI, NO>(in, cstride, loff, coef, L, o, acc, s, N); return; }
  TGPU_CONV(1, 1) TGPU_CONV(1, 2) TGPU_CONV(1, 3) TGPU_CONV(1, 4) TGPU_CONV(1, 5) TGPU_CONV(1, 6) TGPU_CONV(1, 7)
  TGPU_CONV(1, 8) TGPU_CONV(1, 9) TGPU_CONV(2, 1) TGPU_CONV(3, 1) TGPU_CONV(4, 1)
#undef TGPU_CONV
  fprintf(stderr, "tgpu: no FP32 convolution for nin=%d nout=%d\n", nin, nout);
  abort();
}

// ---------------------------------------------------------------------------
// FP32 stencil sums over x-lines.  The stencil is regrouped into lines of
// constant (oy, oz) with a contiguous run of ox (zero weights fill gaps and pad
// each run to a multiple of TX).  A thread owns TX consecutive outputs along
// x and slides a 2*TX register window over each line, so every input value
// loaded serves TX multiply-adds.  Line partial sums are combined with a
// compensated (Kahan) sum so the FP32 result keeps ~1e-7 relative accuracy
// over the ~10^5-point attraction stencil.
// ---------------------------------------------------------------------------
// FP32 single-channel stencil sums in 3-D through shared-memory slabs.
//
// A block owns a 128 (x) by 16 (y) tile of outputs in one z plane; a thread
// owns 8 consecutive x outputs of one row.  The stencil is grouped by its z
// offset oz, and within a plane into x-lines of constant oy (contiguous ox
// runs, zero-padded to a multiple of 8).  For each oz the block copies the
// input slab it needs (rows y0+oy_lo .. y0+15+oy_hi, columns x0-h .. x0+127+h+16
// of plane z+oz of the padded box) into shared memory once, then every thread
// slides a 16-value register window along each line, so one shared-memory
// load feeds 8 multiply-adds.  Shared rows insert one padding word after
// every 8 and use a pitch of 16 mod 32 words, which makes the window loads of
// a warp (16 threads 8 words apart, two rows) hit 32 distinct banks.
// Line sums are combined with a compensated (Kahan) sum.
constexpr int kSlabTX = 128, kSlabTY = 16, kSlabThreads = 256;

__device__ __forceinline__ int slab_phys(int c) { return c + (c >> 3); }

__global__ void __launch_bounds__(kSlabThreads) k_conv_slab(const float *__restrict__ in, long in_total,
                                                          const int4 *__restrict__ planes, int nplanes,
                                                          const int4 *__restrict__ lines,
                                                          const float *__restrict__ lw, double *__restrict__ out,
                                                          int pitch, int ncols, int max_rows, int max_lines,
                                                          int max_w)
{
  extern __shared__ float smem[];
  float *s_slab = smem;                                        // [max_rows][pitch]
  float *s_w = s_slab + (size_t)max_rows * pitch;              // [max_w]
  int4 *s_line = reinterpret_cast<int4 *>(s_w + max_w);       // [max_lines]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int x0 = blockIdx.x * kSlabTX, y0 = blockIdx.y * kSlabTY, z = blockIdx.z;
  const int hx = c_g.h[0];
  float sum[8], comp[8];
#pragma unroll
  for (int o = 0; o < 8; o++) { sum[o] = 0.f; comp[o] = 0.f; }
  for (int pi = 0; pi < nplanes; pi++) {
    const int4 pd = planes[2 * pi];        // {first line, line count, first weight, weight count}
    const int4 pg = planes[2 * pi + 1];    // {oz, oy_lo, oy_hi, 0}
    const int nrows = kSlabTY + pg.z - pg.y;
    __syncthreads();
    for (int k = threadIdx.x; k < pd.y; k += kSlabThreads) s_line[k] = lines[pd.x + k];
    for (int k = threadIdx.x; k < pd.w; k += kSlabThreads) s_w[k] = lw[pd.z + k];
    // padded-box coordinates of the slab origin: x0 - hx + hx = x0, row y0 + oy_lo + h1, plane z + oz + h2
    const long gz = (long)(z + pg.x + c_g.h[2]) * c_g.pstride[2];
    for (int e = threadIdx.x; e < nrows * ncols; e += kSlabThreads) {
      const int r = e / ncols, cidx = e - r * ncols;
      const int gy = y0 + pg.y + r + c_g.h[1];
      const long gi = gz + (long)gy * c_g.pstride[1] + x0 + cidx;
      float v = 0.f;
      if (gy < c_g.P[1] && gi < in_total) v = __ldg(in + gi);
      s_slab[r * pitch + slab_phys(cidx)] = v;
    }
    __syncthreads();
    for (int li = 0; li < pd.y; li++) {
      const int4 ln = s_line[li];          // {row offset oy - oy_lo, first column ox_min + hx, blocks of 8, weight offset}
      const float *row = s_slab + (ty + ln.x) * pitch;
      const float *w = s_w + (ln.w - pd.z);
      const int c0 = 8 * tx + ln.y;
      float acc[8];
#pragma unroll
      for (int o = 0; o < 8; o++) acc[o] = 0.f;
      float win[16];
#pragma unroll
      for (int q = 0; q < 8; q++) win[q] = row[slab_phys(c0 + q)];
      for (int kb = 0; kb < ln.z; kb++) {
#pragma unroll
        for (int q = 0; q < 8; q++) win[8 + q] = row[slab_phys(c0 + 8 * (kb + 1) + q)];
#pragma unroll
        for (int kk = 0; kk < 8; kk++) {
          const float wk = w[8 * kb + kk];
#pragma unroll
          for (int o = 0; o < 8; o++) acc[o] = fmaf(wk, win[o + kk], acc[o]);
        }
#pragma unroll
        for (int q = 0; q < 8; q++) win[q] = win[8 + q];
      }
#pragma unroll
      for (int o = 0; o < 8; o++) {
        const float yv = acc[o] - comp[o];
        const float tv = sum[o] + yv;
        comp[o] = (tv - sum[o]) - yv;
        sum[o] = tv;
      }
    }
  }
  (void)hx;
  const int y = y0 + ty;
  if (y < c_g.nx[1]) {
    const long i0 = (long)c_g.nx[0] * (y + (long)c_g.nx[1] * z);
#pragma unroll
    for (int o = 0; o < 8; o++) {
      const int x = x0 + 8 * tx + o;
      if (x < c_g.nx[0]) out[i0 + x] += (double)sum[o];
    }
  }
}

void launch_conv_slab(const float *in, long in_total, const int4 *planes, int nplanes, const int4 *lines,
                      const float *lw, double *out, int pitch, int ncols, int max_rows, int max_lines, int max_w,
                      int nx, int ny, int nz, cudaStream_t s)
{
  const size_t smem = sizeof(float) * ((size_t)max_rows * pitch + max_w) + sizeof(int4) * max_lines;
  static size_t configured = 0;
  if (smem > configured) {
    cudaFuncSetAttribute(k_conv_slab, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = smem;
  }
  dim3 grid((nx + kSlabTX - 1) / kSlabTX, (ny + kSlabTY - 1) / kSlabTY, nz);
  k_conv_slab<<<grid, kSlabThreads, smem, s>>>(in, in_total, planes, nplanes, lines, lw, out, pitch, ncols, max_rows,
                                                max_lines, max_w);
}

// ---------------------------------------------------------------------------
// Multi-channel FP32 slab sums (the delta stencil's weighted densities and
// their transposes in the Schur products).  The traversal of k_conv_slab with
// NIN input channels staged per plane and NIN*NOUT coefficients per stencil
// point (stored per coefficient along the lines, wstride apart): output channel
// o of the thread's 8 x-outputs accumulates sum_c coef[o*NIN + c] * in_c over
// the stencil in one FP32 chain, as k_conv does point by point.
template <int NIN, int NOUT>
__global__ void __launch_bounds__(kSlabThreads) k_conv_slab_mc(const float *__restrict__ in, long cstride,
                                                             long in_total, const int4 *__restrict__ planes,
                                                             int nplanes, const int4 *__restrict__ lines,
                                                             const float *__restrict__ lw, int wstride, OutPtrs out,
                                                             int pitch, int ncols, int max_rows, int max_lines,
                                                             int max_w)
{
  constexpr int NC = NIN * NOUT;
  extern __shared__ float smem[];
  float *s_slab = smem;                                        // [NIN][max_rows][pitch]
  float *s_w = s_slab + (size_t)NIN * max_rows * pitch;        // [NC][max_w]
  int4 *s_line = reinterpret_cast<int4 *>(s_w + (size_t)NC * max_w);   // [max_lines]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int x0 = blockIdx.x * kSlabTX, y0 = blockIdx.y * kSlabTY, z = blockIdx.z;
  float acc[NOUT][8];
#pragma unroll
  for (int o = 0; o < NOUT; o++)
#pragma unroll
    for (int q = 0; q < 8; q++) acc[o][q] = 0.f;
  for (int pi = 0; pi < nplanes; pi++) {
    const int4 pd = planes[2 * pi];
    const int4 pg = planes[2 * pi + 1];
    const int nrows = kSlabTY + pg.z - pg.y;
    __syncthreads();
    for (int k = threadIdx.x; k < pd.y; k += kSlabThreads) s_line[k] = lines[pd.x + k];
    for (int k = threadIdx.x; k < NC * pd.w; k += kSlabThreads) {
      const int cc = k / pd.w, kk = k - cc * pd.w;
      s_w[cc * max_w + kk] = lw[(long)cc * wstride + pd.z + kk];
    }
    const long gz = (long)(z + pg.x + c_g.h[2]) * c_g.pstride[2];
    for (int e = threadIdx.x; e < nrows * ncols; e += kSlabThreads) {
      const int r = e / ncols, cidx = e - r * ncols;
      const int gy = y0 + pg.y + r + c_g.h[1];
      const long gi = gz + (long)gy * c_g.pstride[1] + x0 + cidx;
#pragma unroll
      for (int c = 0; c < NIN; c++) {
        float v = 0.f;
        if (gy < c_g.P[1] && gi < in_total - (long)c * cstride) v = __ldg(in + (long)c * cstride + gi);
        s_slab[((size_t)c * max_rows + r) * pitch + slab_phys(cidx)] = v;
      }
    }
    __syncthreads();
    for (int li = 0; li < pd.y; li++) {
      const int4 ln = s_line[li];
      const int c0 = 8 * tx + ln.y;
      const float *w = s_w + (ln.w - pd.z);
      float win[NIN][16];
#pragma unroll
      for (int c = 0; c < NIN; c++) {
        const float *row = s_slab + ((size_t)c * max_rows + ty + ln.x) * pitch;
#pragma unroll
        for (int q = 0; q < 8; q++) win[c][q] = row[slab_phys(c0 + q)];
      }
      for (int kb = 0; kb < ln.z; kb++) {
#pragma unroll
        for (int c = 0; c < NIN; c++) {
          const float *row = s_slab + ((size_t)c * max_rows + ty + ln.x) * pitch;
#pragma unroll
          for (int q = 0; q < 8; q++) win[c][8 + q] = row[slab_phys(c0 + 8 * (kb + 1) + q)];
        }
#pragma unroll
        for (int kk = 0; kk < 8; kk++) {
          float wk[NC];
#pragma unroll
          for (int cc = 0; cc < NC; cc++) wk[cc] = w[cc * max_w + 8 * kb + kk];
#pragma unroll
          for (int o = 0; o < NOUT; o++)
#pragma unroll
            for (int c = 0; c < NIN; c++)
#pragma unroll
              for (int q = 0; q < 8; q++) acc[o][q] = fmaf(wk[o * NIN + c], win[c][q + kk], acc[o][q]);
        }
#pragma unroll
        for (int c = 0; c < NIN; c++)
#pragma unroll
          for (int q = 0; q < 8; q++) win[c][q] = win[c][8 + q];
      }
    }
  }
  const int y = y0 + ty;
  if (y < c_g.nx[1]) {
    const long i0 = (long)c_g.nx[0] * (y + (long)c_g.nx[1] * z);
#pragma unroll
    for (int o = 0; o < NOUT; o++) {
      double *dst = out.p[o];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int x = x0 + 8 * tx + q;
        if (x < c_g.nx[0]) dst[i0 + x] += (double)acc[o][q];
      }
    }
  }
}

size_t conv_slab_mc_smem(int nin, int ncoef, int pitch, int max_rows, int max_lines, int max_w)
{
  return sizeof(float) * ((size_t)nin * max_rows * pitch + (size_t)ncoef * max_w) + sizeof(int4) * max_lines;
}

template <int NIN, int NOUT>
static void slab_mc_dispatch(const float *in, long cstride, long in_total, const int4 *planes, int nplanes,
                             const int4 *lines, const float *lw, int wstride, const OutPtrs &o, int pitch, int ncols,
                             int max_rows, int max_lines, int max_w, int nx, int ny, int nz, cudaStream_t s)
{
  const size_t smem = conv_slab_mc_smem(NIN, NIN * NOUT, pitch, max_rows, max_lines, max_w);
  static size_t configured = 0;
  if (smem > configured) {
    cudaFuncSetAttribute(k_conv_slab_mc<NIN, NOUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = smem;
  }
  dim3 grid((nx + kSlabTX - 1) / kSlabTX, (ny + kSlabTY - 1) / kSlabTY, nz);
  k_conv_slab_mc<NIN, NOUT><<<grid, kSlabThreads, smem, s>>>(in, cstride, in_total, planes, nplanes, lines, lw,
                                                              wstride, o, pitch, ncols, max_rows, max_lines, max_w);
}

bool launch_conv_slab_mc(const float *in, long cstride, long in_total, int nin, const int4 *planes, int nplanes,
                         const int4 *lines, const float *lw, int wstride, double *const *out, int nout, int pitch,
                         int ncols, int max_rows, int max_lines, int max_w, int nx, int ny, int nz, cudaStream_t s)
{
  OutPtrs o{};
  for (int k = 0; k < nout; k++) o.p[k] = out[k];
#define TGPU_SLAB_MC(NI, NO)                                                                                       \
  if (nin == NI && nout == NO) {                                                                                  \
    slab_mc_dispatch<NI, NO>(in, cstride, in_total, planes, nplanes, lines, lw, wstride, o, pitch, ncols, max_rows, \
                             max_lines, max_w, nx, ny, nz, s);                                                   \
    return true;                                                                                                 \
  }
  TGPU_SLAB_MC(1, 4) TGPU_SLAB_MC(4, 1)
#undef TGPU_SLAB_MC
  return false;
}

// ---------------------------------------------------------------------------
// FP64-accurate single-channel 3-D stencil sums in float-float arithmetic.
//
// The same slab / x-line traversal as k_conv_slab, on the padded field split
// into FP32 high and low parts (f = f_hi + f_lo, exact to ~2^-48 relative, by
// k_split_hilo) and weights split likewise.  Each term w f is formed as
// p = fl(w_hi f_hi) plus its exact rounding error e = fma(w_hi, f_hi, -p) and
// the cross terms w_hi f_lo + w_lo f_hi; p is added to the running sum s by an
// error-free two-sum and the errors go to a compensation c, so s + c carries
// about 48 bits (Ogita-Rump-Oishi compensated summation) over one x-line.  The
// compensation is reset per line (a few dozen terms: its own rounding stays
// at ~1e-14 of the line); groups of kFFGroup line sums are added in
// double-word arithmetic (the accurate double-word addition of Joldes, Muller
// and Popescu, relative error <= 3 u^2 per addition) and each group goes into
// an FP64 total.  Twelve FP32 operations per term against one FP64 FMA: on
// GB300, whose FP64 pipe runs at 1/64 of the FP32 rate, that is ~5x fewer issue
// slots, and the grouping keeps the FP64 pipe to one addition per kFFGroup
// lines.  Intrinsics (__fmul_rn, __fadd_rn) keep the compiler from fusing
// products into sums.
constexpr int kFFGroup = 8;

// One term: the product's rounding error and cross terms are gathered off the loop-carried chains, so
// s and c each take one addition per term.
__device__ __forceinline__ void ff_term(float wh, float wl, float fh, float fl, float &s, float &c)
{
  const float p = __fmul_rn(wh, fh);
  float e = __fmaf_rn(wh, fh, -p);
  e = __fmaf_rn(wh, fl, e);
  e = __fmaf_rn(wl, fh, e);
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float e2 = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  s = t;
  c = __fadd_rn(c, __fadd_rn(e, e2));
}

// (a, b) <- (a, b) + (c, d) in double-word arithmetic (accurate version: two two-sums, two fast two-sums)
__device__ __forceinline__ void dw_add(float &a, float &b, float c, float d)
{
  const float sh = __fadd_rn(a, c);
  const float z1 = __fsub_rn(sh, a);
  const float sl = __fadd_rn(__fsub_rn(a, __fsub_rn(sh, z1)), __fsub_rn(c, z1));
  const float th = __fadd_rn(b, d);
  const float z2 = __fsub_rn(th, b);
  const float tl = __fadd_rn(__fsub_rn(b, __fsub_rn(th, z2)), __fsub_rn(d, z2));
  const float cc = __fadd_rn(sl, th);
  const float vh = __fadd_rn(sh, cc);
  const float vl = __fsub_rn(cc, __fsub_rn(vh, sh));
  const float w = __fadd_rn(tl, vl);
  a = __fadd_rn(vh, w);
  b = __fsub_rn(w, __fsub_rn(a, vh));
}

__global__ void k_split_hilo(const double *__restrict__ in, long n, float *__restrict__ hi, float *__restrict__ lo)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = in[i];
    const float h = __double2float_rn(v);
    hi[i] = h;
    lo[i] = __double2float_rn(v - (double)h);
  }
}

__global__ void __launch_bounds__(kSlabThreads) k_conv_slab_ff(const float *__restrict__ in_hi,
                                                             const float *__restrict__ in_lo, long in_total,
                                                             const int4 *__restrict__ planes, int nplanes,
                                                             const int4 *__restrict__ lines,
                                                             const float *__restrict__ lw,
                                                             const float *__restrict__ lw_lo,
                                                             double *__restrict__ out, int pitch, int ncols,
                                                             int max_rows, int max_lines, int max_w)
{
  extern __shared__ float smem[];
  float *s_hi = smem;                                          // [max_rows][pitch]
  float *s_lo = s_hi + (size_t)max_rows * pitch;               // [max_rows][pitch]
  float *s_w = s_lo + (size_t)max_rows * pitch;                // [max_w]
  float *s_wl = s_w + max_w;                                   // [max_w]
  int4 *s_line = reinterpret_cast<int4 *>(s_wl + max_w);      // [max_lines]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int x0 = blockIdx.x * kSlabTX, y0 = blockIdx.y * kSlabTY, z = blockIdx.z;
  double total[8];
  float gh[8], gl[8];   // the current group of line sums, double-word
#pragma unroll
  for (int o = 0; o < 8; o++) { total[o] = 0.0; gh[o] = 0.f; gl[o] = 0.f; }
  int ng = 0;
  for (int pi = 0; pi < nplanes; pi++) {
    const int4 pd = planes[2 * pi];
    const int4 pg = planes[2 * pi + 1];
    const int nrows = kSlabTY + pg.z - pg.y;
    __syncthreads();
    for (int k = threadIdx.x; k < pd.y; k += kSlabThreads) s_line[k] = lines[pd.x + k];
    for (int k = threadIdx.x; k < pd.w; k += kSlabThreads) {
      s_w[k] = lw[pd.z + k];
      s_wl[k] = lw_lo[pd.z + k];
    }
    const long gz = (long)(z + pg.x + c_g.h[2]) * c_g.pstride[2];
    for (int e = threadIdx.x; e < nrows * ncols; e += kSlabThreads) {
      const int r = e / ncols, cidx = e - r * ncols;
      const int gy = y0 + pg.y + r + c_g.h[1];
      const long gi = gz + (long)gy * c_g.pstride[1] + x0 + cidx;
      float vh = 0.f, vl = 0.f;
      if (gy < c_g.P[1] && gi < in_total) {
        vh = __ldg(in_hi + gi);
        vl = __ldg(in_lo + gi);
      }
      s_hi[r * pitch + slab_phys(cidx)] = vh;
      s_lo[r * pitch + slab_phys(cidx)] = vl;
    }
    __syncthreads();
    for (int li = 0; li < pd.y; li++) {
      const int4 ln = s_line[li];
      const float *rh = s_hi + (ty + ln.x) * pitch;
      const float *rl = s_lo + (ty + ln.x) * pitch;
      const float *w = s_w + (ln.w - pd.z);
      const float *wlo = s_wl + (ln.w - pd.z);
      const int c0 = 8 * tx + ln.y;
      float sum[8], comp[8];
#pragma unroll
      for (int o = 0; o < 8; o++) { sum[o] = 0.f; comp[o] = 0.f; }
      float wh_[16], wl_[16];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        wh_[q] = rh[slab_phys(c0 + q)];
        wl_[q] = rl[slab_phys(c0 + q)];
      }
      for (int kb = 0; kb < ln.z; kb++) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
          wh_[8 + q] = rh[slab_phys(c0 + 8 * (kb + 1) + q)];
          wl_[8 + q] = rl[slab_phys(c0 + 8 * (kb + 1) + q)];
        }
#pragma unroll
        for (int kk = 0; kk < 8; kk++) {
          const float a = w[8 * kb + kk], al = wlo[8 * kb + kk];
#pragma unroll
          for (int o = 0; o < 8; o++) ff_term(a, al, wh_[o + kk], wl_[o + kk], sum[o], comp[o]);
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
          wh_[q] = wh_[8 + q];
          wl_[q] = wl_[8 + q];
        }
      }
#pragma unroll
      for (int o = 0; o < 8; o++) dw_add(gh[o], gl[o], sum[o], comp[o]);
      if (++ng == kFFGroup) {
#pragma unroll
        for (int o = 0; o < 8; o++) {
          total[o] += (double)gh[o] + (double)gl[o];
          gh[o] = 0.f;
          gl[o] = 0.f;
        }
        ng = 0;
      }
    }
  }
  const int y = y0 + ty;
  if (y < c_g.nx[1]) {
    const long i0 = (long)c_g.nx[0] * (y + (long)c_g.nx[1] * z);
#pragma unroll
    for (int o = 0; o < 8; o++) {
      const int x = x0 + 8 * tx + o;
      if (x < c_g.nx[0]) out[i0 + x] += total[o] + ((double)gh[o] + (double)gl[o]);
    }
  }
}

size_t conv_slab_ff_smem(int pitch, int max_rows, int max_lines, int max_w)
{
  return sizeof(float) * (2 * (size_t)max_rows * pitch + 2 * (size_t)max_w) + sizeof(int4) * max_lines;
}

void launch_split_hilo(const double *in, long n, float *hi, float *lo, cudaStream_t s)
{
  k_split_hilo<<<1184, kThreads, 0, s>>>(in, n, hi, lo);
}

void launch_conv_slab_ff(const float *in_hi, const float *in_lo, long in_total, const int4 *planes, int nplanes,
                         const int4 *lines, const float *lw, const float *lw_lo, double *out, int pitch, int ncols,
                         int max_rows, int max_lines, int max_w, int nx, int ny, int nz, cudaStream_t s)
{
  const size_t smem = conv_slab_ff_smem(pitch, max_rows, max_lines, max_w);
  static size_t configured = 0;
  if (smem > configured) {
    cudaFuncSetAttribute(k_conv_slab_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    configured = smem;
  }
  dim3 grid((nx + kSlabTX - 1) / kSlabTX, (ny + kSlabTY - 1) / kSlabTY, nz);
  k_conv_slab_ff<<<grid, kSlabThreads, smem, s>>>(in_hi, in_lo, in_total, planes, nplanes, lines, lw, lw_lo, out,
                                                   pitch, ncols, max_rows, max_lines, max_w);
}

// ---------------------------------------------------------------------------
// FMT physics at one node.  n is in the reference's n ordering
// (n0, n1, n2, n3, V1[d], V2[d]); sv is the solution-vector ordering
// (n3, n2, n1, n0, V2[d], V1[d]) (solutionVec_to_nOrdering, src/dft_utils.c:205-221).
__device__ __forceinline__ void load_n(const double *__restrict__ x, long i, double *n)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  const double *rb = x + (long)c_g.first_rb * N;
  n[0] = rb[3 * N + i];
  n[1] = rb[2 * N + i];
  n[2] = rb[1 * N + i];
  n[3] = rb[i];
  for (int d = 0; d < nd; d++) {
    n[4 + d] = rb[(4 + nd + d) * N + i];
    n[4 + nd + d] = rb[(4 + d) * N + i];
  }
}

__device__ __forceinline__ void fmt_dphi(const double *n, double *dphi)
{
  fmt_dphi_at(n, dphi, c_g.ndim, c_g.functional);
}

__device__ __forceinline__ void fmt_hess_apply(const double *n, const double *y, double *z, bool transpose = false)
{
  fmt_hess_apply_at(n, y, z, c_g.ndim, c_g.functional, c_g.jac_exact != 0, transpose);
}

// H y at node i from the state x, with the node's Hessian scalars from coef ([kHessCoef][N], the state's, see
// k_hess_coef) when given: the products of one Newton state then skip the FP64 evaluation of f(n3), g(n2, V2)
__device__ __forceinline__ void hess_apply_node(const double *x, const double *coef, long i, const double *y,
                                                double *z)
{
  double n[kMaxRb];
  load_n(x, i, n);
  if (!coef) {
    fmt_hess_apply(n, y, z);
    return;
  }
  const long N = c_g.N;
  HessCoef c;
  c.a = coef[i];
  c.a2 = coef[N + i];
  c.h13 = coef[2 * N + i];
  c.h22 = coef[3 * N + i];
  c.h23 = coef[4 * N + i];
  c.h33 = coef[5 * N + i];
  c.ff = coef[6 * N + i];
  c.gvf1 = coef[7 * N + i];
  c.g2vr_f = coef[8 * N + i];
  c.g2vc_f = coef[9 * N + i];
  c.gvv = coef[10 * N + i];
  c.gvv_out = coef[11 * N + i];
  fmt_hess_apply_coef(c, n, y, z, c_g.ndim, false);
}

// the same in arithmetic T from the state's Hessian scalars (coef must be given)
template <class T>
__device__ __forceinline__ void hess_apply_node_t(const double *x, const double *coef, long i, const T *y, T *z)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  const double *rb = x + (long)c_g.first_rb * N;
  T n[kMaxRb];
  n[0] = to_arith<T>(rb[3 * N + i]);
  n[1] = to_arith<T>(rb[2 * N + i]);
  n[2] = to_arith<T>(rb[1 * N + i]);
  n[3] = to_arith<T>(rb[i]);
  for (int d = 0; d < nd; d++) {
    n[4 + d] = to_arith<T>(rb[(4 + nd + d) * N + i]);
    n[4 + nd + d] = to_arith<T>(rb[(4 + d) * N + i]);
  }
  HessCoefT<T> c;
  c.a = to_arith<T>(coef[i]);
  c.a2 = to_arith<T>(coef[N + i]);
  c.h13 = to_arith<T>(coef[2 * N + i]);
  c.h22 = to_arith<T>(coef[3 * N + i]);
  c.h23 = to_arith<T>(coef[4 * N + i]);
  c.h33 = to_arith<T>(coef[5 * N + i]);
  c.ff = to_arith<T>(coef[6 * N + i]);
  c.gvf1 = to_arith<T>(coef[7 * N + i]);
  c.g2vr_f = to_arith<T>(coef[8 * N + i]);
  c.g2vc_f = to_arith<T>(coef[9 * N + i]);
  c.gvv = to_arith<T>(coef[10 * N + i]);
  c.gvv_out = to_arith<T>(coef[11 * N + i]);
  fmt_hess_apply_coef(c, n, y, z, nd, false);
}

// coef32, when given, receives the FP32 table of k_hess_coef32 in the same pass
__global__ void k_hess_coef(const double *__restrict__ x, double *__restrict__ coef, float *__restrict__ coef32)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    double n[kMaxRb];
    load_n(x, i, n);
    const HessCoef c = fmt_hess_coef_at(n, c_g.ndim, c_g.functional, c_g.jac_exact != 0);
    const double v[kHessCoef] = {c.a, c.a2, c.h13, c.h22, c.h23, c.h33, c.ff, c.gvf1, c.g2vr_f, c.g2vc_f, c.gvv,
                                 c.gvv_out};
    for (int k = 0; k < kHessCoef; k++) coef[(long)k * N + i] = v[k];
    if (coef32) {
      for (int k = 0; k < kHessCoef; k++) coef32[(long)k * N + i] = (float)v[k];
      for (int k = 0; k < c_g.nrb; k++) coef32[(long)(kHessCoef + k) * N + i] = (float)n[k];
    }
  }
}

void launch_hess_coef(const double *x, double *coef, cudaStream_t s, float *coef32)
{
  k_hess_coef<<<1184, kThreads, 0, s>>>(x, coef, coef32);
}

// Transpose-convolution channels from a weighted-density-shaped vector q (n ordering):
// per component A = fac (q0/4piR^2 + q1/4piR + q2), B_d = fac (q_V1d/4piR + q_V2d), C = fac q3
// (formed in the arithmetic of q, stored in FP64)
template <class T>
__device__ __forceinline__ void write_tr_channels(const T *q, double *chan, long i)
{
  const int nd = c_g.ndim;
  const long N = c_g.N;
  for (int ic = 0; ic < c_g.ncomp; ic++) {
    const T f = to_arith<T>(c_g.fac[ic]), i4pr = to_arith<T>(c_g.inv_4pir[ic]), i4pr2 = to_arith<T>(c_g.inv_4pirsq[ic]);
    const long base = (long)ic * (nd + 2);
    chan[base * N + i] = to_f64(f * (q[0] * i4pr2 + q[1] * i4pr + q[2]));
    for (int d = 0; d < nd; d++) chan[(base + 1 + d) * N + i] = to_f64(f * (q[4 + d] * i4pr + q[4 + nd + d]));
    chan[(base + nd + 1) * N + i] = to_f64(f * q[3]);
  }
}

// domain: when non-null, bit kDomainN3 is set where n3 >= 1 (log(1 - n3) and 1/(1 - n3)^k are taken here)
__global__ void k_fmt_local(const double *__restrict__ x, double *__restrict__ chan, unsigned *__restrict__ domain)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < c_g.N; i += (long)gridDim.x * blockDim.x) {
    double n[kMaxRb], dphi[kMaxRb];
    load_n(x, i, n);
    if (domain && n[3] >= 1.0) atomicOr(domain, kDomainN3);
    fmt_dphi(n, dphi);
    write_tr_channels(dphi, chan, i);
  }
}

void launch_fmt_local(const double *x, double *chan, cudaStream_t s, unsigned *domain)
{
  k_fmt_local<<<1184, kThreads, 0, s>>>(x, chan, domain);
}

// The pinned density of a constrained interface: R = ln rho - ln pin_value, J = 1/rho on the diagonal
// only (fill_constant_density, src/dft_fill_EL.c:286-305)
__device__ __forceinline__ bool pin_row(int ic, long i) { return ic == 0 && i == c_g.pin_node; }

__device__ __forceinline__ int row_kind(long i) { return c_g.rowkind ? c_g.rowkind[i] : 0; }

// Euler-Lagrange rows without nonlocal couplings: zero-density rows (R = rho, J = 1), the pinned row and
// the rows of BULK_ZONE / PB_ZONE nodes
__device__ __forceinline__ bool zero_row(const double *vext, const signed char *zero, int ic, long i)
{
  if (pin_row(ic, i)) return true;
  const long k = (long)ic * c_g.N + i;
  return zero[k] || vext[k] == c_g.vext_max || row_kind(i) != 0;
}

// Of those, the rows R = ln rho - ln c with J = 1/rho: the pinned row (c = pin_value), a BULK_ZONE node's
// (c = rho_b: fill_bulk_density, src/dft_fill_EL.c:69-80, 265-284) and a PB_ZONE node's (the ideal gas in
// the external field, chemical potential without the excess terms and no hard-sphere or attraction terms:
// ln c = -mu0 - V_ext, src/dft_fill_EL.c:132-161, 405-410); zero-density rows come first
__device__ __forceinline__ bool log_row(const double *vext, const signed char *zero, int ic, long i)
{
  if (pin_row(ic, i)) return true;
  const long k = (long)ic * c_g.N + i;
  return !(zero[k] || vext[k] == c_g.vext_max) && row_kind(i) != 0;
}

__device__ __forceinline__ double log_row_c(const double *vext, int ic, long i)
{
  const int kind = row_kind(i);   // the bulk and PB rows come before the pinned row (src/dft_fill_EL.c:69-97)
  if (kind == 1) return log(c_g.rho_b[ic]);
  if (kind == 2) {
    const double mu0 = c_g.interface ? -c_g.betamu_if[ic] : -log(c_g.rho_b[ic]);
    return -(mu0 + vext[(long)ic * c_g.N + i]);
  }
  return log(c_g.pin_value);
}

// Euler-Lagrange rows that hold +V_ext: the full rows and the PB_ZONE rows
__device__ __forceinline__ bool vext_row(const double *vext, const signed char *zero, int ic, long i)
{
  if (!zero_row(vext, zero, ic, i)) return true;
  return row_kind(i) == 2 && log_row(vext, zero, ic, i);
}

// dependent weighted densities (one particle size): n1 = n2/4piR, n0 = n2/4piR^2, V1 = V2/4piR
__device__ __forceinline__ bool dep_rb(int k, int *src, double *c)
{
  const int nd = c_g.ndim;
  if (!c_g.single_size) return false;
  if (k == 2) { *src = 1; *c = c_g.inv_4pir[0]; return true; }
  if (k == 3) { *src = 1; *c = c_g.inv_4pirsq[0]; return true; }
  if (k >= 4 + nd) { *src = 4 + (k - 4 - nd); *c = c_g.inv_4pir[0]; return true; }
  return false;
}

// domain: when non-null, bit kDomainRho is set where a live Euler-Lagrange row takes log(rho) of rho <= 0
__global__ void k_assemble(const double *__restrict__ x, const double *__restrict__ vext,
                           const signed char *__restrict__ zero, const double *__restrict__ conv,
                           const double *__restrict__ tr, double *__restrict__ R, unsigned *__restrict__ domain)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const int iu = c_g.first_rho + ic;
      const double xi = x[(long)iu * N + i];
      double r;
      if (zero_row(vext, zero, ic, i)) {
        if (log_row(vext, zero, ic, i)) {
          if (domain && xi <= 0.0) atomicOr(domain, kDomainRho);
          r = log(xi) - log_row_c(vext, ic, i);
        } else {
          r = xi;
        }
      } else {
        double mu;
        if (c_g.interface) {
          mu = -c_g.betamu_if[ic];
        } else {
          mu = -log(c_g.rho_b[ic]) - c_g.betamu_hs_ex[ic];
          if (c_g.attraction) mu -= c_g.betamu_att[ic];
        }
        if (domain && xi <= 0.0) atomicOr(domain, kDomainRho);
        r = log(xi) + mu + vext[(long)ic * N + i] + tr[(long)ic * N + i];
        if (c_g.attraction) r += x[(long)(c_g.first_mf + ic) * N + i];
      }
      R[(long)iu * N + i] = r;
    }
    for (int k = 0; k < c_g.nrb; k++) {
      const int iu = c_g.first_rb + k;
      int src;
      double c;
      double r = -x[(long)iu * N + i];
      if (dep_rb(k, &src, &c)) r += x[(long)(c_g.first_rb + src) * N + i] * c;
      else r += conv[(long)k * N + i];
      R[(long)iu * N + i] = r;
    }
    if (c_g.attraction)
      for (int ic = 0; ic < c_g.ncomp; ic++) {
        const int iu = c_g.first_mf + ic;
        R[(long)iu * N + i] = -x[(long)iu * N + i] + conv[(long)(c_g.nrb + ic) * N + i];
      }
  }
}

void launch_assemble(const double *x, const double *vext, const signed char *zero, const double *conv,
                     const double *tr, double *R, cudaStream_t s, unsigned *domain)
{
  k_assemble<<<1184, kThreads, 0, s>>>(x, vext, zero, conv, tr, R, domain);
}

// Schur local step: y1 = A11^-1 u (u = A12 v in conv), then the EL-side
// channels of H y1 for the transpose sums; y_MF = -u_MF kept for A21.
// T = double, or float for FP32 products (then coef must hold the state's Hessian scalars)
template <class T>
__global__ void k_schur_local(const double *__restrict__ x, const double *__restrict__ conv,
                              double *__restrict__ chan, double *__restrict__ ymf, const double *__restrict__ coef)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    T ysv[kMaxRb], y[kMaxRb], z[kMaxRb];
    for (int k = 0; k < c_g.nrb; k++) {
      int src;
      double c;
      if (dep_rb(k, &src, &c)) ysv[k] = -to_arith<T>(c) * to_arith<T>(conv[(long)src * N + i]);   // -u_dep - B u_ind
      else ysv[k] = -to_arith<T>(conv[(long)k * N + i]);
    }
    y[0] = ysv[3]; y[1] = ysv[2]; y[2] = ysv[1]; y[3] = ysv[0];
    for (int d = 0; d < nd; d++) { y[4 + d] = ysv[4 + nd + d]; y[4 + nd + d] = ysv[4 + d]; }
    if constexpr (sizeof(T) == sizeof(double)) hess_apply_node(x, coef, i, y, z);
    else hess_apply_node_t<T>(x, coef, i, y, z);
    write_tr_channels(z, chan, i);
    if (c_g.attraction)   // the sign flipped on the integer pipe
      for (int ic = 0; ic < c_g.ncomp; ic++)
        ymf[(long)ic * N + i] =
            __longlong_as_double(__double_as_longlong(conv[(long)(c_g.nrb + ic) * N + i]) ^ (long long)0x8000000000000000ull);
  }
}

void launch_schur_local(const double *x, const double *conv, double *chan, double *ymf, const double *coef,
                        cudaStream_t s, bool f32)
{
  if (f32 && coef) k_schur_local<float><<<1184, kThreads, 0, s>>>(x, conv, chan, ymf, coef);
  else k_schur_local<double><<<1184, kThreads, 0, s>>>(x, conv, chan, ymf, coef);
}

// FP32 storage for the FP32 Schur products: the state's Hessian scalars and weighted densities (n order) as FP32
// rows [kHessCoef + nrb][N], made once per state; with the stencil sums, channels and transposed sums also held
// in FP32 the local step converts nothing (conversions between FP64 and FP32 run on GB300's FP64 pipe).
__global__ void k_hess_coef32(const double *__restrict__ x, float *__restrict__ coef)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    double n[kMaxRb];
    load_n(x, i, n);
    const HessCoef c = fmt_hess_coef_at(n, c_g.ndim, c_g.functional, c_g.jac_exact != 0);
    const double v[kHessCoef] = {c.a, c.a2, c.h13, c.h22, c.h23, c.h33, c.ff, c.gvf1, c.g2vr_f, c.g2vc_f, c.gvv,
                                 c.gvv_out};
    for (int k = 0; k < kHessCoef; k++) coef[(long)k * N + i] = (float)v[k];
    for (int k = 0; k < c_g.nrb; k++) coef[(long)(kHessCoef + k) * N + i] = (float)n[k];
  }
}

void launch_hess_coef32(const double *x, float *coef, cudaStream_t s)
{
  k_hess_coef32<<<1184, kThreads, 0, s>>>(x, coef);
}

// k_schur_local with every operand in FP32 storage (conv [nrb + ncomp][N] the stencil sums of A12 v, chan the
// transposed-sum channels, ymf = -u_MF); ND the dimension, so that the per-node arrays stay in registers, and the
// per-component constants converted once per thread
template <int ND>
__global__ void k_schur_local32(const float *__restrict__ conv, const float *__restrict__ coef,
                                float *__restrict__ chan, float *__restrict__ ymf)
{
  constexpr int NRB = 4 + 2 * ND;
  const long N = c_g.N;
  int src_k[NRB];
  float dep_c[NRB];
  bool dep[NRB];
#pragma unroll
  for (int k = 0; k < NRB; k++) {
    double cd = 0.0;
    dep[k] = dep_rb(k, &src_k[k], &cd);
    dep_c[k] = (float)cd;
  }
  const int ncomp = c_g.ncomp;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    float ysv[NRB], y[NRB], z[NRB], n[NRB];
#pragma unroll
    for (int k = 0; k < NRB; k++)
      ysv[k] = dep[k] ? -dep_c[k] * conv[(long)src_k[k] * N + i] : -conv[(long)k * N + i];   // -u_dep - B u_ind
    y[0] = ysv[3]; y[1] = ysv[2]; y[2] = ysv[1]; y[3] = ysv[0];
#pragma unroll
    for (int d = 0; d < ND; d++) { y[4 + d] = ysv[4 + ND + d]; y[4 + ND + d] = ysv[4 + d]; }
#pragma unroll
    for (int k = 0; k < NRB; k++) n[k] = coef[(long)(kHessCoef + k) * N + i];
    HessCoefT<float> hc;
    hc.a = coef[i];
    hc.a2 = coef[N + i];
    hc.h13 = coef[2 * N + i];
    hc.h22 = coef[3 * N + i];
    hc.h23 = coef[4 * N + i];
    hc.h33 = coef[5 * N + i];
    hc.ff = coef[6 * N + i];
    hc.gvf1 = coef[7 * N + i];
    hc.g2vr_f = coef[8 * N + i];
    hc.g2vc_f = coef[9 * N + i];
    hc.gvv = coef[10 * N + i];
    hc.gvv_out = coef[11 * N + i];
    fmt_hess_apply_coef(hc, n, y, z, ND, false);
    for (int ic = 0; ic < ncomp; ic++) {
      const float fc = (float)c_g.fac[ic], i4pr = (float)c_g.inv_4pir[ic], i4pr2 = (float)c_g.inv_4pirsq[ic];
      const long base = (long)ic * (ND + 2);
      chan[base * N + i] = fc * (z[0] * i4pr2 + z[1] * i4pr + z[2]);
#pragma unroll
      for (int d = 0; d < ND; d++) chan[(base + 1 + d) * N + i] = fc * (z[4 + d] * i4pr + z[4 + ND + d]);
      chan[(base + ND + 1) * N + i] = fc * z[3];
    }
    if (c_g.attraction)
      for (int ic = 0; ic < ncomp; ic++) ymf[(long)ic * N + i] = -conv[(long)(NRB + ic) * N + i];
  }
}

void launch_schur_local32(int ndim, const float *conv, const float *coef, float *chan, float *ymf, cudaStream_t s)
{
  if (ndim == 3) k_schur_local32<3><<<1184, kThreads, 0, s>>>(conv, coef, chan, ymf);
  else if (ndim == 2) k_schur_local32<2><<<1184, kThreads, 0, s>>>(conv, coef, chan, ymf);
  else k_schur_local32<1><<<1184, kThreads, 0, s>>>(conv, coef, chan, ymf);
}

// J v local step: channels of H v_rb for the EL rows.
template <class T>
__global__ void k_jv_local(const double *__restrict__ x, const double *__restrict__ v, double *__restrict__ chan,
                           const double *__restrict__ coef)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    T z[kMaxRb];
    if constexpr (sizeof(T) == sizeof(double)) {
      double y[kMaxRb];
      load_n(v, i, y);
      hess_apply_node(x, coef, i, y, z);
    } else {
      double yd[kMaxRb];
      T y[kMaxRb];
      load_n(v, i, yd);
      for (int k = 0; k < c_g.nrb; k++) y[k] = to_arith<T>(yd[k]);
      hess_apply_node_t<T>(x, coef, i, y, z);
    }
    write_tr_channels(z, chan, i);
  }
}

void launch_jv_local(const double *x, const double *v, double *chan, const double *coef, cudaStream_t s, bool f32)
{
  if (f32 && coef) k_jv_local<float><<<1184, kThreads, 0, s>>>(x, v, chan, coef);
  else k_jv_local<double><<<1184, kThreads, 0, s>>>(x, v, chan, coef);
}

__global__ void k_schur_combine(const double *__restrict__ x, const double *__restrict__ vext,
                                const signed char *__restrict__ zero, const double *__restrict__ v2,
                                const double *__restrict__ tr, const double *__restrict__ ymf, double *__restrict__ y2)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long k = (long)ic * N + i;
      if (zero_row(vext, zero, ic, i)) {
        y2[k] = log_row(vext, zero, ic, i) ? v2[k] / x[(long)(c_g.first_rho + ic) * N + i] : v2[k];
      } else {
        double a21y = tr[k];
        if (c_g.attraction) a21y += ymf[k];
        y2[k] = v2[k] / x[(long)(c_g.first_rho + ic) * N + i] - a21y;
      }
    }
}

void launch_schur_combine(const double *x, const double *vext, const signed char *zero, const double *v2,
                          const double *tr, const double *ymf, double *y2, cudaStream_t s)
{
  k_schur_combine<<<1184, kThreads, 0, s>>>(x, vext, zero, v2, tr, ymf, y2);
}

// The Euler-Lagrange rows of a state for the FP32 products: kind 0 a full row, 1 a row ln rho - ln c (pinned,
// BULK_ZONE, PB_ZONE), 2 a zero-density row; inv = 1/rho (0 on zero-density rows), in FP64: the local part v2 / rho
// dominates the product near walls, where rho is small
__global__ void k_row_info32(const double *__restrict__ x, const double *__restrict__ vext,
                             const signed char *__restrict__ zero, double *__restrict__ inv,
                             signed char *__restrict__ kind)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long k = (long)ic * N + i;
      const bool zr = zero_row(vext, zero, ic, i), lr = zr && log_row(vext, zero, ic, i);
      kind[k] = !zr ? 0 : lr ? 1 : 2;
      inv[k] = (!zr || lr) ? 1.0 / x[(long)(c_g.first_rho + ic) * N + i] : 0.0;
    }
}

void launch_row_info32(const double *x, const double *vext, const signed char *zero, double *inv, signed char *kind,
                       cudaStream_t s)
{
  k_row_info32<<<1184, kThreads, 0, s>>>(x, vext, zero, inv, kind);
}

// k_schur_combine with the transposed sums and -u_MF in FP32 storage and the rows of k_row_info32 (no FP64 division
// or comparison per product)
__global__ void k_schur_combine32(const double *__restrict__ inv, const signed char *__restrict__ kind,
                                  const double *__restrict__ v2, const float *__restrict__ tr,
                                  const float *__restrict__ ymf, double *__restrict__ y2)
{
  const long n = (long)c_g.ncomp * c_g.N;
  const bool att = c_g.attraction != 0;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
    const int kd = kind[k];
    if (kd == 2) {
      y2[k] = v2[k];
    } else {
      const double t = v2[k] * inv[k];
      y2[k] = kd == 0 ? t - (double)(att ? tr[k] + ymf[k] : tr[k]) : t;
    }
  }
}

void launch_schur_combine32(const double *inv, const signed char *kind, const double *v2, const float *tr,
                            const float *ymf, double *y2, cudaStream_t s)
{
  k_schur_combine32<<<1184, kThreads, 0, s>>>(inv, kind, v2, tr, ymf, y2);
}

__global__ void k_jv_combine(const double *__restrict__ x, const double *__restrict__ vext,
                             const signed char *__restrict__ zero, const double *__restrict__ v,
                             const double *__restrict__ conv, const double *__restrict__ tr, double *__restrict__ out)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const int iu = c_g.first_rho + ic;
      const long k = (long)iu * N + i;
      if (zero_row(vext, zero, ic, i)) {
        out[k] = log_row(vext, zero, ic, i) ? v[k] / x[k] : v[k];
      } else {
        double r = v[k] / x[k] + tr[(long)ic * N + i];
        if (c_g.attraction) r += v[(long)(c_g.first_mf + ic) * N + i];
        out[k] = r;
      }
    }
    for (int kk = 0; kk < c_g.nrb; kk++) {
      const int iu = c_g.first_rb + kk;
      int src;
      double c;
      double r = -v[(long)iu * N + i];
      if (dep_rb(kk, &src, &c)) r += v[(long)(c_g.first_rb + src) * N + i] * c;
      else r += conv[(long)kk * N + i];
      out[(long)iu * N + i] = r;
    }
    if (c_g.attraction)
      for (int ic = 0; ic < c_g.ncomp; ic++) {
        const int iu = c_g.first_mf + ic;
        out[(long)iu * N + i] = -v[(long)iu * N + i] + conv[(long)(c_g.nrb + ic) * N + i];
      }
  }
}

void launch_jv_combine(const double *x, const double *vext, const signed char *zero, const double *v,
                       const double *conv, const double *tr, double *out, cudaStream_t s)
{
  k_jv_combine<<<1184, kThreads, 0, s>>>(x, vext, zero, v, conv, tr, out);
}

// Schur right-hand side: y1 = A11^-1 b1 from the block-1 part of a full
// vector b, then the channels of H y1 (ComputeRHS, src/dft_Schur_Epetra_Operator.cpp:121-133).
__global__ void k_rhs_local(const double *__restrict__ x, const double *__restrict__ b, double *__restrict__ chan,
                            double *__restrict__ ymf, const double *__restrict__ coef)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    double ysv[kMaxRb], y[kMaxRb], n[kMaxRb], z[kMaxRb];
    const double *brb = b + (long)c_g.first_rb * N;
    for (int k = 0; k < c_g.nrb; k++) {
      int src;
      double c;
      if (dep_rb(k, &src, &c)) ysv[k] = -brb[(long)k * N + i] - c * brb[(long)src * N + i];
      else ysv[k] = -brb[(long)k * N + i];
    }
    y[0] = ysv[3]; y[1] = ysv[2]; y[2] = ysv[1]; y[3] = ysv[0];
    for (int d = 0; d < nd; d++) { y[4 + d] = ysv[4 + nd + d]; y[4 + nd + d] = ysv[4 + d]; }
    (void)n;
    hess_apply_node(x, coef, i, y, z);
    write_tr_channels(z, chan, i);
    if (c_g.attraction)
      for (int ic = 0; ic < c_g.ncomp; ic++) ymf[(long)ic * N + i] = -b[(long)(c_g.first_mf + ic) * N + i];
  }
}

void launch_rhs_local(const double *x, const double *b, double *chan, double *ymf, const double *coef, cudaStream_t s)
{
  k_rhs_local<<<1184, kThreads, 0, s>>>(x, b, chan, ymf, coef);
}

// k_rhs_local in FP32 storage (the FP32 products' right-hand side b2 - A21 A11^-1 b1: FP32 arithmetic on the FP32
// table of the state, FP32 channels for the FP32 transposed sums; ymf = -b_MF)
template <int ND>
__global__ void k_rhs_local32(const double *__restrict__ b, const float *__restrict__ coef, float *__restrict__ chan,
                              float *__restrict__ ymf)
{
  constexpr int NRB = 4 + 2 * ND;
  const long N = c_g.N;
  int src_k[NRB];
  float dep_c[NRB];
  bool dep[NRB];
#pragma unroll
  for (int k = 0; k < NRB; k++) {
    double cd = 0.0;
    dep[k] = dep_rb(k, &src_k[k], &cd);
    dep_c[k] = (float)cd;
  }
  const int ncomp = c_g.ncomp;
  const double *brb = b + (long)c_g.first_rb * N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    float ysv[NRB], y[NRB], z[NRB], n[NRB];
#pragma unroll
    for (int k = 0; k < NRB; k++) {
      const float bk = (float)brb[(long)k * N + i];
      ysv[k] = dep[k] ? -bk - dep_c[k] * (float)brb[(long)src_k[k] * N + i] : -bk;
    }
    y[0] = ysv[3]; y[1] = ysv[2]; y[2] = ysv[1]; y[3] = ysv[0];
#pragma unroll
    for (int d = 0; d < ND; d++) { y[4 + d] = ysv[4 + ND + d]; y[4 + ND + d] = ysv[4 + d]; }
#pragma unroll
    for (int k = 0; k < NRB; k++) n[k] = coef[(long)(kHessCoef + k) * N + i];
    HessCoefT<float> hc;
    hc.a = coef[i];
    hc.a2 = coef[N + i];
    hc.h13 = coef[2 * N + i];
    hc.h22 = coef[3 * N + i];
    hc.h23 = coef[4 * N + i];
    hc.h33 = coef[5 * N + i];
    hc.ff = coef[6 * N + i];
    hc.gvf1 = coef[7 * N + i];
    hc.g2vr_f = coef[8 * N + i];
    hc.g2vc_f = coef[9 * N + i];
    hc.gvv = coef[10 * N + i];
    hc.gvv_out = coef[11 * N + i];
    fmt_hess_apply_coef(hc, n, y, z, ND, false);
    for (int ic = 0; ic < ncomp; ic++) {
      const float fc = (float)c_g.fac[ic], i4pr = (float)c_g.inv_4pir[ic], i4pr2 = (float)c_g.inv_4pirsq[ic];
      const long base = (long)ic * (ND + 2);
      chan[base * N + i] = fc * (z[0] * i4pr2 + z[1] * i4pr + z[2]);
#pragma unroll
      for (int d = 0; d < ND; d++) chan[(base + 1 + d) * N + i] = fc * (z[4 + d] * i4pr + z[4 + ND + d]);
      chan[(base + ND + 1) * N + i] = fc * z[3];
    }
    if (c_g.attraction)
      for (int ic = 0; ic < ncomp; ic++) ymf[(long)ic * N + i] = -(float)b[(long)(c_g.first_mf + ic) * N + i];
  }
}

void launch_rhs_local32(int ndim, const double *b, const float *coef, float *chan, float *ymf, cudaStream_t s)
{
  if (ndim == 3) k_rhs_local32<3><<<1184, kThreads, 0, s>>>(b, coef, chan, ymf);
  else if (ndim == 2) k_rhs_local32<2><<<1184, kThreads, 0, s>>>(b, coef, chan, ymf);
  else k_rhs_local32<1><<<1184, kThreads, 0, s>>>(b, coef, chan, ymf);
}

// b2s = b2 - A21 y1 on full Euler-Lagrange rows (the rows' kinds from k_row_info32), b2 elsewhere
__global__ void k_rhs_combine32(const signed char *__restrict__ kind, const double *__restrict__ b,
                                const float *__restrict__ tr, const float *__restrict__ ymf, double *__restrict__ b2s)
{
  const long n = (long)c_g.ncomp * c_g.N;
  const bool att = c_g.attraction != 0;
  const double *b2 = b + (long)c_g.first_rho * c_g.N;
  for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
    b2s[k] = kind[k] == 0 ? b2[k] - (double)(att ? tr[k] + ymf[k] : tr[k]) : b2[k];
}

void launch_rhs_combine32(const signed char *kind, const double *b, const float *tr, const float *ymf, double *b2s,
                          cudaStream_t s)
{
  k_rhs_combine32<<<1184, kThreads, 0, s>>>(kind, b, tr, ymf, b2s);
}

__global__ void k_rhs_combine(const double *__restrict__ vext, const signed char *__restrict__ zero,
                              const double *__restrict__ b, const double *__restrict__ tr,
                              const double *__restrict__ ymf, double *__restrict__ b2s)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long k = (long)ic * N + i;
      const double bi = b[(long)(c_g.first_rho + ic) * N + i];
      if (zero_row(vext, zero, ic, i)) {
        b2s[k] = bi;
      } else {
        double a21y = tr[k];
        if (c_g.attraction) a21y += ymf[k];
        b2s[k] = bi - a21y;
      }
    }
}

void launch_rhs_combine(const double *vext, const signed char *zero, const double *b, const double *tr,
                        const double *ymf, double *b2s, cudaStream_t s)
{
  k_rhs_combine<<<1184, kThreads, 0, s>>>(vext, zero, b, tr, ymf, b2s);
}

// Back substitution x1 = A11^-1 (b1 - A12 x2) (ComputeX1, src/dft_Schur_Epetra_Operator.cpp:135-147);
// writes the full Newton step dx = [x1; x2].
__global__ void k_x1(const double *__restrict__ b, const double *__restrict__ conv, const double *__restrict__ x2,
                     double *__restrict__ dx)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    double y[kMaxRb];
    const double *brb = b + (long)c_g.first_rb * N;
    for (int k = 0; k < c_g.nrb; k++) {
      int src;
      double c;
      y[k] = dep_rb(k, &src, &c) ? brb[(long)k * N + i] : brb[(long)k * N + i] - conv[(long)k * N + i];
    }
    for (int k = 0; k < c_g.nrb; k++) {
      int src;
      double c;
      double v = dep_rb(k, &src, &c) ? (-y[k] - c * y[src]) : -y[k];
      dx[(long)(c_g.first_rb + k) * N + i] = v;
    }
    for (int ic = 0; ic < c_g.ncomp; ic++) dx[(long)(c_g.first_rho + ic) * N + i] = x2[(long)ic * N + i];
    if (c_g.attraction)
      for (int ic = 0; ic < c_g.ncomp; ic++) {
        const long k = (long)(c_g.first_mf + ic) * N + i;
        dx[k] = -(b[k] - conv[(long)(c_g.nrb + ic) * N + i]);
      }
  }
}

void launch_x1(const double *b, const double *conv, const double *x2, double *dx, cudaStream_t s)
{
  k_x1<<<1184, kThreads, 0, s>>>(b, conv, x2, dx);
}

// ---------------------------------------------------------------------------
// Adjoint (J^T w) local step.  The Jacobian rows of the fill are
//   EL_i(j):  1/rho (diag; 1 on zero rows), + MF_i(j), + sum_o fac w(o) [c(o)^T H(n(j+o))] on rb(j+o)
//   rb_k(j):  -1 (diag), + B (dependent copies), + fac_k w(o) on rho_jc(j+o)
//   MF_i(j):  -1 (diag), + w_att(o) on rho_jc(j+o)
// so for the transpose the rb columns receive H(n(j)) g(j) with g gathered from
// the EL rows by the transposed delta/theta sums (gel: per component the delta
// outputs then the theta output, already scaled by fac), plus -w_rb and the B^T couplings; the MF columns receive -w_MF + w_EL;
// the density columns receive the A22 diagonal times w_EL (the transposed
// weighted-density and mean-field sums are added by the caller).
__global__ void k_jtv_local(const double *__restrict__ x, const double *__restrict__ vext,
                            const signed char *__restrict__ zero, const double *__restrict__ w,
                            const double *__restrict__ gel, int gstride_ic, int v2_first,
                            double *__restrict__ out)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    double g[kMaxRb], n[kMaxRb], z[kMaxRb];
    for (int k = 0; k < 4 + 2 * nd; k++) g[k] = 0.0;
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const double *G = gel + (long)ic * gstride_ic * N;
      const double g0 = G[i];
      g[2] += g0;
      g[1] += c_g.inv_4pir[ic] * g0;
      g[0] += c_g.inv_4pirsq[ic] * g0;
      g[3] += G[(long)(gstride_ic - 1) * N + i];   // theta sum: last in the component's block
      for (int d = 0; d < nd; d++) {
        const double gd = G[(long)(v2_first + d) * N + i];
        g[4 + nd + d] -= gd;
        g[4 + d] -= c_g.inv_4pir[ic] * gd;
      }
    }
    load_n(x, i, n);
    fmt_hess_apply(n, g, z, true);
    // rb columns in solution-vector order: -w_rb + B^T w_dep + z
    double wrb[kMaxRb];
    for (int k = 0; k < c_g.nrb; k++) wrb[k] = w[(long)(c_g.first_rb + k) * N + i];
    double o[kMaxRb];
    o[0] = -wrb[0] + z[3];
    o[1] = -wrb[1] + z[2];
    o[2] = -wrb[2] + z[1];
    o[3] = -wrb[3] + z[0];
    for (int d = 0; d < nd; d++) {
      o[4 + d] = -wrb[4 + d] + z[4 + nd + d];
      o[4 + nd + d] = -wrb[4 + nd + d] + z[4 + d];
    }
    if (c_g.single_size) {
      o[1] += c_g.inv_4pir[0] * wrb[2] + c_g.inv_4pirsq[0] * wrb[3];
      for (int d = 0; d < nd; d++) o[4 + d] += c_g.inv_4pir[0] * wrb[4 + nd + d];
    }
    for (int k = 0; k < c_g.nrb; k++) out[(long)(c_g.first_rb + k) * N + i] = o[k];
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long kr = (long)(c_g.first_rho + ic) * N + i;
      const bool zr = zero_row(vext, zero, ic, i);
      const double wel = zr ? 0.0 : w[kr];
      // density column: transposed sums already in out; add the A22 diagonal
      out[kr] += (zr && !log_row(vext, zero, ic, i)) ? w[kr] : w[kr] / x[kr];
      if (c_g.attraction) {
        const long km = (long)(c_g.first_mf + ic) * N + i;
        out[km] = -w[km] + wel;
      }
    }
  }
}

void launch_jtv_local(const double *x, const double *vext, const signed char *zero, const double *w,
                      const double *gel, int gstride_ic, int v2_first, double *out, cudaStream_t s)
{
  k_jtv_local<<<1184, kThreads, 0, s>>>(x, vext, zero, w, gel, gstride_ic, v2_first, out);
}

// Adjoint channels from the rb and MF rows of w, per component jc ([jc][ndim+2][N]):
// A = w_n2 + w_n1/4piR + w_n0/4piR^2, B_d = w_V2d + w_V1d/4piR, C = w_n3 (the rb rows'
// dependence on rho_jc, without fac); then the ncomp MF rows.  With one particle
// size the n1, n0, V1 rows do not depend on the densities and drop out.
__global__ void k_adj_rb_channels(const double *__restrict__ w, double *__restrict__ chan)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  const int cpc = nd + 2;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    const double *W = w + (long)c_g.first_rb * N + i;
    const double wn3 = W[0], wn2 = W[N];
    const double wn1 = c_g.single_size ? 0.0 : W[2 * N], wn0 = c_g.single_size ? 0.0 : W[3 * N];
    for (int jc = 0; jc < c_g.ncomp; jc++) {
      double *ch = chan + (long)jc * cpc * N + i;
      ch[0] = wn2 + c_g.inv_4pir[jc] * wn1 + c_g.inv_4pirsq[jc] * wn0;
      for (int d = 0; d < nd; d++) {
        const double wv1 = c_g.single_size ? 0.0 : W[(long)(4 + nd + d) * N];
        ch[(long)(1 + d) * N] = W[(long)(4 + d) * N] + c_g.inv_4pir[jc] * wv1;
      }
      ch[(long)(nd + 1) * N] = wn3;
    }
    if (c_g.attraction)
      for (int ic = 0; ic < c_g.ncomp; ic++)
        chan[(long)(c_g.ncomp * cpc + ic) * N + i] = w[(long)(c_g.first_mf + ic) * N + i];
  }
}

void launch_adj_rb_channels(const double *w, double *chan, cudaStream_t s)
{
  k_adj_rb_channels<<<1184, kThreads, 0, s>>>(w, chan);
}

// y = A11^-T u on the block-1 rows of full vectors (density rows set to zero):
// y_dep = -u_dep, y_ind = -u_ind - B^T u_dep, y_MF = -u_MF
__global__ void k_a11inv_t(const double *__restrict__ u, double *__restrict__ y)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    double v[kMaxRb];
    for (int k = 0; k < c_g.nrb; k++) v[k] = -u[(long)(c_g.first_rb + k) * N + i];
    if (c_g.single_size) {
      v[1] -= c_g.inv_4pir[0] * u[(long)(c_g.first_rb + 2) * N + i] + c_g.inv_4pirsq[0] * u[(long)(c_g.first_rb + 3) * N + i];
      for (int d = 0; d < nd; d++) v[4 + d] -= c_g.inv_4pir[0] * u[(long)(c_g.first_rb + 4 + nd + d) * N + i];
    }
    for (int k = 0; k < c_g.nrb; k++) y[(long)(c_g.first_rb + k) * N + i] = v[k];
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      y[(long)(c_g.first_rho + ic) * N + i] = 0.0;
      if (c_g.attraction) y[(long)(c_g.first_mf + ic) * N + i] = -u[(long)(c_g.first_mf + ic) * N + i];
    }
  }
}

void launch_a11inv_t(const double *u, double *y, cudaStream_t s)
{
  k_a11inv_t<<<1184, kThreads, 0, s>>>(u, y);
}

// mode 0: out[r][i] = w[first + r][i] on non-zero EL rows, 0 on zero rows (masking of the EL block of w)
// mode 1: out[r][i] *= !zero_density[r][i] (density columns exist only off zero-density nodes)
__global__ void k_mask_rows(double *__restrict__ out, const double *__restrict__ w, const double *__restrict__ vext,
                            const signed char *__restrict__ zero, int first, int nrows, int mode)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int r = 0; r < nrows; r++) {
      const long k = (long)r * N + i;
      if (mode == 0) out[k] = zero_row(vext, zero, r, i) ? 0.0 : w[(long)(first + r) * N + i];
      else if (zero[k]) out[k] = 0.0;
    }
}

void launch_mask_rows(double *out, const double *w, const double *vext, const signed char *zero, int first, int nrows,
                      int mode, cudaStream_t s)
{
  k_mask_rows<<<1184, kThreads, 0, s>>>(out, w, vext, zero, first, nrows, mode);
}

// ---------------------------------------------------------------------------
// Hard-wall boundary weights: for target nodes whose stencils reach a
// boundary node, replace w by the fluid-element part of the point's corner
// weights (HW_boundary_weight) for the weighted-density and mean-field sums.
__device__ long map_offset(const int *ijk, const short *off, int *refl)
{
  int idx[3] = {0, 0, 0};
  *refl = 0;
  for (int d = 0; d < c_g.ndim; d++) {
    const int q = ijk[d] + c_g.h[d] + off[d];
    const int m = c_g.map[d][q];
    if (m < 0) return m;
    if (m & kReflBit) *refl |= 1 << d;
    idx[d] = m & ~kReflBit;
  }
  return idx[0] + (long)c_g.nx[0] * (idx[1] + (long)c_g.nx[1] * idx[2]);
}

struct HwStencil {
  int L;
  const short *off;
  const double *w, *hw;
};

// The hard-wall stencils: theta and delta per component, the mean-field stencils per (output component,
// input component) pair (ua[ic + kMaxC jc])
struct HwSet {
  HwStencil th[kMaxC], de[kMaxC], ua[kMaxC * kMaxC];
};

// kind 0: theta -> n3; 1: delta -> n2 [n1 n0] V2 [V1]; 2: mean field -> row orow (no prefactor)
__device__ void hw_apply(const HwStencil &st, int kind, int orow, int jc, int jlist, const int *ijk,
                         const double *field, long fcs, int ffirst, const signed char *zero, const int *bnodes,
                         const short *fmask, double *acc)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  const int nel = 1 << nd;
  for (int s = 0; s < st.L; s++) {
    int refl;
    const short *o = st.off + (long)s * 3;
    const long jn = map_offset(ijk, o, &refl);
    if (jn < 0) continue;
    if (bnodes[(long)jlist * N + jn] == -1) continue;
    if (zero[(long)jc * N + jn]) continue;
    const int mask = fmask[((long)jlist * nel + refl) * N + jn];
    double w = 0.0;
    for (int l = 0; l < nel; l++)
      if (mask & (1 << l)) w += st.hw[(long)s * nel + l];
    const double dw = w - st.w[s];
    const double rho = field[(long)(ffirst + jc) * fcs + jn];
    const double f = c_g.fac[jc];
    if (kind == 0) {          // theta -> n3
      acc[0] += f * dw * rho;
    } else if (kind == 1) {   // delta -> n2, n1, n0, V2, V1
      acc[1] += f * dw * rho;
      if (!c_g.single_size) {
        acc[2] += f * c_g.inv_4pir[jc] * dw * rho;
        acc[3] += f * c_g.inv_4pirsq[jc] * dw * rho;
      }
      for (int d = 0; d < nd; d++) {
        const double v = (double)o[d] * c_g.esize[d] * c_g.inv_rad[jc];
        acc[4 + d] += f * v * dw * rho;
        if (!c_g.single_size) acc[4 + nd + d] += f * c_g.inv_4pir[jc] * v * dw * rho;
      }
    } else {                  // mean field
      acc[orow] += dw * rho;
    }
  }
}

// conv rows 0..nrb-1 (do_fmt) and nrb..nrb+ncomp-1 (do_mf) of the target nodes
__global__ void k_hw_correct(const double *__restrict__ field, long fcs, int ffirst, HwSet hs, int do_fmt, int do_mf,
                             const int *__restrict__ targets, int ntargets, const signed char *__restrict__ zero,
                             const int *__restrict__ bnodes, const short *__restrict__ fmask,
                             double *__restrict__ conv)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntargets) return;
  const long i = targets[t];
  int ijk[3];
  node_ijk(i, ijk);
  const int nc = c_g.ncomp;
  double acc[kMaxRb + kMaxC];
  for (int k = 0; k < kMaxRb + kMaxC; k++) acc[k] = 0.0;
  for (int jc = 0; jc < nc; jc++) {
    const int jlist = (c_g.nlists <= 2) ? 0 : jc;
    if (do_fmt) {
      hw_apply(hs.th[jc], 0, 0, jc, jlist, ijk, field, fcs, ffirst, zero, bnodes, fmask, acc);
      hw_apply(hs.de[jc], 1, 0, jc, jlist, ijk, field, fcs, ffirst, zero, bnodes, fmask, acc);
    }
    if (do_mf)
      for (int ic = 0; ic < nc; ic++)
        hw_apply(hs.ua[ic + kMaxC * jc], 2, c_g.nrb + ic, jc, jlist, ijk, field, fcs, ffirst, zero, bnodes, fmask, acc);
  }
  if (do_fmt)
    for (int k = 0; k < c_g.nrb; k++) conv[(long)k * c_g.N + i] += acc[k];
  if (do_mf)
    for (int ic = 0; ic < nc; ic++) conv[(long)(c_g.nrb + ic) * c_g.N + i] += acc[c_g.nrb + ic];
}

static HwSet hw_set(const DevStencil *theta, const DevStencil *delta, const DevStencil *uatt, int ncomp)
{
  HwSet h{};
  for (int c = 0; c < kMaxC && c < ncomp; c++) {
    if (theta && theta[c].L) h.th[c] = {theta[c].L, theta[c].d_off, theta[c].d_w, theta[c].d_hw};
    if (delta && delta[c].L) h.de[c] = {delta[c].L, delta[c].d_off, delta[c].d_w, delta[c].d_hw};
  }
  if (uatt)
    for (int jc = 0; jc < kMaxC && jc < ncomp; jc++)
      for (int ic = 0; ic < kMaxC && ic < ncomp; ic++) {
        const DevStencil &u = uatt[ic + ncomp * jc];
        if (u.L && u.d_hw) h.ua[ic + kMaxC * jc] = {u.L, u.d_off, u.d_w, u.d_hw};
      }
  return h;
}

void launch_hw_correct(const double *field, long fcs, int ffirst, const DevStencil *theta, const DevStencil *delta,
                       const DevStencil *uatt, int ncomp, bool do_fmt, bool do_mf, const int *targets, int ntargets,
                       const signed char *zero, const int *bnodes, const short *fmask, double *conv, cudaStream_t s)
{
  if (ntargets <= 0) return;
  k_hw_correct<<<(ntargets + 127) / 128, 128, 0, s>>>(field, fcs, ffirst, hw_set(theta, delta, uatt, ncomp),
                                                       do_fmt ? 1 : 0, do_mf ? 1 : 0, targets, ntargets, zero, bnodes,
                                                       fmask, conv);
}

// Reflecting boundaries in the transposed sums.  A forward sum reads a mirrored
// position p (beyond a reflecting boundary) as its interior image m(p), with a
// sign flip of vector channels; its transpose therefore evaluates the transposed
// sum T(p) = sum_s coef_s in(p - o_s) also at mirrored positions (the input is
// the zero extension, k_pad with no_mirror, read at interior nodes only) and adds sign T(p) into out(m(p)).
// One thread per padded position; mirrored positions of one interior node come
// from several threads: FP64 atomic additions.
struct FoldOut {
  double *p[kMaxRb];
  int signmask[kMaxRb];   // bit d: the output flips sign under a reflection in dimension d
};

__global__ void k_reflect_fold(const double *__restrict__ in, long cstride, int nin, const short *__restrict__ off,
                               const double *__restrict__ coef, int L, int nout, FoldOut out)
{
  const long NP = c_g.NP;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < NP; p += (long)gridDim.x * blockDim.x) {
    const int q[3] = {(int)(p % c_g.P[0]), (int)((p / c_g.P[0]) % c_g.P[1]), (int)(p / ((long)c_g.P[0] * c_g.P[1]))};
    int refl = 0, idx[3] = {0, 0, 0};
    bool ok = true;
    for (int d = 0; d < c_g.ndim; d++) {
      const int m = c_g.map[d][q[d]];
      if (m < 0) { ok = false; break; }
      if (m & kReflBit) refl |= 1 << d;
      idx[d] = m & ~kReflBit;
    }
    if (!ok || !refl) continue;
    const long node = idx[0] + (long)c_g.nx[0] * (idx[1] + (long)c_g.nx[1] * idx[2]);
    double t[kMaxRb];
    for (int o = 0; o < nout; o++) t[o] = 0.0;
    for (int s = 0; s < L; s++) {
      // only reads from interior nodes p - o_s exist (a periodic image in the halo is the same read landing
      // at another padded position, counted there)
      const short *os = off + (long)s * 3;
      long qi = 0;
      bool inb = true;
      for (int d = 0; d < c_g.ndim; d++) {
        const int qq = q[d] - os[d];
        if (qq < c_g.h[d] || qq >= c_g.h[d] + c_g.nx[d]) { inb = false; break; }
        qi += (long)qq * c_g.pstride[d];
      }
      if (!inb) continue;
      for (int o = 0; o < nout; o++)
        for (int c = 0; c < nin; c++) t[o] += coef[((long)s * nout + o) * nin + c] * in[(long)c * cstride + qi];
    }
    for (int o = 0; o < nout; o++) {
      const double v = (__popc(refl & out.signmask[o]) & 1) ? -t[o] : t[o];
      if (v != 0.0) atomicAdd(out.p[o] + node, v);
    }
  }
}

void launch_reflect_fold(const double *in, long cstride, int nin, const short *off, const double *coef, int L,
                         double *const *outs, const int *signmask, int nout, cudaStream_t s)
{
  FoldOut o{};
  for (int k = 0; k < nout; k++) {
    o.p[k] = outs[k];
    o.signmask[k] = signmask[k];
  }
  k_reflect_fold<<<1184, kThreads, 0, s>>>(in, cstride, nin, off, coef, L, nout, o);
}

// Transpose of the hard-wall correction: the density column of every boundary node j receives, from each
// target node i whose stencil point lands on j, the weight change times the adjoint rows at i (the
// coefficients of hw_apply): the rb rows of w for theta and delta, the mean-field rows (mfw, N apart) for the
// mean-field stencils.  Several targets reach one j: FP64 atomic additions.
__device__ void hw_apply_t(const HwStencil &st, int kind, int jc, int jlist, const int *ijk,
                           const double *__restrict__ W, const signed char *zero, const int *bnodes,
                           const short *fmask, double *out)
{
  const long N = c_g.N;
  const int nd = c_g.ndim;
  const int nel = 1 << nd;
  for (int s = 0; s < st.L; s++) {
    int refl;
    const short *o = st.off + (long)s * 3;
    const long jn = map_offset(ijk, o, &refl);
    if (jn < 0) continue;
    if (bnodes[(long)jlist * N + jn] == -1) continue;
    if (zero[(long)jc * N + jn]) continue;
    const int mask = fmask[((long)jlist * nel + refl) * N + jn];
    double wh = 0.0;
    for (int l = 0; l < nel; l++)
      if (mask & (1 << l)) wh += st.hw[(long)s * nel + l];
    const double dw = wh - st.w[s];
    double g;
    if (kind == 0) {
      g = c_g.fac[jc] * W[0];
    } else if (kind == 1) {
      g = W[N];
      if (!c_g.single_size) g += c_g.inv_4pir[jc] * W[2 * N] + c_g.inv_4pirsq[jc] * W[3 * N];
      for (int d = 0; d < nd; d++) {
        const double v = (double)o[d] * c_g.esize[d] * c_g.inv_rad[jc];
        g += v * W[(long)(4 + d) * N];
        if (!c_g.single_size) g += c_g.inv_4pir[jc] * v * W[(long)(4 + nd + d) * N];
      }
      g *= c_g.fac[jc];
    } else {
      g = W[0];
    }
    atomicAdd(out + (long)(c_g.first_rho + jc) * N + jn, dw * g);
  }
}

__global__ void k_hw_correct_t(const double *__restrict__ w, const double *__restrict__ mfw, HwSet hs, int do_fmt,
                               int do_mf, const int *__restrict__ targets, int ntargets,
                               const signed char *__restrict__ zero, const int *__restrict__ bnodes,
                               const short *__restrict__ fmask, double *__restrict__ out)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntargets) return;
  const long i = targets[t];
  const long N = c_g.N;
  int ijk[3];
  node_ijk(i, ijk);
  const int nc = c_g.ncomp;
  for (int jc = 0; jc < nc; jc++) {
    const int jlist = (c_g.nlists <= 2) ? 0 : jc;
    if (do_fmt) {
      const double *W = w + (long)c_g.first_rb * N + i;   // adjoint rb rows at i, N apart
      hw_apply_t(hs.th[jc], 0, jc, jlist, ijk, W, zero, bnodes, fmask, out);
      hw_apply_t(hs.de[jc], 1, jc, jlist, ijk, W, zero, bnodes, fmask, out);
    }
    if (do_mf)
      for (int ic = 0; ic < nc; ic++)
        hw_apply_t(hs.ua[ic + kMaxC * jc], 2, jc, jlist, ijk, mfw + (long)ic * N + i, zero, bnodes, fmask, out);
  }
}

void launch_hw_correct_t(const double *w, const double *mfw, const DevStencil *theta, const DevStencil *delta,
                         const DevStencil *uatt, int ncomp, bool do_fmt, bool do_mf, const int *targets, int ntargets,
                         const signed char *zero, const int *bnodes, const short *fmask, double *out, cudaStream_t s)
{
  if (ntargets <= 0) return;
  k_hw_correct_t<<<(ntargets + 127) / 128, 128, 0, s>>>(w, mfw, hw_set(theta, delta, uatt, ncomp), do_fmt ? 1 : 0,
                                                         do_mf ? 1 : 0, targets, ntargets, zero, bnodes, fmask, out);
}

// ---------------------------------------------------------------------------
// Krylov and Newton vector kernels.  Reductions are two-level and ordered
// (per-block partials, then one block in fixed order): results do not depend
// on scheduling, so runs repeat bit for bit.
int reduce_blocks(long n)
{
  long b = (n + kThreads * 4 - 1) / (kThreads * 4);
  if (b > 1024) b = 1024;
  if (b < 1) b = 1;
  return (int)b;
}

__device__ __forceinline__ double block_sum(double v, double *sh)
{
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  v = 0.0;
  if (wid == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

__device__ __forceinline__ double block_min(double v, double *sh)
{
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  v = 1.0e300;
  if (wid == 0) {
    v = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 1.0e300;
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  }
  __syncthreads();
  return v;
}

// The last block of a reduction to finish adds up every block's partials, in block order as k_reduce_rows does
// (the same result, without its launch): the blocks count themselves in an unsigned counter, which that last
// block resets.  Partials written by other blocks are read through L2.
__device__ __forceinline__ bool last_block_done(unsigned *counter)
{
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  return last;
}

__device__ void reduce_rows_last(const double *partial, int nb, int nrow, double *out, double *sh, unsigned *counter)
{
  for (int j = 0; j < nrow; j++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += __ldcg(partial + (long)j * nb + b);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[j] = s;
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// partial[j*nb + b] = sum over block b's chunk of V[j] . w; out[j] = sum over b (the last block)
__global__ void k_multidot(const double *__restrict__ V, long ldv, int nvec, const double *__restrict__ w, long n,
                           double *__restrict__ partial, double *__restrict__ out, unsigned *__restrict__ counter)
{
  __shared__ double sh[32];
  const long chunk = (n + gridDim.x - 1) / gridDim.x;
  const long b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  for (int j = 0; j < nvec; j++) {
    double s = 0.0;
    for (long i = b0 + threadIdx.x; i < b1; i += blockDim.x) s = fma(V[(long)j * ldv + i], w[i], s);
    s = block_sum(s, sh);
    if (threadIdx.x == 0) partial[(long)j * gridDim.x + blockIdx.x] = s;
  }
  if (last_block_done(counter)) reduce_rows_last(partial, gridDim.x, nvec, out, sh, counter);
}

__global__ void k_reduce_rows(const double *__restrict__ partial, int nb, int nrow, double *__restrict__ out)
{
  __shared__ double sh[32];
  for (int j = 0; j < nrow; j++) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += partial[(long)j * nb + b];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[j] = s;
  }
}

// partial: the base of a kPartialWords reduction buffer (its last word is the completion counter)
void launch_multidot(const double *V, long ldv, int nvec, const double *w, long n, double *partial, int nblocks,
                     double *result, cudaStream_t s)
{
  unsigned *counter = reinterpret_cast<unsigned *>(partial + kPartialWords - 1);
  k_multidot<<<nblocks, kThreads, 0, s>>>(V, ldv, nvec, w, n, partial, result, counter);
}

__global__ void k_multiaxpy(double *__restrict__ w, const double *__restrict__ V, long ldv, int nvec,
                            const double *__restrict__ coef, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double s = w[i];
    for (int j = 0; j < nvec; j++) s -= coef[j] * V[(long)j * ldv + i];
    w[i] = s;
  }
}

void launch_multiaxpy(double *w, const double *V, long ldv, int nvec, const double *coef, long n, cudaStream_t s)
{
  k_multiaxpy<<<1184, kThreads, 0, s>>>(w, V, ldv, nvec, coef, n);
}

__global__ void k_scale(double *__restrict__ y, const double *__restrict__ x, double a, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] = a * x[i];
}

void launch_scale(double *y, const double *x, double a, long n, cudaStream_t s)
{
  k_scale<<<1184, kThreads, 0, s>>>(y, x, a, n);
}

__global__ void k_axpby(double *__restrict__ y, double a, const double *__restrict__ x, double b, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    y[i] = a * x[i] + b * y[i];
}

void launch_axpby(double *y, double a, const double *x, double b, long n, cudaStream_t s)
{
  k_axpby<<<1184, kThreads, 0, s>>>(y, a, x, b, n);
}

// A22^-1: A22 is diagonal, 1/rho on Euler-Lagrange rows and 1 on zero-density rows.
__global__ void k_precond(const double *__restrict__ x, const double *__restrict__ vext,
                          const signed char *__restrict__ zero, const double *__restrict__ in, double *__restrict__ out)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long k = (long)ic * N + i;
      out[k] = (zero_row(vext, zero, ic, i) && !log_row(vext, zero, ic, i))
                   ? in[k]
                   : in[k] * x[(long)(c_g.first_rho + ic) * N + i];
    }
}

void launch_precond(const double *x, const double *vext, const signed char *zero, const double *in, double *out,
                    cudaStream_t s)
{
  k_precond<<<1184, kThreads, 0, s>>>(x, vext, zero, in, out);
}

__global__ void k_newton_frac(const double *__restrict__ x, const double *__restrict__ dx, double floor_frac,
                              double *__restrict__ partial)
{
  __shared__ double sh[32];
  const long N = c_g.N;
  double m = 1.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long k = (long)(c_g.first_rho + ic) * N + i;
      if (x[k] + dx[k] < 0.0) {
        double f = fmin(1.0, x[k] / (-dx[k]));
        f = fmax(f, floor_frac);
        m = fmin(m, f);
      }
    }
  m = block_min(m, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = m;
}

__global__ void k_min_final(const double *__restrict__ partial, int nb, double *__restrict__ out)
{
  __shared__ double sh[32];
  double m = 1.0e300;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) m = fmin(m, partial[b]);
  m = block_min(m, sh);
  if (threadIdx.x == 0) out[0] = m;
}

void launch_newton_frac(const double *x, const double *dx, double floor_frac, double *partial, int nblocks,
                        double *result, cudaStream_t s)
{
  k_newton_frac<<<nblocks, kThreads, 0, s>>>(x, dx, floor_frac, partial);
  k_min_final<<<1, kThreads, 0, s>>>(partial, nblocks, result);
}

// partial != null: also the weighted update norm (a convergence test, <= 1): its quotients in FP32 and its squares
// summed in FP32 per thread (FP64 divisions per unknown made this kernel FP64-bound); the residual-targeted Newton
// needs no norm and skips it
__global__ void k_newton_update(double *__restrict__ x, const double *__restrict__ dx, double frac, double rel,
                                double abs_tol, double *__restrict__ partial)
{
  __shared__ double sh[32];
  const long N = c_g.N;
  const bool norm = partial != nullptr;
  float s = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int iu = 0; iu < c_g.nunk; iu++) {
      const long k = (long)iu * N + i;
      const double xo = x[k], d = dx[k];
      const double xn = fma(frac, d, xo);
      if (norm) {
        float t = (float)(frac * d) / (float)fma(rel, xo, abs_tol);
        if (fabsf(t) > 1.0e18f) t = 1.0e18f;   // any term above 1 fails the test; NaN passes through to the check
        s = fmaf(t, t, s);
      }
      const bool is_rho = iu >= c_g.first_rho && iu < c_g.first_rho + c_g.ncomp;
      if (is_rho && xn < 1.e-99) x[k] = 0.1 * xo;
      else if (iu == c_g.first_rb && xn > 1.0) x[k] = xo + 0.5 * (1.0 - xo);
      else x[k] = xn;
    }
  if (!norm) return;
  const double sb = block_sum((double)s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = sb;
}

void launch_newton_update(double *x, const double *dx, double frac, double rel, double abs_tol, double *partial,
                          int nblocks, double *result, cudaStream_t s)
{
  if (!partial) {
    k_newton_update<<<nblocks, kThreads, 0, s>>>(x, dx, frac, rel, abs_tol, nullptr);
    return;
  }
  k_newton_update<<<nblocks, kThreads, 0, s>>>(x, dx, frac, rel, abs_tol, partial);
  k_reduce_rows<<<1, kThreads, 0, s>>>(partial, nblocks, 1, result);
}

__global__ void k_norm2(const double *__restrict__ x, long n, double *__restrict__ partial, double *__restrict__ out,
                        unsigned *__restrict__ counter)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    s = fma(x[i], x[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
  if (last_block_done(counter)) reduce_rows_last(partial, gridDim.x, 1, out, sh, counter);
}

// partial: the base of a kPartialWords reduction buffer (its last word is the completion counter)
void launch_norm2(const double *x, long n, double *partial, int nblocks, double *result, cudaStream_t s)
{
  unsigned *counter = reinterpret_cast<unsigned *>(partial + kPartialWords - 1);
  k_norm2<<<nblocks, kThreads, 0, s>>>(x, n, partial, result, counter);
}

// out = a - ref; result[0] = max |a - ref|, result[1] = max |a|
__global__ void k_delta_maxabs(const double *__restrict__ a, const double *__restrict__ ref, long n,
                               double *__restrict__ out, double *__restrict__ partial)
{
  __shared__ double sh[32];
  double m0 = 0.0, m1 = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double d = a[i] - ref[i];
    out[i] = d;
    m0 = fmax(m0, fabs(d));
    m1 = fmax(m1, fabs(a[i]));
  }
  m0 = -block_min(-m0, sh);
  m1 = -block_min(-m1, sh);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = m0;
    partial[gridDim.x + blockIdx.x] = m1;
  }
}

__global__ void k_max_final2(const double *__restrict__ partial, int nb, double *__restrict__ out)
{
  __shared__ double sh[32];
  double m0 = 0.0, m1 = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    m0 = fmax(m0, partial[b]);
    m1 = fmax(m1, partial[nb + b]);
  }
  m0 = -block_min(-m0, sh);
  m1 = -block_min(-m1, sh);
  if (threadIdx.x == 0) {
    out[0] = m0;
    out[1] = m1;
  }
}

void launch_delta_maxabs(const double *a, const double *ref, long n, double *out, double *partial, int nblocks,
                         double *result, cudaStream_t s)
{
  k_delta_maxabs<<<nblocks, kThreads, 0, s>>>(a, ref, n, out, partial);
  k_max_final2<<<1, kThreads, 0, s>>>(partial, nblocks, result);
}

// counts non-finite entries (result = count as double)
__global__ void k_count_nonfinite(const double *__restrict__ x, long n, double *__restrict__ partial)
{
  __shared__ double sh[32];
  double s = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    if (!isfinite(x[i])) s += 1.0;
  s = block_sum(s, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

void launch_check_finite(const double *x, long n, double *partial, int nblocks, double *result, cudaStream_t s)
{
  k_count_nonfinite<<<nblocks, kThreads, 0, s>>>(x, n, partial);
  k_reduce_rows<<<1, kThreads, 0, s>>>(partial, nblocks, 1, result);
}

// ---------------------------------------------------------------------------
// Objectives of a state: the surface excess grand free energy Omega_s of
// calc_free_energy (src/dft_energy.c:31-168: ideal gas, chemical potential,
// external field, hard-sphere and mean-field terms, each minus its bulk term)
// and the excess adsorption of calc_adsorption (src/dft_out_ads.c:33-112),
// both as integrateInSpace sums (src/dft_out_utils.c:38-62) with per-node
// weights wf (Nel_hit2) and wb (Nel_hit) that already hold Vol_el /
// Nnodes_per_el_V and the area / reflection factors.  The mean-field term takes
// the attraction sums S_ic (int_stencil, src/dft_energy_CLSintsten.c:73) of
// the densities; the hard-sphere term Phi(n) reads the weighted-density
// unknowns and uses component 0's wb, as integrand_hs_freen does.
// partial rows: [0] Omega_s, [1 + ic] Gamma_ex[ic].
__global__ void k_objectives(const double *__restrict__ x, const double *__restrict__ vext,
                             const double *__restrict__ satt, const double *__restrict__ wf,
                             const double *__restrict__ wb, ObjConst oc, double *__restrict__ partial)
{
  __shared__ double sh[32];
  const long N = c_g.N;
  const int nc = c_g.ncomp;
  double om = 0.0, gam[kMaxC];
  for (int ic = 0; ic < kMaxC; ic++) gam[ic] = 0.0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    for (int ic = 0; ic < nc; ic++) {
      const long k = (long)ic * N + i;
      const double rho = x[(long)(c_g.first_rho + ic) * N + i];
      double e = 0.0;
      if (rho > kDensityMin) e = rho * (log(rho) - 1.0) - rho * oc.betamu[ic] + rho * vext[k];
      if (c_g.attraction && rho > 0.0) e += 0.5 * rho * satt[k];
      om += wf[k] * e - wb[k] * oc.bulk[ic];
      gam[ic] += wf[k] * rho - wb[k] * c_g.rho_b[ic];
    }
    double n[kMaxRb];
    load_n(x, i, n);
    om += wb[i] * (fmt_phi(n, c_g.ndim, c_g.functional) - oc.phi_b);
  }
  om = block_sum(om, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = om;
  for (int ic = 0; ic < nc; ic++) {
    const double v = block_sum(gam[ic], sh);
    if (threadIdx.x == 0) partial[(long)(1 + ic) * gridDim.x + blockIdx.x] = v;
  }
}

void launch_objectives(const double *x, const double *vext, const double *satt, const double *wf, const double *wb,
                       const ObjConst &oc, int ncomp, double *partial, int nblocks, double *result, cudaStream_t s)
{
  k_objectives<<<nblocks, kThreads, 0, s>>>(x, vext, satt, wf, wb, oc, partial);
  k_reduce_rows<<<1, kThreads, 0, s>>>(partial, nblocks, 1 + ncomp, result);
}

// Partial derivatives of an objective at fixed V_ext.
//   kind 0 (Omega_s): d/drho_ic = wf (ln rho - betamu + V) + wf S/2 and, from the
//   other nodes' mean-field terms, T_ic/2 (added by the caller: the transposed
//   attraction sums of wf rho); d/dn_k = wb0 dPhi/dn_k; d/dV_ic = wf rho.
//   kind 1 (Gamma_ex[icomp]): d/drho_icomp = wf.
// gx [nunk][N], gv [ncomp][N]; the MF unknowns do not enter (the mean-field
// term integrates the attraction sums of the densities, not the unknowns).
// chan (kind 0, attraction): wf rho on rho > 0 nodes per component [ncomp][N].
__global__ void k_objective_grad(const double *__restrict__ x, const double *__restrict__ vext,
                                 const double *__restrict__ satt, const double *__restrict__ wf,
                                 const double *__restrict__ wb, ObjConst oc, int kind, int icomp,
                                 double *__restrict__ gx, double *__restrict__ gv, double *__restrict__ chan)
{
  const long N = c_g.N;
  const int nc = c_g.ncomp;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    for (int u = 0; u < c_g.nunk; u++) gx[(long)u * N + i] = 0.0;
    for (int ic = 0; ic < nc; ic++) {
      const long k = (long)ic * N + i;
      const double rho = x[(long)(c_g.first_rho + ic) * N + i];
      double g = 0.0, v = 0.0;
      if (kind == 0) {
        if (rho > kDensityMin) {
          g = wf[k] * (log(rho) - oc.betamu[ic] + vext[k]);
          v = wf[k] * rho;
        }
        if (c_g.attraction) {
          if (rho > 0.0) g += 0.5 * wf[k] * satt[k];
          chan[k] = rho > 0.0 ? wf[k] * rho : 0.0;
        }
      } else if (ic == icomp) {
        g = wf[k];
      }
      gx[(long)(c_g.first_rho + ic) * N + i] = g;
      gv[k] = v;
    }
    if (kind == 0) {
      double n[kMaxRb], d[kMaxRb];
      load_n(x, i, n);
      fmt_dphi(n, d);
      const int nd = c_g.ndim;
      const double w0 = wb[i];
      double *G = gx + (long)c_g.first_rb * N + i;
      G[0] = w0 * d[3];
      G[N] = w0 * d[2];
      G[2 * N] = w0 * d[1];
      G[3 * N] = w0 * d[0];
      for (int dd = 0; dd < nd; dd++) {
        G[(long)(4 + dd) * N] = w0 * d[4 + nd + dd];
        G[(long)(4 + nd + dd) * N] = w0 * d[4 + dd];
      }
    }
  }
}

void launch_objective_grad(const double *x, const double *vext, const double *satt, const double *wf,
                           const double *wb, const ObjConst &oc, int kind, int icomp, double *gx, double *gv,
                           double *chan, cudaStream_t s)
{
  k_objective_grad<<<1184, kThreads, 0, s>>>(x, vext, satt, wf, wb, oc, kind, icomp, gx, gv, chan);
}

// dF/dV_ext = dF/dV|_x - lambda on the Euler-Lagrange rows that hold +V_ext (full rows and PB_ZONE rows),
// dF/dV|_x elsewhere
__global__ void k_vext_sens(const double *__restrict__ lam, const double *__restrict__ gv,
                            const double *__restrict__ vext, const signed char *__restrict__ zero,
                            double *__restrict__ out)
{
  const long N = c_g.N;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
    for (int ic = 0; ic < c_g.ncomp; ic++) {
      const long k = (long)ic * N + i;
      out[k] = vext_row(vext, zero, ic, i) ? gv[k] - lam[(long)(c_g.first_rho + ic) * N + i] : gv[k];
    }
}

void launch_vext_sens(const double *lam, const double *gv, const double *vext, const signed char *zero, double *out,
                      cudaStream_t s)
{
  k_vext_sens<<<1184, kThreads, 0, s>>>(lam, gv, vext, zero, out);
}

}  // namespace tgpu
