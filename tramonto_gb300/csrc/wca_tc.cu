// Large 3-D single-channel stencil sums on the tensor cores (tcgen05, split FP16 x3, FP32 accumulate).
//
// out(x, y, z) (+)= sum_(ox,oy,oz) w(ox,oy,oz) f(x+ox, y+oy, z+oz)
//
// For one stencil line (oy, oz) the sum over ox is a 1-D convolution along x,
// i.e. a banded Toeplitz matrix T[k][n] = w(k - n - const) applied to x-rows
// of the field.  A CTA owns a tile of 64 x-outputs by 128 y-rows of one
// z-plane and accumulates, for every line, D[y][n] += sum_k F[y + oy][k] T[k][n]
// with one tcgen05.mma (M = 128 y-rows, N = 64, K = 16 x-inputs) per 16 inputs
// of the line's band:
//   A (M x K, K-major, shared memory) = the field slab of plane z + oz: rows
//     y0 - hy .. y0 + 127 + hy, 128 x-inputs from x0 - 32; the line's oy is a
//     row offset of the descriptor's start address (rows are 16 B apart in the
//     no-swizzle core-matrix layout, so any row offset is a valid start);
//   B (N x K, K-major, shared memory) = the line's Toeplitz matrix with the
//     output index reversed (n' = 63 - n), which makes it a Hankel matrix: its
//     8x8 core matrices depend only on g + j' (k-group + n'-group), so a line
//     needs 24 distinct core matrices (3 KB) and the descriptor walks them with
//     both strides equal to one core matrix (128 B);
//   D (128 x 64 FP32) = 64 TMEM columns, read back with tcgen05.ld and written
//     (x reversed) to the FP64 output.
// The field slab of each plane (high and low parts) arrives by one 5-D TMA tile
// load from a copy of the padded field kept as [part][z][x/8][y][x%8] FP16 (the
// core-matrix order), the line tables (high and low) by 1-D bulk copies into a
// ring; one warp produces, one issues the MMAs, tcgen05.commit releases slots
// through mbarriers, and four warps drain the TMEM accumulators.  Every mbarrier wait is bounded: a wait that
// runs out sets an error flag, the CTA drains what it started and frees TMEM.
//
// Precision: the field is scaled by a power of two so that max |f| <= 1 and
// the weights so that max |w| <= 1, and each is split into FP16 high and low
// parts (f = f_hi + f_lo, w = w_hi + w_lo); every K-step issues three MMAs,
// f_hi w_hi + f_hi w_lo + f_lo w_hi, so the products carry ~22 bits (the
// FP32-class accuracy a single FP16 pass, ~11 bits, does not reach on rough
// fields).  The epilogue undoes both scales.
#include <cuda.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <map>
#include <vector>

#include "tgpu_internal.h"

namespace tgpu {

namespace {

constexpr int kRing = kTcRing;

template <typename T>
T *upload_vec(const std::vector<T> &h, cudaStream_t s)
{
  T *d = nullptr;
  if (cudaMalloc(&d, std::max<size_t>(1, h.size()) * sizeof(T)) != cudaSuccess) return nullptr;
  if (!h.empty()) cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
  return d;
}
constexpr int kTableHalfs = kTcCores * 64;              // one part (high or low) of a line's table
// a record: int4 {oy_a, oy_b, first K-step | last K-step << 8, lines (1 or 2)}, then the high and the low
// table; the lines oy_a and oy_b of one plane share it when their weights are equal (the stencil's mirror
// symmetry in y)
constexpr int kRecHalfs = 8 + 2 * kTableHalfs;
constexpr uint32_t kTableBytes = 2 * kRecHalfs;
constexpr long kSpin = 1L << 21;
constexpr int kAccBufs = 4;   // chunk accumulator sets in TMEM
constexpr int kRot = 1;       // accumulators per set (64 columns each), taken in turn by consecutive MMAs
constexpr int kChunk = 4;     // lines per accumulation chunk

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// bounded wait for the phase with the given parity to complete (limit: try_wait attempts)
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long limit = kSpin)
{
  for (long i = 0; i < limit; i++) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            int c4, uint32_t bar)
{
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

__device__ __forceinline__ void bulk_load(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// shared-memory matrix descriptor: no swizzle, start / leading (K) / stride (M or N) byte offsets
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, uint32_t *r)
{
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}

struct TcArgs {
  const int4 *planes;     // {oz, first record, records, lines}
  const __half *tables;   // records: int4 header, high and low tables
  int nplanes, nring;
  int nsplit;             // CTAs per output tile, each over a contiguous range of planes
  int split_first[9];     // plane ranges [split_first[k], split_first[k + 1])
  int nx, ny, nz, hy, hz, R;
  const float *in_scale;  // device: the field's scale
  double out_mult;        // 1 / weight scale
  double *out;
  int accumulate;
  int *err;
  long spin;              // limit of the pipeline's waits (the drain before exit always uses kSpin)
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// shared memory (128-B aligned): two plane buffers [part][16][R][8] halves, the
// ring of line tables [part][24][8][8], then the mbarriers plane_full[2]
// plane_empty[2] b_full[kRing] b_empty[kRing] acc_full[kAccBufs]
// acc_empty[kAccBufs] acc_done, the TMEM address, the abort flag and the
// per-slot counts of started and consumed copies.
//
// Warps 0-3 drain the accumulators (warp w owns TMEM lanes 32w..32w+31, i.e.
// y rows), warp 4 lane 0 produces the copies, warp 5 lane 0 issues the MMAs.
// The lines are taken in chunks of kChunk; chunk c accumulates in TMEM set
// c % kAccBufs from zero (kRot accumulators of 64 columns per set, used in
// turn by consecutive MMAs; one is fastest: rotating over four measured 30%
// slower, consecutive MMAs into the same accumulator being the cheap case), and the drain warps add each
// finished chunk into FP32 register sums (ordinary round-to-nearest adds).  Short chunks keep the number of
// accumulations into one FP32 accumulator small: the tensor core adds the
// products of an MMA to the accumulator with a rounding that shrinks its
// magnitude slightly, which over the ~2e4 MMAs of a whole stencil grows to a
// few 1e-4 of the sum, and to ~1e-6 over one chunk.
__global__ void __launch_bounds__(192, 1) k_sten_tc(const __grid_constant__ CUtensorMap tmap, TcArgs P)
{
  extern __shared__ uint8_t smem_raw[];
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 127u) & ~127u;
  uint8_t *gb = smem_raw + (base - raw);
  const uint32_t part_bytes = 256u * (uint32_t)P.R;   // one part of one plane: 16 groups x R rows x 16 B
  const uint32_t plane_bytes = 2 * part_bytes;
  const uint32_t plane[2] = {base, base + plane_bytes};
  const uint32_t ring = base + 2 * plane_bytes;
  const int nring = P.nring;
  const uint32_t bars = ring + nring * kTableBytes;
  const uint32_t pfull = bars, pempty = bars + 16, bfull = bars + 32, bempty = bars + 32 + 8 * kRing;
  const uint32_t afull = bars + 32 + 16 * kRing, aempty = afull + 8 * kAccBufs;
  const uint32_t accb = aempty + 8 * kAccBufs;
  const uint32_t tslot = accb + 8;
  volatile int *abort_flag = reinterpret_cast<volatile int *>(gb + (tslot + 4 - base));
  int *armed = reinterpret_cast<int *>(gb + (tslot + 8 - base));
  int *used = armed + 2 + kRing;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x0 = blockIdx.x * kTcN, y0 = blockIdx.y * kTcM;
  const int z = blockIdx.z / P.nsplit, part = blockIdx.z % P.nsplit;
  const int p_begin = P.split_first[part], p_end = P.split_first[part + 1];
  const int np = p_end - p_begin;
  int nlines_total = 0;
  for (int pi = p_begin; pi < p_end; pi++) nlines_total += P.planes[pi].w;
  const int nchunks = (nlines_total + kChunk - 1) / kChunk;

  if (threadIdx.x == 0) {
    for (int i = 0; i < 2; i++) {
      mbar_init(pfull + 8 * i, 1);
      mbar_init(pempty + 8 * i, 1);
    }
    for (int i = 0; i < nring; i++) {
      mbar_init(bfull + 8 * i, 1);
      mbar_init(bempty + 8 * i, 1);
    }
    for (int i = 0; i < kAccBufs; i++) {
      mbar_init(afull + 8 * i, 1);
      mbar_init(aempty + 8 * i, 128);
    }
    mbar_init(accb, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (threadIdx.x < 2 + kRing) armed[threadIdx.x] = used[threadIdx.x] = 0;
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tslot),
                 "r"(kTcN * kAccBufs * kRot)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(gb + (tslot - base));

  if (warp == 4) {
    if (lane == 0) {
      // producer: plane slabs (5-D TMA, both parts) and line tables (bulk copies)
      bool ok = true;
      int ri = 0;   // running record index (ring slot)
      for (int pi = 0; pi < np && ok; pi++) {
        const int4 pl = P.planes[p_begin + pi];
        const int s = pi & 1;
        if (pi >= 2 && !mbar_wait(pempty + 8 * s, ((pi >> 1) - 1) & 1, P.spin)) { ok = false; break; }
        mbar_expect_tx(pfull + 8 * s, plane_bytes);
        tma_load_5d(plane[s], &tmap, 0, y0, x0 / 8, z + pl.x + P.hz, 0, pfull + 8 * s);
        armed[s]++;
        for (int rj = 0; rj < pl.z; rj++, ri++) {
          const int bs = ri % nring;
          if (ri >= nring && !mbar_wait(bempty + 8 * bs, ((ri / nring) - 1) & 1, P.spin)) { ok = false; break; }
          if (*abort_flag) { ok = false; break; }
          mbar_expect_tx(bfull + 8 * bs, kTableBytes);
          bulk_load(ring + bs * kTableBytes, P.tables + (size_t)(pl.y + rj) * kRecHalfs, kTableBytes, bfull + 8 * bs);
          armed[2 + bs]++;
        }
      }
      if (!ok) {
        *abort_flag = 1;
        atomicExch(P.err, 1);
      }
    }
    __syncwarp();
  } else if (warp == 5) {
    if (lane == 0) {
      // MMA issue: M = 128 (y), N = 64 (x, reversed), K = 16 per instruction; FP16 inputs, FP32 accumulator
      const uint32_t idesc = (1u << 4) | ((uint32_t)(kTcN >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);
      const uint32_t lbo_a = 16u * (uint32_t)P.R;
      bool ok = true;
      int bi = 0;   // running line index (chunks)
      int ri = 0;   // running record index (ring slot)
      int rot = 0;                        // next accumulator of the current set
      uint32_t fresh = (1u << kRot) - 1;  // accumulators not yet written in the current chunk
      for (int pi = 0; pi < np && ok; pi++) {
        const int4 pl = P.planes[p_begin + pi];
        const int s = pi & 1;
        if (!mbar_wait(pfull + 8 * s, (pi >> 1) & 1, P.spin)) { ok = false; break; }
        used[s]++;
        for (int rj = 0; rj < pl.z && ok; rj++, ri++) {
          const int bs = ri % nring;
          if (!mbar_wait(bfull + 8 * bs, (ri / nring) & 1, P.spin)) { ok = false; break; }
          if (*abort_flag) { ok = false; break; }
          used[2 + bs]++;
          tc_fence_after();
          const uint32_t btab = ring + bs * kTableBytes;
          const int4 hd = *reinterpret_cast<const int4 *>(gb + (btab - base));   // the record's header
          const int k_lo = hd.z & 0xff, k_hi = hd.z >> 8;
          for (int j = 0; j < hd.w; j++, bi++) {
            const int chunk = bi / kChunk, cb = chunk % kAccBufs;
            const bool chunk_start = bi % kChunk == 0;
            if (chunk_start && chunk >= kAccBufs && !mbar_wait(aempty + 8 * cb, ((chunk / kAccBufs) - 1) & 1, P.spin)) {
              ok = false;
              break;
            }
            if (chunk_start) tc_fence_after();
            if (chunk_start) {
              rot = 0;
              fresh = (1u << kRot) - 1;
            }
            const int oy = j == 0 ? hd.x : hd.y;
            const uint32_t arow = plane[s] + 16u * (uint32_t)(oy + P.hy);
            const uint32_t dset = tmem + (uint32_t)(cb * kRot * kTcN);
            for (int k = k_lo; k <= k_hi; k++) {
              const uint32_t ak = arow + 2u * (uint32_t)k * lbo_a, bk = btab + 16u + 256u * (uint32_t)k;
              const uint64_t a_hi = sdesc(ak, lbo_a, 128), a_lo = sdesc(ak + part_bytes, lbo_a, 128);
              const uint64_t b_hi = sdesc(bk, 128, 128), b_lo = sdesc(bk + 2u * kTableHalfs, 128, 128);
              // the set's accumulators in turn (one per set: consecutive MMAs into the same accumulator)
              const uint64_t ops[3][2] = {{a_lo, b_hi}, {a_hi, b_lo}, {a_hi, b_hi}};
#pragma unroll
              for (int q = 0; q < 3; q++) {
                const uint32_t use = (fresh >> rot) & 1u ? 0u : 1u;
                tc_mma(dset + (uint32_t)(rot * kTcN), ops[q][0], ops[q][1], idesc, use);
                fresh &= ~(1u << rot);
                rot = (rot + 1) % kRot;
              }
            }
            if (bi % kChunk == kChunk - 1 || bi == nlines_total - 1) tc_commit(afull + 8 * cb);
          }
          tc_commit(bempty + 8 * bs);
        }
        if (!ok) break;
        tc_commit(pempty + 8 * s);
      }
      tc_commit(accb);   // fires once every MMA issued above has completed
      if (!ok) {
        *abort_flag = 1;
        atomicExch(P.err, 2);
      }
    }
    __syncwarp();
  } else {
    // drain warps: add every finished chunk into FP32 register sums (round-to-nearest, unbiased), then write
    float sum[kTcN];
#pragma unroll
    for (int n = 0; n < kTcN; n++) sum[n] = 0.0f;
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
    bool ok = true;
    for (int c = 0; c < nchunks; c++) {
      const int cb = c % kAccBufs;
      bool got = false;
      for (int it = 0; it < 4 && !got; it++) {
        if (*abort_flag) break;
        got = mbar_wait(afull + 8 * cb, (c / kAccBufs) & 1, P.spin);
      }
      got = __all_sync(0xffffffffu, got);
      if (!got) { ok = false; break; }
      tc_fence_after();
      uint32_t r[16];
      for (int q = 0; q < kRot; q++) {
#pragma unroll
        for (int h = 0; h < kTcN; h += 16) {
          tc_ld16(tmem + lane_off + (uint32_t)((cb * kRot + q) * kTcN + h), r);
          asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
          for (int n = 0; n < 16; n++) sum[h + n] += __uint_as_float(r[n]);
        }
      }
      tc_fence_before();
      mbar_arrive(aempty + 8 * cb);
    }
    if (ok) {
      const int y = y0 + warp * 32 + lane;
      const double mult = P.out_mult / (double)P.in_scale[0];
      if (y < P.ny) {
        double *row = P.out + ((long)z * P.ny + y) * P.nx;
#pragma unroll
        for (int n = 0; n < kTcN; n++) {
          const int x = x0 + kTcN - 1 - n;
          const double v = (double)sum[n] * mult;
          if (x < P.nx) {
            if (P.nsplit > 1) atomicAdd(row + x, v);
            else row[x] = P.accumulate ? row[x] + v : v;
          }
        }
      }
    } else if (lane == 0) {
      *abort_flag = 1;
      atomicExch(P.err, 3);
    }
  }
  // every MMA has completed before TMEM is freed; copies started but not consumed land before exit
  if (threadIdx.x == 0) mbar_wait(accb, 0, kSpin);
  tc_fence_before();
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < 2 + nring; i++)
      if (armed[i] > used[i]) {
        const uint32_t bar = i < 2 ? pfull + 8 * i : bfull + 8 * (i - 2);
        mbar_wait(bar, (armed[i] - 1) & 1, kSpin);
      }
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcN * kAccBufs * kRot)
                 : "memory");
  }
}

// FP32 padded channel -> FP16 slab copy [part][zp][g][yp][8] (x index xs = 8 g + l - 32 + h0 in the FP32
// box), scaled; part 0 holds the FP16 rounding of the value, part 1 the FP16 rounding of the remainder
__global__ void k_slab16(const float *__restrict__ pad, long P0, long P1, long P2, int h0, int G,
                         const float *__restrict__ scale, __half *__restrict__ slab)
{
  const long total = (long)P2 * G * P1 * 8;
  const float s = scale[0];
  for (long o = blockIdx.x * (long)blockDim.x + threadIdx.x; o < total; o += (long)gridDim.x * blockDim.x) {
    const int l = (int)(o & 7);
    const long yp = (o >> 3) % P1;
    const long g = (o / (8 * P1)) % G;
    const long zp = o / (8 * P1 * G);
    const long xs = 8 * g + l - kTcXHalo + h0;
    float v = 0.0f;
    if (xs >= 0 && xs < P0) v = pad[(zp * P1 + yp) * P0 + xs] * s;
    const __half hi = __float2half_rn(v);
    slab[o] = hi;
    slab[total + o] = __float2half_rn(v - __half2float(hi));
  }
}

// max |pad| into scale[1] (as the bits of a non-negative float; scale[1] zeroed before)
__global__ void k_absmax(const float *__restrict__ pad, long n, float *__restrict__ scale)
{
  float m = 0.0f;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(pad[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(reinterpret_cast<int *>(scale + 1), __float_as_int(m));
}

// scale[0] = 2^-e with 2^(e-1) <= max |pad| < 2^e (1 for an all-zero or non-finite field)
__global__ void k_scale_from_max(float *scale)
{
  const float m = scale[1];
  int e = 0;
  if (m > 0.0f && isfinite(m)) frexpf(m, &e);
  scale[0] = ldexpf(1.0f, -e);
}

}  // namespace

size_t tc_smem_bytes(int R, int nring)
{
  return 128 + 2 * 512 * (size_t)R + (size_t)nring * kTableBytes + 32 + 16 * kRing + 16 * kAccBufs + 16 +
         8 * (2 + kRing);
}

bool tc_build_tables(const std::vector<short> &off, const std::vector<double> &w, int L, int hy, TcTables &t,
                     cudaStream_t s)
{
  // lines (oz, oy) -> {ox -> w}
  std::map<int, std::map<int, std::map<int, double>>> lines;
  double wmax = 0.0;
  for (int k = 0; k < L; k++) {
    const int ox = off[(size_t)k * 3], oy = off[(size_t)k * 3 + 1], oz = off[(size_t)k * 3 + 2];
    if (ox < -kTcXHalo || ox > kTcXHalo || oy < -hy || oy > hy) return false;
    lines[oz][oy][ox] += w[k];
    wmax = std::max(wmax, std::fabs(w[k]));
  }
  if (wmax == 0.0) return false;
  int e = 0;
  std::frexp(wmax, &e);
  const double sw = std::ldexp(1.0, -e);
  std::vector<int4> planes, lns;
  std::vector<__half> tab;
  auto same_profile = [&](const std::map<int, double> &a, const std::map<int, double> &b) {
    if (a.size() != b.size()) return false;
    for (auto ia = a.begin(), ib = b.begin(); ia != a.end(); ++ia, ++ib)
      if (ia->first != ib->first || std::fabs(ia->second - ib->second) > 1e-12 * wmax) return false;
    return true;
  };
  for (auto &pz : lines) {
    const int first = (int)(tab.size() / kRecHalfs);
    int nl = 0;
    for (auto &py : pz.second) {
      if (py.first < 0) {
        auto mirror = pz.second.find(-py.first);
        if (mirror != pz.second.end() && same_profile(py.second, mirror->second)) continue;   // shares +oy's record
      }
      int oy_b = INT32_MIN, nrec = 1;
      if (py.first > 0) {
        auto mirror = pz.second.find(-py.first);
        if (mirror != pz.second.end() && same_profile(py.second, mirror->second)) { oy_b = -py.first; nrec = 2; }
      }
      int l = 0;
      for (auto &px : py.second) l = std::max(l, std::abs(px.first));
      const int table = (int)(tab.size() / kRecHalfs);
      tab.resize(tab.size() + kRecHalfs, __float2half_rn(0.0f));
      __half *T = tab.data() + (size_t)table * kRecHalfs + 8;
      // core matrix d, row b (n' in group), column a (k in group): w(8d + a + b - (32 + 63)); high then low part
      for (int d = 0; d < kTcCores; d++)
        for (int b = 0; b < 8; b++)
          for (int a = 0; a < 8; a++) {
            const int ox = 8 * d + a + b - (kTcXHalo + kTcN - 1);
            auto it = py.second.find(ox);
            if (it == py.second.end()) continue;
            const double v = it->second * sw;
            const __half hi = __float2half_rn((float)v);
            T[d * 64 + b * 8 + a] = hi;
            T[kTableHalfs + d * 64 + b * 8 + a] = __float2half_rn((float)(v - (double)__half2float(hi)));
          }
      const int k_lo = (kTcXHalo - l) / 16, k_hi = (kTcXHalo + kTcN - 1 + l) / 16;
      const int4 head = make_int4(py.first, oy_b, k_lo | (k_hi << 8), nrec);
      std::memcpy(tab.data() + (size_t)table * kRecHalfs, &head, sizeof(head));
      lns.push_back(head);
      nl += nrec;
    }
    planes.push_back(make_int4(pz.first, first, (int)(tab.size() / kRecHalfs) - first, nl));
  }
  t.nplanes = (int)planes.size();
  t.nlines = 0;
  for (auto &pl : planes) t.nlines += pl.w;
  // plane ranges for 1..8 CTAs per tile, balanced by line count
  for (int ns = 1; ns <= 8; ns++) {
    t.split_first[ns][0] = 0;
    int k = 1, acc = 0;
    for (int pi = 0; pi < t.nplanes && k < ns; pi++) {
      acc += planes[pi].w;
      if ((long)acc * ns >= (long)k * t.nlines) t.split_first[ns][k++] = pi + 1;
    }
    while (k <= ns) t.split_first[ns][k++] = t.nplanes;
  }
  t.out_mult = 1.0 / sw;
  t.d_planes = upload_vec(planes, s);
  t.d_lines = upload_vec(lns, s);
  t.d_tables = upload_vec(tab, s);
  cudaStreamSynchronize(s);
  return t.d_planes && t.d_lines && t.d_tables;
}

namespace {
using EncodeFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                              const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                              CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
}

bool tc_make_slab(TcSlab &sl, const DevGeom &g, std::string &why)
{
  sl.G = (int)((g.nx[0] + 2 * kTcXHalo + 7) / 8);
  sl.Yp = g.P[1];
  sl.Zp = g.P[2];
  sl.R = kTcM + 2 * g.h[1];
  sl.hy = g.h[1];
  sl.hz = g.h[2];
  if (sl.R > 256) { why = "y reach above 64 nodes"; return false; }
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaDeviceGetAttribute(&sl.nsm, cudaDevAttrMultiProcessorCount, dev);
  sl.nring = 0;
  for (int r = kTcRing; r >= 2; r--)
    if (tc_smem_bytes(sl.R, r) <= (size_t)optin) { sl.nring = r; break; }
  if (sl.nring < 2) { why = "shared memory too small for the slab planes"; return false; }
  const size_t n = (size_t)2 * sl.Zp * sl.G * sl.Yp * 8;
  if (cudaMalloc(&sl.d_slab, n * sizeof(__half)) != cudaSuccess) { why = "cudaMalloc"; return false; }
  cudaMemset(sl.d_slab, 0, n * sizeof(__half));
  if (cudaMalloc(&sl.d_scale, 4 * sizeof(float)) != cudaSuccess) { why = "cudaMalloc"; return false; }
  if (cudaMalloc(&sl.d_err, sizeof(int)) != cudaSuccess) { why = "cudaMalloc"; return false; }
  cudaMemset(sl.d_err, 0, sizeof(int));
  void *fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !fn) {
    why = "cuTensorMapEncodeTiled not available";
    return false;
  }
  const cuuint64_t part = (cuuint64_t)sl.Zp * sl.G * sl.Yp * 16;
  const cuuint64_t dims[5] = {8, (cuuint64_t)sl.Yp, (cuuint64_t)sl.G, (cuuint64_t)sl.Zp, 2};
  const cuuint64_t strides[4] = {16, (cuuint64_t)sl.Yp * 16, (cuuint64_t)sl.G * sl.Yp * 16, part};
  const cuuint32_t box[5] = {8, (cuuint32_t)sl.R, 16, 1, 2};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = reinterpret_cast<EncodeFn>(fn)(&sl.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 5, sl.d_slab, dims,
                                                    strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) { why = "cuTensorMapEncodeTiled failed"; return false; }
  if (cudaFuncSetAttribute(k_sten_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)tc_smem_bytes(sl.R, sl.nring)) != cudaSuccess) {
    why = "dynamic shared memory";
    return false;
  }
  return true;
}

void tc_free_slab(TcSlab &sl)
{
  if (sl.d_slab) cudaFree(sl.d_slab);
  if (sl.d_scale) cudaFree(sl.d_scale);
  if (sl.d_err) cudaFree(sl.d_err);
  sl.d_slab = nullptr;
  sl.d_scale = nullptr;
  sl.d_err = nullptr;
}

void tc_free_tables(TcTables &t)
{
  if (t.d_planes) cudaFree(t.d_planes);
  if (t.d_lines) cudaFree(t.d_lines);
  if (t.d_tables) cudaFree(t.d_tables);
  t = TcTables{};
}

void launch_sten_tc(const float *pad_channel, const DevGeom &g, const TcSlab &sl, const TcTables &t, double *out,
                    bool accumulate, cudaStream_t s)
{
  cudaMemsetAsync(sl.d_scale + 1, 0, sizeof(float), s);
  k_absmax<<<1184, 256, 0, s>>>(pad_channel, g.NP, sl.d_scale);
  k_scale_from_max<<<1, 1, 0, s>>>(sl.d_scale);
  k_slab16<<<1184, 256, 0, s>>>(pad_channel, g.P[0], g.P[1], g.P[2], g.h[0], sl.G, sl.d_scale,
                                static_cast<__half *>(sl.d_slab));
  TcArgs a;
  a.planes = t.d_planes;
  a.tables = static_cast<const __half *>(t.d_tables);
  a.nplanes = t.nplanes;
  a.nring = sl.nring;
  a.nx = g.nx[0];
  a.ny = g.nx[1];
  a.nz = g.nx[2];
  a.hy = sl.hy;
  a.hz = sl.hz;
  a.R = sl.R;
  a.in_scale = sl.d_scale;
  a.out_mult = t.out_mult;
  a.out = out;
  a.accumulate = accumulate ? 1 : 0;
  a.err = sl.d_err;
  a.spin = sl.spin > 0 ? sl.spin : kSpin;
  const int tiles = ((g.nx[0] + kTcN - 1) / kTcN) * ((g.nx[1] + kTcM - 1) / kTcM) * g.nx[2];
  const int ns = accumulate ? t.split_for(tiles, sl.nsm) : 1;
  a.nsplit = ns;
  for (int k = 0; k <= ns; k++) a.split_first[k] = t.split_first[ns][k];
  const dim3 grid((g.nx[0] + kTcN - 1) / kTcN, (g.nx[1] + kTcM - 1) / kTcM, g.nx[2] * ns);
  k_sten_tc<<<grid, 192, tc_smem_bytes(sl.R, sl.nring), s>>>(sl.tmap, a);
}

}  // namespace tgpu
