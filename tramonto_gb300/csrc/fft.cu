// Three-dimensional real-to-complex FFTs for the stencil sums (FP64 in the accurate fills and FP64-accurate
// products, FP32 in the FP32 products and fills).
//
// A stencil sum out(i) = sum_o c(o) f(i + o) over the mesh, with the reference's boundary rules, is a
// correlation.  Along a periodic dimension of n nodes it is exactly the circular correlation of period n; along
// any other dimension the padded channel (the field extended by the boundary rules over the stencil's reach h)
// is transformed on a length F >= P = n + 2h, where the circular correlation equals the sum for every interior
// output.  So the transform box is [F2][F1][F0] with F_d = n_d on periodic dimensions (when n_d is a product of
// 2, 3 and 5) and the smallest such F_d >= P_d elsewhere; with the correlation kernel g[(-o) mod F] = c(o)
// (points that wrap onto the same position add up, as the reference folds a stencil wider than a periodic box),
// one forward transform of the field, a product with the kernel's spectrum and one inverse transform give the
// sum at a cost that does not depend on the stencil's length.  At 128^3 with the attraction reach of 25 nodes
// that is a 180 x 128 x 128 box: 2.9e6 points against 5.8e6 for a box padded in every dimension.
//
// The field is real, so only the half spectrum k0 < F0/2 + 1 is kept ([F2][F1][F0/2 + 1] complex): along x two
// real lines are packed as the real and imaginary parts of one complex line, transformed together and split
// by Hermitian symmetry (A[k] = (Z[k] + conj Z[-k]) / 2, B[k] = (Z[k] - conj Z[-k]) / 2i); the inverse packs
// two half-spectrum lines as Z = A + iB (extended by conjugate symmetry) and returns them as the real and
// imaginary parts of one inverse transform.  The x passes read the padded channel directly and write the
// interior outputs directly (no load or extraction pass); the y and z passes are batches of complex transforms
// over the half-spectrum box.
//
// Each 1-D transform runs in shared memory as a mixed-radix Stockham autosort FFT (radices 2, 3, 4, 5; the
// iteration of Govindaraju, Lloyd, Dotsenko, Smith and Manferdelli, "High performance discrete Fourier
// transforms on graphics processors", SC 2008: butterfly j reads j + r n/R, multiplies by
// W_{Ns R}^{r (j mod Ns)}, takes an R-point DFT and writes (j / Ns) Ns R + (j mod Ns) + r Ns).  The 3- and
// 5-point DFTs use the symmetric forms that share the sums and differences of mirrored inputs (two real
// multiplications per output pair instead of a full complex product per term).  Twiddles are tabulated on
// the host in extended precision.  The inverse uses conjugate twiddles; its 1/(F0 F1 F2) is applied on output.
// The spectral products (one kernel spectrum per output, or the sum of channel-times-kernel products of a
// transposed sum) are formed while the first inverse pass loads its lines.
#include <cmath>
#include <type_traits>
#include <vector>

#include "tgpu_internal.h"

namespace tgpu {

namespace {

constexpr int kFftLines = 8;     // complex lines per CTA tile
constexpr int kFftThreads = 256;
constexpr int kFftMaxN = 432;    // two ping-pong tiles of kFftLines lines and the twiddles fit in shared memory
constexpr int kBlockLoadBatch = 4;   // global loads a thread issues before storing them to the tile

struct Stages {
  int nst;
  int rad[16];
  int Ns[16];                    // product of the earlier radices (one-warp-per-line passes)
  int step[16];                  // twiddle stride n / (Ns R)
  unsigned magic[16];            // ceil(2^32 / Ns), 0 when Ns = 1: j / Ns = umulhi(j, magic) for j < 2^16
};

template <class C>
struct Real;
template <>
struct Real<double2> {
  using T = double;
};
template <>
struct Real<float2> {
  using T = float;
};

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

// a + s (-i b) for the forward transform (s = +1), a + s (i b) for the inverse
template <class C>
__device__ __forceinline__ C add_mi(C a, C b, int inv)
{
  return inv ? C{a.x - b.y, a.y + b.x} : C{a.x + b.y, a.y - b.x};
}
template <class C>
__device__ __forceinline__ C sub_mi(C a, C b, int inv)
{
  return inv ? C{a.x + b.y, a.y - b.x} : C{a.x - b.y, a.y + b.x};
}

// R-point DFT of v in place (forward: exp(-2 pi i r k / R); inverse: conjugate); R known at compile time so that
// v stays in registers
template <int R, class C>
__device__ __forceinline__ void dft_small(C *v, int inv)
{
  using T = typename Real<C>::T;
  if (R == 2) {
    const C a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (R == 3) {
    // y1,2 = v0 - (v1 + v2)/2 -/+ i (sqrt 3 / 2)(v1 - v2)
    const T s3 = (T)0.86602540378443864676;
    const C a = cadd(v[1], v[2]), b = csub(v[1], v[2]);
    const C m = C{v[0].x - (T)0.5 * a.x, v[0].y - (T)0.5 * a.y};
    const C s = C{s3 * b.x, s3 * b.y};
    v[0] = cadd(v[0], a);
    v[1] = add_mi(m, s, inv);
    v[2] = sub_mi(m, s, inv);
  } else if (R == 4) {
    const C y0 = cadd(v[0], v[2]), y1 = csub(v[0], v[2]), y2 = cadd(v[1], v[3]), y3 = csub(v[1], v[3]);
    v[0] = cadd(y0, y2);
    v[2] = csub(y0, y2);
    v[1] = add_mi(y1, y3, inv);
    v[3] = sub_mi(y1, y3, inv);
  } else {
    // 5 points: with a1 = v1 + v4, b1 = v1 - v4, a2 = v2 + v3, b2 = v2 - v3,
    // y1,4 = v0 + c1 a1 + c2 a2 -/+ i (s1 b1 + s2 b2),  y2,3 = v0 + c2 a1 + c1 a2 -/+ i (s2 b1 - s1 b2)
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
    const C a1 = cadd(v[1], v[4]), b1 = csub(v[1], v[4]), a2 = cadd(v[2], v[3]), b2 = csub(v[2], v[3]);
    const C m1 = C{v[0].x + c1 * a1.x + c2 * a2.x, v[0].y + c1 * a1.y + c2 * a2.y};
    const C m2 = C{v[0].x + c2 * a1.x + c1 * a2.x, v[0].y + c2 * a1.y + c1 * a2.y};
    const C n1 = C{s1 * b1.x + s2 * b2.x, s1 * b1.y + s2 * b2.y};
    const C n2 = C{s2 * b1.x - s1 * b2.x, s2 * b1.y - s1 * b2.y};
    v[0] = C{v[0].x + a1.x + a2.x, v[0].y + a1.y + a2.y};
    v[1] = add_mi(m1, n1, inv);
    v[4] = sub_mi(m1, n1, inv);
    v[2] = add_mi(m2, n2, inv);
    v[3] = sub_mi(m2, n2, inv);
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
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tw, r * k * step, inv));
    }
    dft_small<R, C>(v, inv);
    const int idx = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) dst[idx + r * Ns] = v[r];
  }
}

// stages of one tile of nlines lines (line stride ls) from buf0; returns the buffer holding the result
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

// ---- compile-time codelets for the common lengths -------------------------------------------------------------
// The passes are bound by instruction issue; for the lengths the 3-D workloads use, the stages' radices, strides,
// twiddle steps and the direction are template constants (no runtime switch, division or direction selects).  The
// radices of N in stage order (fours first, then 2, 3, 5; any order gives the DFT in natural order):
__host__ __device__ constexpr int ct_radix(int n, int s)
{
  for (int k = 0; n > 1; k++) {
    const int r = n % 4 == 0 ? 4 : n % 2 == 0 ? 2 : n % 3 == 0 ? 3 : n % 5 == 0 ? 5 : 0;
    if (r == 0) return 0;
    if (k == s) return r;
    n /= r;
  }
  return 0;
}
__host__ __device__ constexpr int ct_ns(int n, int s)   // product of the radices before stage s
{
  int p = 1;
  for (int k = 0; k < s; k++) p *= ct_radix(n, k);
  return p;
}
__host__ __device__ constexpr bool ct_factors(int n)    // n a product of 2, 3, 5
{
  while (n % 2 == 0) n /= 2;
  while (n % 3 == 0) n /= 3;
  while (n % 5 == 0) n /= 5;
  return n == 1;
}

template <int R, int N, int NS, bool INV, class C>
__device__ __forceinline__ void fft_stage_ct(const C *in, C *out, int ls, int nlines, const C *tw)
{
  constexpr int nb = N / R, step = N / (NS * R);
  for (int t = threadIdx.x; t < nlines * nb; t += blockDim.x) {
    const int line = t / nb, j = t - line * nb;
    const C *src = in + line * ls;
    C *dst = out + line * ls;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * nb];
    const int q = j / NS, k = j - q * NS;
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        C w = tw[r * k * step];
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dft_small<R, C>(v, INV ? 1 : 0);
    const int idx = q * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) dst[idx + r * NS] = v[r];
  }
}

template <int N, int S, bool INV, class C>
struct TileFftCt {
  static __device__ __forceinline__ C *run(C *in, C *out, int ls, int nlines, const C *tw)
  {
    constexpr int R = ct_radix(N, S);
    if constexpr (R == 0) {
      return in;
    } else {
      fft_stage_ct<R, N, ct_ns(N, S), INV, C>(in, out, ls, nlines, tw);
      __syncthreads();
      return TileFftCt<N, S + 1, INV, C>::run(out, in, ls, nlines, tw);
    }
  }
};

// fft_tile for the lengths with codelets (N = 0: the run-time stages)
template <int N, bool INV, class C>
__device__ __forceinline__ C *tile_fft_n(C *b0, C *b1, int n, int ls, int nlines, const Stages &st, const C *tw)
{
  if constexpr (N == 0) return fft_tile<C>(b0, b1, n, ls, nlines, st, tw, INV ? 1 : 0);
  else return TileFftCt<N, 0, INV, C>::run(b0, b1, ls, nlines, tw);
}

// Geometry of the real box as the x passes see it: where a line's values come from (forward) or go to (inverse)
struct XGeom {
  int F0, F1, Fh;            // transform lengths along x and y, half-spectrum length along x
  long nlines;               // real lines F1 * F2
  // forward source: element (x, y, z) of the box is the source at padded position (x + off0, y + off1, z + off2)
  // when x < ext0, y < ext1, z < ext2, else 0
  int off[3], ext[3];
  // inverse destination: box position p holds output node p - e (interior nodes only)
  int e[3], nx[3];
};

// Sources of the forward x pass: element (x, y, z) of the real box (x < ext0, y < ext1, z < ext2; 0 beyond)
// at padded position (x + off0, y + off1, z + off2)
template <class T>
struct BoxSrc {   // a padded channel, or a real box [F2][F1][F0] (off 0)
  const T *p;
  long sy, sz;
  __device__ __forceinline__ T operator()(const XGeom &g, int x, int y, int z) const
  {
    return p[(long)(z + g.off[2]) * sz + (long)(y + g.off[1]) * sy + x + g.off[0]];
  }
  // a line's part of the address, then the element (the warp passes read a line at a time)
  struct Line {
    long base;
  };
  __device__ __forceinline__ Line line(const XGeom &g, int y, int z) const
  {
    return Line{(long)(z + g.off[2]) * sz + (long)(y + g.off[1]) * sy + g.off[0]};
  }
  __device__ __forceinline__ T at(const XGeom &, const Line &L, int x) const { return p[L.base + x]; }
};
template <class T>
struct MappedSrc {   // the unpadded channel through the boundary maps (the padded box's values, computed)
  MapSrc m;
  __device__ __forceinline__ T operator()(const XGeom &g, int x, int y, int z) const
  {
    const int q[3] = {x + g.off[0], y + g.off[1], z + g.off[2]};
    int idx[3] = {0, 0, 0}, refl = 0;
    for (int d = 0; d < m.ndim; d++) {
      const int v = m.map[d][q[d]];
      if (v < 0) {   // the first out-of-range dimension decides (the reference's order)
        if (v == kSentBulk) return (T)m.bulk_lo;
        if (v == kSentBulkHi) return (T)m.bulk_hi;
        if (v == kSentWall) return (T)0;
        return (T)__longlong_as_double(0x7ff8000000000000ULL);   // no node to read (as the padded box holds)
      }
      if (v & kReflBit) refl |= 1 << d;
      idx[d] = v & ~kReflBit;
    }
    const long node = idx[0] + (long)m.nx[0] * (idx[1] + (long)m.nx[1] * idx[2]);
    if (m.zc >= 0 && m.zero[(long)m.zc * m.N + node]) return (T)0;
    const T v = m.src32 ? (T)m.src32[node] : to_arith<T>(m.src[node]);
    return (__popc(refl & m.signmask) & 1) ? -v : v;
  }
  // the same with the y and z part of a line resolved once: the node offset and reflections of the line, or the
  // sentinel of its first out-of-range dimension after x (x still decides first)
  struct Line {
    long base;
    int refl, sent;   // sent 0: the line is inside
  };
  __device__ __forceinline__ Line line(const XGeom &g, int y, int z) const
  {
    Line L{0, 0, 0};
    const int q[3] = {0, y + g.off[1], z + g.off[2]};
    long idx[3] = {0, 0, 0};
    for (int d = 1; d < m.ndim; d++) {
      const int v = m.map[d][q[d]];
      if (v < 0) {
        L.sent = v;
        return L;
      }
      if (v & kReflBit) L.refl |= 1 << d;
      idx[d] = v & ~kReflBit;
    }
    L.base = (long)m.nx[0] * (idx[1] + (long)m.nx[1] * idx[2]);
    return L;
  }
  __device__ __forceinline__ T sentinel(int v) const
  {
    if (v == kSentBulk) return (T)m.bulk_lo;
    if (v == kSentBulkHi) return (T)m.bulk_hi;
    if (v == kSentWall) return (T)0;
    return (T)__longlong_as_double(0x7ff8000000000000ULL);
  }
  __device__ __forceinline__ T at(const XGeom &g, const Line &L, int x) const
  {
    const int v = m.map[0][x + g.off[0]];
    if (v < 0) return sentinel(v);
    if (L.sent) return sentinel(L.sent);
    const int refl = L.refl | ((v & kReflBit) ? 1 : 0);
    const long node = L.base + (v & ~kReflBit);
    if (m.zc >= 0 && m.zero[(long)m.zc * m.N + node]) return (T)0;
    const T val = m.src32 ? (T)m.src32[node] : to_arith<T>(m.src[node]);
    return (__popc(refl & m.signmask) & 1) ? -val : val;
  }
};

// spectral products formed by a pass as it loads its lines: value = sum_t a_t * k_t (n = 0: the input itself)
constexpr int kMaxTerms = 6;
template <class C>
struct Terms {
  const C *a[kMaxTerms];
  const C *k[kMaxTerms];
  int n;
};

// up to kMaxBatch transforms of one plan in one launch (blockIdx.y selects the transform)
constexpr int kMaxBatch = 8;
template <class C>
struct PassBatch {
  const C *in[kMaxBatch];
  C *out[kMaxBatch];
  Terms<C> terms[kMaxBatch];
};

template <class Src, class C>
struct SrcBatch {
  Src src[kMaxBatch];
  C *spec[kMaxBatch];
};

template <class C>
struct OutBatch {
  const C *spec[kMaxBatch];
  double *out[kMaxBatch];
  float *out32[kMaxBatch];   // FP32 outputs (the FP32 transforms; used instead of out when set)
};

// x pass of the forward transform: two real lines per complex line, split into two half-spectrum lines
template <class T, class C, class Src, int NC = 0>
__global__ void __launch_bounds__(kFftThreads) k_rfft_x(SrcBatch<Src, C> sb, XGeom g, Stages st,
                                                      const C *__restrict__ tw_g)
{
  const Src &src = sb.src[blockIdx.y];
  C *__restrict__ spec = sb.spec[blockIdx.y];
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int n = NC ? NC : g.F0, ls = n + 1;
  C *b0 = sm, *b1 = sm + kFftLines * ls, *tw = b1 + kFftLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  const long pair0 = (long)blockIdx.x * kFftLines;
  const long npairs = (g.nlines + 1) / 2;
  const int np = (int)min((long)kFftLines, npairs - pair0);
  for (int q = threadIdx.x; q < np * n; q += blockDim.x) {
    const int l = q / n, x = q - l * n;
    T v[2] = {0, 0};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const long L = 2 * (pair0 + l) + h;
      if (L >= g.nlines) break;
      const int y = (int)(L % g.F1), z = (int)(L / g.F1);
      if (x < g.ext[0] && y < g.ext[1] && z < g.ext[2]) v[h] = src(g, x, y, z);
    }
    b0[l * ls + x] = C{v[0], v[1]};
  }
  __syncthreads();
  const C *res = tile_fft_n<NC, false, C>(b0, b1, n, ls, np, st, tw);
  using R = T;
  for (int q = threadIdx.x; q < np * g.Fh; q += blockDim.x) {
    const int l = q / g.Fh, k = q - l * g.Fh;
    const C Z = res[l * ls + k], Zm = res[l * ls + (k == 0 ? 0 : n - k)];
    const long L = 2 * (pair0 + l);
    spec[L * g.Fh + k] = C{(R)0.5 * (Z.x + Zm.x), (R)0.5 * (Z.y - Zm.y)};
    if (L + 1 < g.nlines) spec[(L + 1) * g.Fh + k] = C{(R)0.5 * (Z.y + Zm.y), (R)0.5 * (Zm.x - Z.x)};
  }
}

// x pass of the inverse transform: two half-spectrum lines as one complex line, written out as the real outputs
// of the interior nodes (out[node] = scale * value, or += when accumulate)
template <class C, int NC = 0>
__global__ void __launch_bounds__(kFftThreads) k_irfft_x(OutBatch<C> ob, XGeom g, Stages st,
                                                       const C *__restrict__ tw_g, double scale, int accumulate)
{
  const C *__restrict__ spec = ob.spec[blockIdx.y];
  double *__restrict__ out = ob.out[blockIdx.y];
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int n = NC ? NC : g.F0, ls = n + 1;
  C *b0 = sm, *b1 = sm + kFftLines * ls, *tw = b1 + kFftLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  const long pair0 = (long)blockIdx.x * kFftLines;
  const long npairs = (g.nlines + 1) / 2;
  const int np = (int)min((long)kFftLines, npairs - pair0);
  for (int q = threadIdx.x; q < np * n; q += blockDim.x) {
    const int l = q / n, k = q - l * n;
    const long L = 2 * (pair0 + l);
    const bool up = k < g.Fh;
    const int kk = up ? k : n - k;
    const C A = spec[L * g.Fh + kk];
    const C B = L + 1 < g.nlines ? spec[(L + 1) * g.Fh + kk] : C{0, 0};
    // Z = A + iB on the stored half; conj(A) + i conj(B) on the mirrored half
    b0[l * ls + k] = up ? C{A.x - B.y, A.y + B.x} : C{A.x + B.y, B.x - A.y};
  }
  __syncthreads();
  const C *res = tile_fft_n<NC, true, C>(b0, b1, n, ls, np, st, tw);
  const int nx0 = g.nx[0];
  for (int q = threadIdx.x; q < np * 2 * nx0; q += blockDim.x) {
    const int lh = q / nx0, x = q - lh * nx0;
    const int l = lh >> 1, h = lh & 1;
    const long L = 2 * (pair0 + l) + h;
    if (L >= g.nlines) continue;
    const int y = (int)(L % g.F1) - g.e[1], z = (int)(L / g.F1) - g.e[2];
    if (y < 0 || y >= g.nx[1] || z < 0 || z >= g.nx[2]) continue;
    const C r = res[l * ls + x + g.e[0]];
    const double v = scale * (double)(h ? r.y : r.x);
    double *o = out + ((long)z * g.nx[1] + y) * nx0 + x;
    *o = accumulate ? *o + v : v;
  }
}

// y and z passes: lines of element stride es; a CTA takes kFftLines consecutive x at one (outer) index; reads `in`
// (or the products of `terms`) and writes `out` (in place when out == in)
template <class C, int NC, bool INV>
__global__ void __launch_bounds__(kFftThreads) k_fft_strided(PassBatch<C> pb, int X, int n_rt, long es,
                                                           long outer_stride, Stages st, const C *__restrict__ tw_g)
{
  const int n = NC ? NC : n_rt;
  const C *in = pb.in[blockIdx.y];
  C *out = pb.out[blockIdx.y];
  const Terms<C> &terms = pb.terms[blockIdx.y];
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int ls = n + 1;
  C *b0 = sm, *b1 = sm + kFftLines * ls, *tw = b1 + kFftLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  const int xblocks = (X + kFftLines - 1) / kFftLines;
  const int x0 = (blockIdx.x % xblocks) * kFftLines;
  const long base = (long)(blockIdx.x / xblocks) * outer_stride + x0;
  const int nl = min(kFftLines, X - x0);
  const int total = kFftLines * n;
  for (int q0 = threadIdx.x; q0 < total; q0 += kBlockLoadBatch * blockDim.x) {   // loads first, then stores
    C v[kBlockLoadBatch];
#pragma unroll
    for (int b = 0; b < kBlockLoadBatch; b++) {
      const int q = q0 + b * blockDim.x;
      const int e = q / kFftLines, l = q - e * kFftLines;
      v[b] = C{0, 0};
      if (q < total && l < nl) {
        const long idx = base + e * es + l;
        if (terms.n == 0) {
          v[b] = in[idx];
        } else {
          v[b] = cmul(terms.a[0][idx], terms.k[0][idx]);
          for (int t = 1; t < terms.n; t++) v[b] = cadd(v[b], cmul(terms.a[t][idx], terms.k[t][idx]));
        }
      }
    }
#pragma unroll
    for (int b = 0; b < kBlockLoadBatch; b++) {
      const int q = q0 + b * blockDim.x;
      if (q < total) b0[(q % kFftLines) * ls + q / kFftLines] = v[b];
    }
  }
  __syncthreads();
  const C *res = tile_fft_n<NC, INV, C>(b0, b1, n, ls, nl, st, tw);
  for (int q = threadIdx.x; q < kFftLines * n; q += blockDim.x) {
    const int e = q / kFftLines, l = q - e * kFftLines;
    if (l < nl) out[base + e * es + l] = res[l * ls + e];
  }
}

// ---- FP32 passes: one warp per line ------------------------------------------------------------------------
// The FP32 passes are bound by latency and instruction issue, not arithmetic: here a warp owns a line, so the
// stages of a line synchronise only the warp (the block synchronises around its coalesced loads and stores), and
// the butterflies index without runtime divisions (j / Ns by a precomputed 32-bit reciprocal).  The FP64 passes
// keep the block tile above: FP64 issue slots are the bound there, and spreading a stage's butterflies over the
// whole block leaves fewer of them on partly filled warps (at 180 points a warp per line leaves up to 28 of 64
// lane slots of a stage idle).
constexpr int kWLines = 16;   // lines (one warp each) per CTA
constexpr int kLoadBatch = 4; // global loads a thread issues before it stores them to shared memory

template <int R, class C>
__device__ __forceinline__ void warp_stage(const C *src, C *dst, int n, int Ns, int step, unsigned magic,
                                           const C *tw, int inv, int lane)
{
  const int nb = n / R;
  for (int j = lane; j < nb; j += 32) {
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * nb];
    const int q = Ns == 1 ? j : (int)__umulhi((unsigned)j, magic);   // j / Ns
    const int k = j - q * Ns;
    if (Ns > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) v[r] = cmul(v[r], twiddle(tw, r * k * step, inv));
    }
    dft_small<R, C>(v, inv);
    const int idx = q * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) dst[idx + r * Ns] = v[r];
  }
}

// every stage of one line (this warp's buffers b0, b1); returns the buffer that holds the result
template <class C>
__device__ __forceinline__ C *warp_fft(C *b0, C *b1, int n, const Stages &st, const C *tw, int inv, int lane)
{
  C *in = b0, *out = b1;
  for (int s = 0; s < st.nst; s++) {
    switch (st.rad[s]) {
      case 2: warp_stage<2, C>(in, out, n, st.Ns[s], st.step[s], st.magic[s], tw, inv, lane); break;
      case 3: warp_stage<3, C>(in, out, n, st.Ns[s], st.step[s], st.magic[s], tw, inv, lane); break;
      case 4: warp_stage<4, C>(in, out, n, st.Ns[s], st.step[s], st.magic[s], tw, inv, lane); break;
      default: warp_stage<5, C>(in, out, n, st.Ns[s], st.step[s], st.magic[s], tw, inv, lane); break;
    }
    __syncwarp();
    C *t = in;
    in = out;
    out = t;
  }
  return in;
}

// ---- compile-time codelets of the warp passes for the common lengths ------------------------------------------
// (the radices' helpers ct_radix, ct_ns are defined with the tile codelets above)

template <int R, int N, int NS, bool INV, class C>
__device__ __forceinline__ void warp_stage_ct(const C *src, C *dst, const C *tw, int lane)
{
  constexpr int nb = N / R, step = N / (NS * R);
#pragma unroll
  for (int j0 = 0; j0 < nb; j0 += 32) {
    const int j = j0 + lane;
    if (nb % 32 != 0 && j >= nb) break;
    C v[R];
#pragma unroll
    for (int r = 0; r < R; r++) v[r] = src[j + r * nb];
    const int q = j / NS, k = j - q * NS;
    if (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; r++) {
        C w = tw[r * k * step];
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dft_small<R, C>(v, INV ? 1 : 0);
    const int idx = q * NS * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) dst[idx + r * NS] = v[r];
  }
}

// the stages from S on, ping-ponging between the warp's two line buffers; returns the buffer with the result
template <int N, int S, bool INV, class C>
struct WarpFftCt {
  static __device__ __forceinline__ C *run(C *in, C *out, const C *tw, int lane)
  {
    constexpr int R = ct_radix(N, S);
    if constexpr (R == 0) {
      return in;
    } else {
      warp_stage_ct<R, N, ct_ns(N, S), INV, C>(in, out, tw, lane);
      __syncwarp();
      return WarpFftCt<N, S + 1, INV, C>::run(out, in, tw, lane);
    }
  }
};

// warp_fft for the lengths with codelets (N = 0: the run-time stages)
template <int N, bool INV, class C>
__device__ __forceinline__ C *warp_fft_n(C *b0, C *b1, int n, const Stages &st, const C *tw, int lane)
{
  if constexpr (N == 0) return warp_fft<C>(b0, b1, n, st, tw, INV ? 1 : 0, lane);
  else return WarpFftCt<N, 0, INV, C>::run(b0, b1, tw, lane);
}

// forward x pass: each warp packs two real lines into one complex line, transforms it and splits it
template <class T, class C, class Src, int NC = 0>
__global__ void __launch_bounds__(32 * kWLines) k_rfft_xw(SrcBatch<Src, C> sb, XGeom g, Stages st,
                                                        const C *__restrict__ tw_g)
{
  const Src &src = sb.src[blockIdx.y];
  C *__restrict__ spec = sb.spec[blockIdx.y];
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int n = NC ? NC : g.F0, ls = n + 1;
  C *tw = sm + 2 * kWLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long L = 2 * ((long)blockIdx.x * kWLines + w);
  if (L >= g.nlines) return;
  C *b0 = sm + w * ls, *b1 = sm + (kWLines + w) * ls;
  const bool two = L + 1 < g.nlines;
  const int y0 = (int)(L % g.F1), z0 = (int)(L / g.F1);
  const int y1 = (int)((L + 1) % g.F1), z1 = (int)((L + 1) / g.F1);
  const bool r0 = y0 < g.ext[1] && z0 < g.ext[2], r1 = two && y1 < g.ext[1] && z1 < g.ext[2];
  // (lines beyond the source's extent are zeros and read no map)
  const typename Src::Line l0 = r0 ? src.line(g, y0, z0) : typename Src::Line{};
  const typename Src::Line l1 = r1 ? src.line(g, y1, z1) : typename Src::Line{};
  for (int x0 = lane; x0 < n; x0 += 32 * kLoadBatch) {
    T a[kLoadBatch], b[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; u++) {
      const int x = x0 + 32 * u;
      a[u] = 0;
      b[u] = 0;
      if (x < g.ext[0]) {
        if (r0) a[u] = src.at(g, l0, x);
        if (r1) b[u] = src.at(g, l1, x);
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; u++)
      if (x0 + 32 * u < n) b0[x0 + 32 * u] = C{a[u], b[u]};
  }
  __syncwarp();
  const C *res = warp_fft_n<NC, false, C>(b0, b1, n, st, tw, lane);
  for (int k = lane; k < g.Fh; k += 32) {
    const C Z = res[k], Zm = res[k == 0 ? 0 : n - k];
    spec[L * g.Fh + k] = C{(T)0.5 * (Z.x + Zm.x), (T)0.5 * (Z.y - Zm.y)};
    if (two) spec[(L + 1) * g.Fh + k] = C{(T)0.5 * (Z.y + Zm.y), (T)0.5 * (Zm.x - Z.x)};
  }
}

// inverse x pass: each warp packs two half-spectrum lines into one complex line and writes the real and
// imaginary parts of its inverse as the outputs of the interior nodes
template <class C, int NC = 0>
__global__ void __launch_bounds__(32 * kWLines) k_irfft_xw(OutBatch<C> ob, XGeom g, Stages st,
                                                         const C *__restrict__ tw_g, double scale, int accumulate)
{
  const C *__restrict__ spec = ob.spec[blockIdx.y];
  double *__restrict__ out = ob.out[blockIdx.y];
  float *__restrict__ out32 = ob.out32[blockIdx.y];
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int n = NC ? NC : g.F0, ls = n + 1;
  C *tw = sm + 2 * kWLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long L = 2 * ((long)blockIdx.x * kWLines + w);
  if (L >= g.nlines) return;
  C *b0 = sm + w * ls, *b1 = sm + (kWLines + w) * ls;
  const bool two = L + 1 < g.nlines;
  for (int k0 = lane; k0 < n; k0 += 32 * kLoadBatch) {
    C A[kLoadBatch], B[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; u++) {
      const int k = k0 + 32 * u;
      const int kk = k < g.Fh ? k : n - k;
      A[u] = C{0, 0};
      B[u] = C{0, 0};
      if (k < n) {
        A[u] = spec[L * g.Fh + kk];
        if (two) B[u] = spec[(L + 1) * g.Fh + kk];
      }
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; u++) {
      const int k = k0 + 32 * u;
      if (k < n)
        b0[k] = k < g.Fh ? C{A[u].x - B[u].y, A[u].y + B[u].x} : C{A[u].x + B[u].y, B[u].x - A[u].y};
    }
  }
  __syncwarp();
  const C *res = warp_fft_n<NC, true, C>(b0, b1, n, st, tw, lane);
  const int nx0 = g.nx[0];
#pragma unroll
  for (int h = 0; h < 2; h++) {
    if (h == 1 && !two) break;
    const int y = (int)((L + h) % g.F1) - g.e[1], z = (int)((L + h) / g.F1) - g.e[2];
    if (y < 0 || y >= g.nx[1] || z < 0 || z >= g.nx[2]) continue;
    const float sc = (float)scale;
    if (out32) {
      float *o = out32 + ((long)z * g.nx[1] + y) * nx0;
      for (int x = lane; x < nx0; x += 32) {
        const C r = res[x + g.e[0]];
        const float v = sc * (h ? r.y : r.x);
        o[x] = accumulate ? o[x] + v : v;
      }
      continue;
    }
    double *o = out + ((long)z * g.nx[1] + y) * nx0;
    for (int x = lane; x < nx0; x += 32) {
      const C r = res[x + g.e[0]];
      const double v = (double)(sc * (h ? r.y : r.x));   // scaled in FP32
      o[x] = accumulate ? o[x] + v : v;
    }
  }
}

// y and z passes: kWLines consecutive x at one outer index, one warp per line
template <class C, int NC, bool INV>
__global__ void __launch_bounds__(32 * kWLines) k_fft_stridedw(PassBatch<C> pb, int X, int n_rt, long es,
                                                             long outer_stride, Stages st,
                                                             const C *__restrict__ tw_g)
{
  const int n = NC ? NC : n_rt;
  const C *in = pb.in[blockIdx.y];
  C *out = pb.out[blockIdx.y];
  const Terms<C> &terms = pb.terms[blockIdx.y];
  extern __shared__ __align__(16) unsigned char smraw[];
  C *sm = reinterpret_cast<C *>(smraw);
  const int ls = n + 1;
  C *tw = sm + 2 * kWLines * ls;
  for (int q = threadIdx.x; q < n; q += blockDim.x) tw[q] = tw_g[q];
  const int xblocks = (X + kWLines - 1) / kWLines;
  const int x0 = (blockIdx.x % xblocks) * kWLines;
  const long base = (long)(blockIdx.x / xblocks) * outer_stride + x0;
  const int nl = min(kWLines, X - x0);
  // loads in groups of kLoadBatch per thread, all issued before any shared-memory store (the pass is bound by
  // global-load latency)
  const int total = kWLines * n;
  for (int q0 = threadIdx.x; q0 < total; q0 += kLoadBatch * blockDim.x) {
    C v[kLoadBatch];
#pragma unroll
    for (int b = 0; b < kLoadBatch; b++) {
      const int q = q0 + b * blockDim.x;
      const int e = q / kWLines, l = q % kWLines;
      v[b] = C{0, 0};
      if (q < total && l < nl) {
        const long idx = base + e * es + l;
        if (terms.n == 0) {
          v[b] = in[idx];
        } else {
          v[b] = cmul(terms.a[0][idx], terms.k[0][idx]);
          for (int t = 1; t < terms.n; t++) v[b] = cadd(v[b], cmul(terms.a[t][idx], terms.k[t][idx]));
        }
      }
    }
#pragma unroll
    for (int b = 0; b < kLoadBatch; b++) {
      const int q = q0 + b * blockDim.x;
      if (q < total) sm[(q % kWLines) * ls + q / kWLines] = v[b];
    }
  }
  __syncthreads();
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // every warp runs its line (beyond nl on stale data, never stored) so that all results sit in the same buffer
  C *b0 = sm + w * ls;
  const C *res = warp_fft_n<NC, INV, C>(b0, sm + (kWLines + w) * ls, n, st, tw, lane);
  const int rofs = (int)(res - b0);   // 0 or kWLines * ls
  __syncthreads();
  for (int q = threadIdx.x; q < kWLines * n; q += blockDim.x) {
    const int e = q / kWLines, l = q % kWLines;
    if (l < nl) out[base + e * es + l] = sm[rofs + l * ls + e];
  }
}

// correlation kernel of coefficient q of a stencil in the real box: coef[k * ncoef + q] added at (-offset_k) mod F
// (offsets that wrap onto the same position add up)
__global__ void k_fft_kernel_box(const short *__restrict__ off3, const double *__restrict__ coef, int L, int ncoef,
                                 int q, double *__restrict__ box, int F0, int F1, int F2)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= L) return;
  const int x = ((-(int)off3[3 * k]) % F0 + F0) % F0;
  const int y = ((-(int)off3[3 * k + 1]) % F1 + F1) % F1;
  const int z = ((-(int)off3[3 * k + 2]) % F2 + F2) % F2;
  atomicAdd(box + ((long)z * F1 + y) * F0 + x, coef[(long)k * ncoef + q]);
}

// the products of `t` as a spectrum (a box without y or z passes to form them in)
template <class C>
__global__ void k_spec_terms(Terms<C> t, C *__restrict__ out, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    C v = cmul(t.a[0][i], t.k[0][i]);
    for (int j = 1; j < t.n; j++) v = cadd(v, cmul(t.a[j][i], t.k[j][i]));
    out[i] = v;
  }
}

__global__ void k_to_float2(const double2 *__restrict__ in, float2 *__restrict__ out, long n)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = make_float2((float)in[i].x, (float)in[i].y);
}

int grid_for(long n) { return (int)std::min<long>((n + 255) / 256, 152L * 16); }

bool smooth(int F)
{
  int m = F;
  for (int r : {2, 3, 5})
    while (m % r == 0) m /= r;
  return m == 1;
}

// radix list of a length (4s first)
bool stages_of(int F, Stages &st)
{
  if (F < 1 || F > kFftMaxN || !smooth(F)) return false;
  int m = F;
  st.nst = 0;
  while (m % 4 == 0) { st.rad[st.nst++] = 4; m /= 4; }
  while (m % 2 == 0) { st.rad[st.nst++] = 2; m /= 2; }
  while (m % 3 == 0) { st.rad[st.nst++] = 3; m /= 3; }
  while (m % 5 == 0) { st.rad[st.nst++] = 5; m /= 5; }
  return st.nst <= 16;
}

Stages stages(const FftAxis &a)
{
  Stages st{};
  st.nst = a.nst;
  int Ns = 1;
  for (int k = 0; k < a.nst; k++) {
    st.rad[k] = a.rad[k];
    st.Ns[k] = Ns;
    st.step[k] = a.n / (Ns * a.rad[k]);
    st.magic[k] = Ns == 1 ? 0u : (unsigned)((((unsigned long long)1 << 32) + Ns - 1) / Ns);
    Ns *= a.rad[k];
  }
  return st;
}

size_t wtile_smem(int n) { return sizeof(float2) * (2 * (size_t)kWLines * (n + 1) + n); }

// f(std::integral_constant<int, N>) for the lengths with codelets (the y/z lengths 96, 128, 256 and the x lengths
// 150, 180, 320 of the 96^3, 128^3 and 256^3 workloads), f(std::integral_constant<int, 0>) otherwise
template <class F>
void with_length(int n, F &&f)
{
  switch (n) {
    case 96: f(std::integral_constant<int, 96>{}); return;
    case 128: f(std::integral_constant<int, 128>{}); return;
    case 150: f(std::integral_constant<int, 150>{}); return;
    case 180: f(std::integral_constant<int, 180>{}); return;
    case 256: f(std::integral_constant<int, 256>{}); return;
    case 320: f(std::integral_constant<int, 320>{}); return;
    default: f(std::integral_constant<int, 0>{}); return;
  }
}

template <class C>
size_t tile_smem(int n)
{
  return sizeof(C) * (2 * (size_t)kFftLines * (n + 1) + n);
}

// the block-tile codelet length for C (the FP64 passes; the FP32 ones run one warp per line)
template <class C>
constexpr int tile_codelet(int n)
{
  return std::is_same<C, double2>::value ? n : 0;
}

template <class T, class C>
void set_smem_limits(const FftPlan &p)
{
  const int sx = (int)tile_smem<C>(p.F[0]);
  with_length(p.F[0], [&](auto L) {
    constexpr int NC = tile_codelet<C>(decltype(L)::value);
    cudaFuncSetAttribute(k_rfft_x<T, C, BoxSrc<T>, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, sx);
    cudaFuncSetAttribute(k_rfft_x<T, C, MappedSrc<T>, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, sx);
    cudaFuncSetAttribute(k_irfft_x<C, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, sx);
  });
  const int ss = (int)std::max(tile_smem<C>(p.F[1]), tile_smem<C>(p.F[2]));
  for (int d = 1; d <= 2; d++)
    with_length(p.F[d], [&](auto L) {
      constexpr int NC = tile_codelet<C>(decltype(L)::value);
      cudaFuncSetAttribute(k_fft_strided<C, NC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, ss);
      cudaFuncSetAttribute(k_fft_strided<C, NC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, ss);
    });
  if (std::is_same<C, float2>::value) {
    const int wx = (int)wtile_smem(p.F[0]), ws = (int)std::max(wtile_smem(p.F[1]), wtile_smem(p.F[2]));
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = decltype(L)::value;
      cudaFuncSetAttribute(k_rfft_xw<float, float2, BoxSrc<float>, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           wx);
      cudaFuncSetAttribute(k_rfft_xw<float, float2, MappedSrc<float>, NC>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, wx);
      cudaFuncSetAttribute(k_irfft_xw<float2, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, wx);
    });
    for (int d = 1; d <= 2; d++)
      with_length(p.F[d], [&](auto L) {
        constexpr int NC = decltype(L)::value;
        cudaFuncSetAttribute(k_fft_stridedw<float2, NC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, ws);
        cudaFuncSetAttribute(k_fft_stridedw<float2, NC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, ws);
      });
  }
}

XGeom xgeom(const FftPlan &p)
{
  XGeom g{};
  g.F0 = p.F[0];
  g.F1 = p.F[1];
  g.Fh = p.Fh;
  g.nlines = (long)p.F[1] * p.F[2];
  for (int d = 0; d < 3; d++) {
    g.off[d] = p.off[d];
    g.ext[d] = p.ext[d];
    g.e[d] = p.h[d] - p.off[d];
    g.nx[d] = p.nx[d];
  }
  return g;
}

// Optional timing of every FP32 y/z pass launch (the solves' leading kernel): a CUDA event pair around each launch
// on its own stream and the launch's algorithmic bytes (per transform the half spectrum written once and read once,
// or the two operands of each spectral product read); collected and reset by pass_timer_collect.
struct PassTimer {
  bool on = false;
  std::vector<cudaEvent_t> ev;   // begin, end of each launch
  std::vector<double> bytes;
  std::vector<int> fields;
};
PassTimer g_pass_timer;

// one y (d = 1) or z (d = 2) pass of nb transforms of the plan in one launch: FP32 one warp per line, FP64 the
// block tile
template <class C>
void strided_pass_batch(const PassBatch<C> &pb, int nb, const FftPlan &p, int d, bool inverse, const C *tw,
                        cudaStream_t s)
{
  const int X = p.Fh, n = p.F[d];
  const long es = d == 1 ? (long)X : (long)X * p.F[1];
  const long outer = d == 1 ? (long)X * p.F[1] : (long)X;   // axis 1: outer index z; axis 2: outer index y
  const long nouter = d == 1 ? p.F[2] : p.F[1];
  if constexpr (std::is_same<C, float2>::value) {
    const int xb = (X + kWLines - 1) / kWLines;
    const bool timed = g_pass_timer.on;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (timed) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, s);
    }
    const dim3 grid((unsigned)(xb * nouter), (unsigned)nb);
    with_length(n, [&](auto L) {
      constexpr int NC = decltype(L)::value;
      if (inverse)
        k_fft_stridedw<float2, NC, true><<<grid, 32 * kWLines, wtile_smem(n), s>>>(pb, X, n, es, outer,
                                                                                   stages(p.ax[d]), tw);
      else
        k_fft_stridedw<float2, NC, false><<<grid, 32 * kWLines, wtile_smem(n), s>>>(pb, X, n, es, outer,
                                                                                    stages(p.ax[d]), tw);
    });
    if (timed) {
      cudaEventRecord(e1, s);
      double units = 0.0;   // half spectra moved
      for (int b = 0; b < nb; b++) units += 1.0 + (pb.terms[b].n > 0 ? 2.0 * pb.terms[b].n : 1.0);
      g_pass_timer.ev.push_back(e0);
      g_pass_timer.ev.push_back(e1);
      g_pass_timer.bytes.push_back(units * (double)p.NH * sizeof(float2));
      g_pass_timer.fields.push_back(nb);
    }
  } else {
    const int xblocks = (X + kFftLines - 1) / kFftLines;
    const dim3 grid((unsigned)(xblocks * nouter), (unsigned)nb);
    with_length(n, [&](auto L) {
      constexpr int NC = tile_codelet<C>(decltype(L)::value);
      if (inverse)
        k_fft_strided<C, NC, true><<<grid, kFftThreads, tile_smem<C>(n), s>>>(pb, X, n, es, outer, stages(p.ax[d]),
                                                                             tw);
      else
        k_fft_strided<C, NC, false><<<grid, kFftThreads, tile_smem<C>(n), s>>>(pb, X, n, es, outer, stages(p.ax[d]),
                                                                              tw);
    });
  }
}

// one y (d = 1) or z (d = 2) pass over the half-spectrum box
template <class C>
void strided_pass(const C *in, C *out, const Terms<C> &terms, const FftPlan &p, int d, bool inverse, const C *tw,
                  cudaStream_t s)
{
  PassBatch<C> pb{};
  pb.in[0] = in;
  pb.out[0] = out;
  pb.terms[0] = terms;
  strided_pass_batch<C>(pb, 1, p, d, inverse, tw, s);
}

template <class T, class C, class Src>
void rfft_forward_impl(const Src &src, bool padded, C *spec, const FftPlan &p, const C *const *tw, cudaStream_t s)
{
  XGeom g = xgeom(p);
  if (!padded)   // a real box [F2][F1][F0]
    for (int d = 0; d < 3; d++) {
      g.off[d] = 0;
      g.ext[d] = p.F[d];
    }
  const long npairs = (g.nlines + 1) / 2;
  if constexpr (std::is_same<C, float2>::value) {
    SrcBatch<Src, C> sb{};
    sb.src[0] = src;
    sb.spec[0] = spec;
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = decltype(L)::value;
      k_rfft_xw<T, C, Src, NC><<<(unsigned)((npairs + kWLines - 1) / kWLines), 32 * kWLines, wtile_smem(p.F[0]), s>>>(
          sb, g, stages(p.ax[0]), tw[0]);
    });
  } else {
    SrcBatch<Src, C> sb{};
    sb.src[0] = src;
    sb.spec[0] = spec;
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = tile_codelet<C>(decltype(L)::value);
      k_rfft_x<T, C, Src, NC><<<(unsigned)((npairs + kFftLines - 1) / kFftLines), kFftThreads, tile_smem<C>(p.F[0]),
                                s>>>(sb, g, stages(p.ax[0]), tw[0]);
    });
  }
  const Terms<C> none{};
  for (int d = 1; d <= 2; d++)
    if (p.F[d] > 1) strided_pass<C>(spec, spec, none, p, d, false, tw[d], s);
}

// inverse of the products in `terms`, formed by the first inverse pass into `spec` (the work box)
template <class C>
void rfft_inverse_impl(const Terms<C> &terms, C *spec, const FftPlan &p, double scale, double *out, float *out32,
                       bool accumulate, const C *const *tw, cudaStream_t s)
{
  const Terms<C> none{};
  bool pending = true;   // products not formed yet
  for (int d = 2; d >= 1; d--) {
    if (p.F[d] == 1) continue;
    strided_pass<C>(spec, spec, pending ? terms : none, p, d, true, tw[d], s);
    pending = false;
  }
  if (pending) k_spec_terms<C><<<grid_for(p.NH), 256, 0, s>>>(terms, spec, p.NH);
  const XGeom g = xgeom(p);
  const long npairs = (g.nlines + 1) / 2;
  if constexpr (std::is_same<C, float2>::value) {
    OutBatch<C> ob{};
    ob.spec[0] = spec;
    ob.out[0] = out;
    ob.out32[0] = out32;
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = decltype(L)::value;
      k_irfft_xw<C, NC><<<(unsigned)((npairs + kWLines - 1) / kWLines), 32 * kWLines, wtile_smem(p.F[0]), s>>>(
          ob, g, stages(p.ax[0]), tw[0], scale, accumulate ? 1 : 0);
    });
  } else {
    OutBatch<C> ob{};
    ob.spec[0] = spec;
    ob.out[0] = out;
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = tile_codelet<C>(decltype(L)::value);
      k_irfft_x<C, NC><<<(unsigned)((npairs + kFftLines - 1) / kFftLines), kFftThreads, tile_smem<C>(p.F[0]), s>>>(
          ob, g, stages(p.ax[0]), tw[0], scale, accumulate ? 1 : 0);
    });
  }
}

// nb forward transforms of mapped channels in one launch per pass
template <class T, class C>
void rfft_forward_mapped_batch_impl(const MapSrc *m, int nb, C *const *spec, const FftPlan &p, const C *const *tw,
                                    cudaStream_t s)
{
  const XGeom g = xgeom(p);
  const long npairs = (g.nlines + 1) / 2;
  SrcBatch<MappedSrc<T>, C> sb{};
  PassBatch<C> pb{};
  for (int b = 0; b < nb; b++) {
    sb.src[b] = MappedSrc<T>{m[b]};
    sb.spec[b] = spec[b];
    pb.in[b] = spec[b];
    pb.out[b] = spec[b];
  }
  if constexpr (std::is_same<C, float2>::value)
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = decltype(L)::value;
      k_rfft_xw<T, C, MappedSrc<T>, NC>
          <<<dim3((unsigned)((npairs + kWLines - 1) / kWLines), (unsigned)nb), 32 * kWLines, wtile_smem(p.F[0]), s>>>(
              sb, g, stages(p.ax[0]), tw[0]);
    });
  else
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = tile_codelet<C>(decltype(L)::value);
      k_rfft_x<T, C, MappedSrc<T>, NC><<<dim3((unsigned)((npairs + kFftLines - 1) / kFftLines), (unsigned)nb),
                                         kFftThreads, tile_smem<C>(p.F[0]), s>>>(sb, g, stages(p.ax[0]), tw[0]);
    });
  for (int d = 1; d <= 2; d++)
    if (p.F[d] > 1) strided_pass_batch<C>(pb, nb, p, d, false, tw[d], s);
}

// nb inverse transforms, output b the inverse of a * k[b] (formed by the first inverse pass in work[b])
template <class C>
void rfft_inverse_batch_impl(const C *a, const C *const *k, int nb, C *const *work, const FftPlan &p, double scale,
                             double *const *out, float *const *out32, bool accumulate, const C *const *tw,
                             cudaStream_t s)
{
  PassBatch<C> pb{}, plain{};
  OutBatch<C> ob{};
  for (int b = 0; b < nb; b++) {
    pb.in[b] = plain.in[b] = work[b];
    pb.out[b] = plain.out[b] = work[b];
    pb.terms[b].a[0] = a;
    pb.terms[b].k[0] = k[b];
    pb.terms[b].n = 1;
    ob.spec[b] = work[b];
    ob.out[b] = out ? out[b] : nullptr;
    ob.out32[b] = out32 ? out32[b] : nullptr;
  }
  bool pending = true;
  for (int d = 2; d >= 1; d--) {
    if (p.F[d] == 1) continue;
    strided_pass_batch<C>(pending ? pb : plain, nb, p, d, true, tw[d], s);
    pending = false;
  }
  if (pending)
    for (int b = 0; b < nb; b++) k_spec_terms<C><<<grid_for(p.NH), 256, 0, s>>>(pb.terms[b], work[b], p.NH);
  const XGeom g = xgeom(p);
  const long npairs = (g.nlines + 1) / 2;
  if constexpr (std::is_same<C, float2>::value)
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = decltype(L)::value;
      k_irfft_xw<C, NC><<<dim3((unsigned)((npairs + kWLines - 1) / kWLines), (unsigned)nb), 32 * kWLines,
                          wtile_smem(p.F[0]), s>>>(ob, g, stages(p.ax[0]), tw[0], scale, accumulate ? 1 : 0);
    });
  else
    with_length(p.F[0], [&](auto L) {
      constexpr int NC = tile_codelet<C>(decltype(L)::value);
      k_irfft_x<C, NC><<<dim3((unsigned)((npairs + kFftLines - 1) / kFftLines), (unsigned)nb), kFftThreads,
                         tile_smem<C>(p.F[0]), s>>>(ob, g, stages(p.ax[0]), tw[0], scale, accumulate ? 1 : 0);
    });
}

}  // namespace

bool fft_make_plan(FftPlan &p, const int P[3], const int nx[3], const int h[3], const int periodic[3], int ndim,
                   cudaStream_t s)
{
  p.NR = 1;
  for (int d = 0; d < 3; d++) {
    FftAxis &a = p.ax[d];
    p.P[d] = d < ndim ? P[d] : 1;
    p.nx[d] = d < ndim ? nx[d] : 1;
    p.h[d] = d < ndim ? h[d] : 0;
    if (d >= ndim) {
      p.F[d] = 1;
      p.off[d] = 0;
      p.ext[d] = 1;
      a.n = 1;
      a.nst = 0;
      continue;
    }
    Stages st{};
    if (periodic[d] && stages_of(nx[d], st)) {   // the period itself: no padding
      p.F[d] = nx[d];
      p.off[d] = h[d];
      p.ext[d] = nx[d];
    } else {
      int F = P[d];
      while (F <= kFftMaxN && !smooth(F)) F++;
      if (!stages_of(F, st)) return false;
      p.F[d] = F;
      p.off[d] = 0;
      p.ext[d] = P[d];
    }
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
    p.NR *= p.F[d];
  }
  p.Fh = p.F[0] / 2 + 1;
  p.NH = (long)p.Fh * p.F[1] * p.F[2];
  set_smem_limits<double, double2>(p);
  set_smem_limits<float, float2>(p);
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

void rfft_forward(const double *pad, double2 *spec, const FftPlan &p, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  rfft_forward_impl<double, double2>(BoxSrc<double>{pad, p.P[0], (long)p.P[0] * p.P[1]}, true, spec, p, tw, s);
}

void rfft_forward(const float *pad, float2 *spec, const FftPlan &p, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  rfft_forward_impl<float, float2>(BoxSrc<float>{pad, p.P[0], (long)p.P[0] * p.P[1]}, true, spec, p, tw, s);
}

void rfft_forward_mapped(const MapSrc &m, double2 *spec, const FftPlan &p, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  rfft_forward_impl<double, double2>(MappedSrc<double>{m}, true, spec, p, tw, s);
}

void rfft_forward_mapped(const MapSrc &m, float2 *spec, const FftPlan &p, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  rfft_forward_impl<float, float2>(MappedSrc<float>{m}, true, spec, p, tw, s);
}

void rfft_forward_box(const double *box, double2 *spec, const FftPlan &p, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  rfft_forward_impl<double, double2>(BoxSrc<double>{box, p.F[0], (long)p.F[0] * p.F[1]}, false, spec, p, tw, s);
}

template <class C>
Terms<C> make_terms(const C *const *a, const C *const *k, int n)
{
  Terms<C> t{};
  t.n = n;
  for (int j = 0; j < n; j++) {
    t.a[j] = a[j];
    t.k[j] = k[j];
  }
  return t;
}

void rfft_inverse_products(const double2 *const *a, const double2 *const *k, int nterms, double2 *work,
                           const FftPlan &p, double scale, double *out, bool accumulate, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  rfft_inverse_impl<double2>(make_terms(a, k, nterms), work, p, scale, out, nullptr, accumulate, tw, s);
}

void rfft_inverse_products(const float2 *const *a, const float2 *const *k, int nterms, float2 *work,
                           const FftPlan &p, double scale, double *out, bool accumulate, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  rfft_inverse_impl<float2>(make_terms(a, k, nterms), work, p, scale, out, nullptr, accumulate, tw, s);
}

void rfft_inverse_products(const float2 *const *a, const float2 *const *k, int nterms, float2 *work,
                           const FftPlan &p, double scale, float *out, bool accumulate, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  rfft_inverse_impl<float2>(make_terms(a, k, nterms), work, p, scale, nullptr, out, accumulate, tw, s);
}

int fft_max_terms() { return kMaxTerms; }
int fft_max_batch() { return kMaxBatch; }

void rfft_forward_mapped_batch(const MapSrc *m, int nb, float2 *const *spec, const FftPlan &p, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  for (int b0 = 0; b0 < nb; b0 += kMaxBatch)
    rfft_forward_mapped_batch_impl<float, float2>(m + b0, std::min(kMaxBatch, nb - b0), spec + b0, p, tw, s);
}

void rfft_forward_mapped_batch(const MapSrc *m, int nb, double2 *const *spec, const FftPlan &p, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  for (int b0 = 0; b0 < nb; b0 += kMaxBatch)
    rfft_forward_mapped_batch_impl<double, double2>(m + b0, std::min(kMaxBatch, nb - b0), spec + b0, p, tw, s);
}

void rfft_inverse_batch(const float2 *a, const float2 *const *k, int nb, float2 *const *work, const FftPlan &p,
                        double scale, double *const *out, bool accumulate, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  for (int b0 = 0; b0 < nb; b0 += kMaxBatch)
    rfft_inverse_batch_impl<float2>(a, k + b0, std::min(kMaxBatch, nb - b0), work + b0, p, scale, out + b0, nullptr,
                                    accumulate, tw, s);
}

void rfft_inverse_batch(const float2 *a, const float2 *const *k, int nb, float2 *const *work, const FftPlan &p,
                        double scale, float *const *out, bool accumulate, cudaStream_t s)
{
  const float2 *tw[3] = {p.ax[0].d_tw32, p.ax[1].d_tw32, p.ax[2].d_tw32};
  for (int b0 = 0; b0 < nb; b0 += kMaxBatch)
    rfft_inverse_batch_impl<float2>(a, k + b0, std::min(kMaxBatch, nb - b0), work + b0, p, scale, nullptr, out + b0,
                                    accumulate, tw, s);
}

void rfft_inverse_batch(const double2 *a, const double2 *const *k, int nb, double2 *const *work, const FftPlan &p,
                        double scale, double *const *out, bool accumulate, cudaStream_t s)
{
  const double2 *tw[3] = {p.ax[0].d_tw, p.ax[1].d_tw, p.ax[2].d_tw};
  for (int b0 = 0; b0 < nb; b0 += kMaxBatch)
    rfft_inverse_batch_impl<double2>(a, k + b0, std::min(kMaxBatch, nb - b0), work + b0, p, scale, out + b0, nullptr,
                                     accumulate, tw, s);
}

void fft_pass(double2 *spec, const FftPlan &p, int d, bool inverse, cudaStream_t s)
{
  const Terms<double2> none{};
  strided_pass<double2>(spec, spec, none, p, d, inverse, p.ax[d].d_tw, s);
}

void fft_pass(float2 *spec, const FftPlan &p, int d, bool inverse, cudaStream_t s)
{
  const Terms<float2> none{};
  strided_pass<float2>(spec, spec, none, p, d, inverse, p.ax[d].d_tw32, s);
}

void launch_fft_kernel_box(const short *off3, const double *coef, int L, int ncoef, int q, double *box,
                           const FftPlan &p, cudaStream_t s)
{
  cudaMemsetAsync(box, 0, sizeof(double) * p.NR, s);
  if (L > 0) k_fft_kernel_box<<<(L + 255) / 256, 256, 0, s>>>(off3, coef, L, ncoef, q, box, p.F[0], p.F[1], p.F[2]);
}

void launch_to_float2(const double2 *in, float2 *out, long n, cudaStream_t s)
{
  k_to_float2<<<grid_for(n), 256, 0, s>>>(in, out, n);
}

void pass_timer_enable(bool on)
{
  g_pass_timer.on = on;
}

void pass_timer_collect(long *launches, double *ms_total, double *bytes_total, long *fields_total)
{
  double ms = 0.0, bytes = 0.0;
  long fields = 0;
  const size_t nl = g_pass_timer.bytes.size();
  for (size_t i = 0; i < nl; i++) {
    float t = 0.f;
    cudaEventSynchronize(g_pass_timer.ev[2 * i + 1]);
    cudaEventElapsedTime(&t, g_pass_timer.ev[2 * i], g_pass_timer.ev[2 * i + 1]);
    ms += t;
    bytes += g_pass_timer.bytes[i];
    fields += g_pass_timer.fields[i];
  }
  for (cudaEvent_t e : g_pass_timer.ev) cudaEventDestroy(e);
  g_pass_timer.ev.clear();
  g_pass_timer.bytes.clear();
  g_pass_timer.fields.clear();
  if (launches) *launches = (long)nl;
  if (ms_total) *ms_total = ms;
  if (bytes_total) *bytes_total = bytes;
  if (fields_total) *fields_total = fields;
}

}  // namespace tgpu
