// External fields of planar walls on the GPU (set-up): one thread per node.
// The wall forms, sides, roughness patches and clipping are described with
// tgpu_wall_field in include/tramonto_gpu.h.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "../../include/tramonto_gpu.h"

namespace {

constexpr double kPi = 3.141592653589793238462643383279502884197;
constexpr int kMaxPatches = 4096;

struct DevWall {
  int form, side;
  double position, eps, sigma, cut, pattern;
  int py, pz;
  const double *h;       // device [py][pz] or nullptr
};

struct DevField {
  int ndim, nx[3];
  double esize[3];
  int nwalls;
  DevWall w[2];
  double vext_max;
};

__device__ double wall_shape(const DevWall &w, double d)
{
  const double s = w.sigma / d;
  const double s3 = s * s * s;
  if (w.form == TGPU_WALL_LJ123) {
    const double s6 = s3 * s3;
    return w.eps * (s6 * s6 - s3);
  }
  if (d > w.cut) return 0.0;
  const double c = w.sigma / w.cut, c3 = c * c * c, c9 = c3 * c3 * c3, s9 = s3 * s3 * s3;
  return w.eps * (2.0 * kPi / 3.0) * w.sigma * w.sigma * w.sigma * ((2.0 / 15.0) * (s9 - c9) - (s3 - c3));
}

__global__ void k_wall_field(DevField f, long N, double *out)
{
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
    const int ix = (int)(i % f.nx[0]);
    const long r = i / f.nx[0];
    const int iy = f.ndim >= 2 ? (int)(r % f.nx[1]) : 0;
    const int iz = f.ndim == 3 ? (int)(r / f.nx[1]) : 0;
    const double x = ix * f.esize[0];
    double v = 0.0;
    bool clip = false;
    for (int k = 0; k < f.nwalls; k++) {
      const DevWall &w = f.w[k];
      double h = 0.0;
      if (w.h) {
        const int jy = f.ndim >= 2 ? (int)(((long)iy * w.py) / f.nx[1]) : 0;
        const int jz = f.ndim == 3 ? (int)(((long)iz * w.pz) / f.nx[2]) : 0;
        h = w.h[(long)jy * w.pz + jz];
      }
      const double d = w.side == 0 ? x - (w.position + h) : (w.position - h) - x;
      if (!(d > 0.0)) {
        clip = true;
        continue;
      }
      double e = 1.0;
      if (f.ndim >= 2 && w.pattern != 0.0)
        e = 1.0 + w.pattern * cos(2.0 * kPi * (iy * f.esize[1]) / (f.nx[1] * f.esize[1]));
      v += e * wall_shape(w, d);
    }
    out[i] = (clip || !(v < f.vext_max)) ? f.vext_max : v;
  }
}

int wall_field(const tgpu_wall_field *f, double *d_out)
{
  if (!f || !d_out || f->ndim < 1 || f->ndim > 3 || f->nwalls < 1 || f->nwalls > 2) return TGPU_ERR_ARG;
  DevField df{};
  df.ndim = f->ndim;
  long N = 1;
  for (int d = 0; d < 3; d++) {
    df.nx[d] = d < f->ndim ? f->nx[d] : 1;
    df.esize[d] = d < f->ndim ? f->esize[d] : 0.0;
    if (df.nx[d] < 1) return TGPU_ERR_ARG;
    N *= df.nx[d];
  }
  df.nwalls = f->nwalls;
  df.vext_max = f->vext_max;
  double *dh[2] = {nullptr, nullptr};
  int st = TGPU_OK;
  for (int k = 0; k < f->nwalls && st == TGPU_OK; k++) {
    const tgpu_wall &w = f->wall[k];
    if ((w.form != TGPU_WALL_LJ93_CS && w.form != TGPU_WALL_LJ123) || (w.side != 0 && w.side != 1) ||
        !(w.sigma > 0.0) || (w.form == TGPU_WALL_LJ93_CS && !(w.cut > 0.0))) {
      st = TGPU_ERR_ARG;
      break;
    }
    DevWall &o = df.w[k];
    o.form = w.form;
    o.side = w.side;
    o.position = w.position;
    o.eps = w.eps;
    o.sigma = w.sigma;
    o.cut = w.cut;
    o.pattern = w.pattern;
    o.py = w.heights ? w.patches[0] : 0;
    o.pz = w.heights ? w.patches[1] : 0;
    o.h = nullptr;
    if (w.heights) {
      if (o.py < 1 || o.pz < 1 || (long)o.py * o.pz > kMaxPatches * kMaxPatches) {
        st = TGPU_ERR_ARG;
        break;
      }
      const size_t n = (size_t)o.py * o.pz;
      if (cudaMalloc(&dh[k], n * sizeof(double)) != cudaSuccess ||
          cudaMemcpy(dh[k], w.heights, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
        st = TGPU_ERR_CUDA;
        break;
      }
      o.h = dh[k];
    }
  }
  if (st == TGPU_OK) {
    k_wall_field<<<(unsigned)std::min<long>((N + 255) / 256, 1L << 16), 256>>>(df, N, d_out);
    if (cudaDeviceSynchronize() != cudaSuccess || cudaGetLastError() != cudaSuccess) st = TGPU_ERR_CUDA;
  }
  for (double *p : dh)
    if (p) cudaFree(p);
  return st;
}

}  // namespace

extern "C" {

int tgpu_wall_field_device(const tgpu_wall_field *f, double *d_out)
{
  return wall_field(f, d_out);
}

int tgpu_wall_field_host(const tgpu_wall_field *f, double *out)
{
  if (!f || !out || f->ndim < 1 || f->ndim > 3) return TGPU_ERR_ARG;
  long N = 1;
  for (int d = 0; d < f->ndim; d++) N *= f->nx[d] > 0 ? f->nx[d] : 0;
  if (N <= 0) return TGPU_ERR_ARG;
  double *d = nullptr;
  if (cudaMalloc(&d, N * sizeof(double)) != cudaSuccess) return TGPU_ERR_CUDA;
  int st = wall_field(f, d);
  if (st == TGPU_OK && cudaMemcpy(out, d, N * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    st = TGPU_ERR_CUDA;
  cudaFree(d);
  return st;
}

}  // extern "C"
