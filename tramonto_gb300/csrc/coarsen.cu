// Quadrature zones and mesh coarsening on the device.
//
// Zones (calc_stencils, src/dft_stencil.c:96-109, 229-236): a node of zone z >= 1 takes its stencil sums
// from zone z's tables (elements 2^z times the mesh's, offsets in fine-node units).  The sums of every
// zone are formed over the whole mesh and each node keeps its own zone's (zone_merge); the coarse tables
// are short, so the extra passes cost a fraction of the zone-0 pass.
//
// Coarsened nodes (set_mesh_coarsen_flag, src/dft_mesh.c:2788-2850): every unknown of a node off its
// zone's coarse lattice has the row fac (x_c - sum_k a_k x_k) over the two neighbours along one axis
// (load_coarse_node_Ndim / locate_neighbor_unks, src/dft_fill_coarse.c:66-123; with two zones a
// coarsened neighbour is replaced by its own neighbours), fac = 1 on density rows and -1 elsewhere.
// Term columns are node indices, or -1 / -3 for the bulk beyond the low / high IN_BULK boundary
// (constant_boundary, src/dft_utils.c:89-110: the unknown's bulk value, bulk[u] / bulk[nunk + u]).
// With L1D_bc, nodes near the two ends along one dimension have the rows x_c - x_line with fac 1 on every
// unknown (load_coarse_node_1dim, src/dft_fill_coarse.c:37-64): kind 1.
//
// The Newton step is solved on the other nodes only: the coarsened nodes' values follow from the rest
// through the prolongation x_c = sum_f P_cf x_f (+ bulk terms), which satisfies every averaged row
// exactly; prolong() applies it to whole rows of unknowns, prolong_t() its transpose (the adjoint).
#include "tgpu_internal.h"

namespace tgpu {

namespace {

__global__ void k_zone_merge(const double *__restrict__ src, double *__restrict__ dst, int nrows, long N,
                             const int *__restrict__ zone, int z)
{
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N || zone[i] != z) return;
  for (int r = 0; r < nrows; r++) dst[(long)r * N + i] = src[(long)r * N + i];
}

__global__ void k_zone_mask(double *__restrict__ buf, int nrows, long N, const int *__restrict__ zone, int z)
{
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= N || zone[i] == z) return;
  for (int r = 0; r < nrows; r++) buf[(long)r * N + i] = 0.0;
}

__device__ __forceinline__ double row_fac(int u, int first_rho, int ncomp, signed char kind)
{
  return (kind || (u >= first_rho && u < first_rho + ncomp)) ? 1.0 : -1.0;
}

// the bulk value of unknown u beyond the boundary a negative column names
__device__ __forceinline__ double bulk_value(const double *bulk, long j, int u, int nunk)
{
  return bulk ? bulk[u + (j == kSentBulkHi ? nunk : 0)] : 0.0;
}

// one thread per (coarsened node, unknown): out[u][c] = fac (in[u][c] - sum_k a_k in[u][col_k])
__global__ void k_coarse_rows(const double *__restrict__ in, double *__restrict__ out, int nunk, int first_rho,
                              int ncomp, long N, int ncoarse, const int *__restrict__ cnode,
                              const int *__restrict__ ptr, const long *__restrict__ col,
                              const double *__restrict__ a, const signed char *__restrict__ kind,
                              const double *__restrict__ bulk)
{
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)ncoarse * nunk) return;
  const int k = (int)(t % ncoarse), u = (int)(t / ncoarse);
  const long c = cnode[k];
  const double *row = in + (long)u * N;
  double s = row[c];
  for (int e = ptr[k]; e < ptr[k + 1]; e++) {
    const long j = col[e];
    const double v = j >= 0 ? row[j] : bulk_value(bulk, j, u, nunk);
    s -= a[e] * v;
  }
  out[(long)u * N + c] = row_fac(u, first_rho, ncomp, kind[k]) * s;
}

// transpose of the averaged rows: out[u][c] += fac w[u][c]; out[u][col_k] -= fac a_k w[u][c]
__global__ void k_coarse_rows_t(const double *__restrict__ w, double *__restrict__ out, int nunk, int first_rho,
                                int ncomp, long N, int ncoarse, const int *__restrict__ cnode,
                                const int *__restrict__ ptr, const long *__restrict__ col,
                                const double *__restrict__ a, const signed char *__restrict__ kind)
{
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)ncoarse * nunk) return;
  const int k = (int)(t % ncoarse), u = (int)(t / ncoarse);
  const long c = cnode[k];
  const double fw = row_fac(u, first_rho, ncomp, kind[k]) * w[(long)u * N + c];
  atomicAdd(out + (long)u * N + c, fw);
  for (int e = ptr[k]; e < ptr[k + 1]; e++) {
    const long j = col[e];
    if (j >= 0) atomicAdd(out + (long)u * N + j, -a[e] * fw);
  }
}

// prolongation of rows row0 .. row0+nrows-1: vec[r][c] = sum_e p_e vec[r][col_e] (+ p_e times the bulk
// value of unknown row0+r at a negative column)
__global__ void k_prolong(double *__restrict__ vec, int row0, int nrows, int nunk, long N, int ncoarse,
                          const int *__restrict__ cnode, const int *__restrict__ ptr, const long *__restrict__ col,
                          const double *__restrict__ p, const double *__restrict__ bulk)
{
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)ncoarse * nrows) return;
  const int k = (int)(t % ncoarse), r = (int)(t / ncoarse);
  double *row = vec + (long)(row0 + r) * N;
  double s = 0.0;
  for (int e = ptr[k]; e < ptr[k + 1]; e++) {
    const long j = col[e];
    s += p[e] * (j >= 0 ? row[j] : bulk_value(bulk, j, row0 + r, nunk));
  }
  row[cnode[k]] = s;
}

// transpose of the prolongation: vec[r][col_e] += p_e vec[r][c], then vec[r][c] = 0 (columns are never
// coarsened nodes, so the adds and the reads do not meet)
__global__ void k_prolong_t(double *__restrict__ vec, int row0, int nrows, long N, int ncoarse,
                            const int *__restrict__ cnode, const int *__restrict__ ptr, const long *__restrict__ col,
                            const double *__restrict__ p)
{
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)ncoarse * nrows) return;
  const int k = (int)(t % ncoarse), r = (int)(t / ncoarse);
  double *row = vec + (long)(row0 + r) * N;
  const double v = row[cnode[k]];
  for (int e = ptr[k]; e < ptr[k + 1]; e++) {
    const long j = col[e];
    if (j >= 0 && v != 0.0) atomicAdd(row + j, p[e] * v);
  }
  row[cnode[k]] = 0.0;
}

__global__ void k_zero_nodes(double *__restrict__ vec, int nrows, long N, int ncoarse, const int *__restrict__ cnode)
{
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)ncoarse * nrows) return;
  const int k = (int)(t % ncoarse), r = (int)(t / ncoarse);
  vec[(long)r * N + cnode[k]] = 0.0;
}

inline int nblk(long n) { return (int)((n + 255) / 256); }

}  // namespace

void launch_zone_merge(const double *src, double *dst, int nrows, long N, const int *zone, int z, cudaStream_t s)
{
  if (N > 0) k_zone_merge<<<nblk(N), 256, 0, s>>>(src, dst, nrows, N, zone, z);
}

void launch_zone_mask(double *buf, int nrows, long N, const int *zone, int z, cudaStream_t s)
{
  if (N > 0) k_zone_mask<<<nblk(N), 256, 0, s>>>(buf, nrows, N, zone, z);
}

void launch_coarse_rows(const double *in, double *out, int nunk, int first_rho, int ncomp, long N,
                        const CoarseRows &cr, const double *bulk, cudaStream_t s)
{
  const long n = (long)cr.ncoarse * nunk;
  if (n > 0)
    k_coarse_rows<<<nblk(n), 256, 0, s>>>(in, out, nunk, first_rho, ncomp, N, cr.ncoarse, cr.d_node, cr.d_rptr,
                                          cr.d_rcol, cr.d_ra, cr.d_kind, bulk);
}

void launch_coarse_rows_t(const double *w, double *out, int nunk, int first_rho, int ncomp, long N,
                          const CoarseRows &cr, cudaStream_t s)
{
  const long n = (long)cr.ncoarse * nunk;
  if (n > 0)
    k_coarse_rows_t<<<nblk(n), 256, 0, s>>>(w, out, nunk, first_rho, ncomp, N, cr.ncoarse, cr.d_node, cr.d_rptr,
                                            cr.d_rcol, cr.d_ra, cr.d_kind);
}

void launch_prolong(double *vec, int row0, int nrows, int nunk, long N, const CoarseRows &cr, const double *bulk,
                    cudaStream_t s)
{
  const long n = (long)cr.ncoarse * nrows;
  if (n > 0)
    k_prolong<<<nblk(n), 256, 0, s>>>(vec, row0, nrows, nunk, N, cr.ncoarse, cr.d_node, cr.d_pptr, cr.d_pcol,
                                      cr.d_pw, bulk);
}

void launch_prolong_t(double *vec, int row0, int nrows, long N, const CoarseRows &cr, cudaStream_t s)
{
  const long n = (long)cr.ncoarse * nrows;
  if (n > 0)
    k_prolong_t<<<nblk(n), 256, 0, s>>>(vec, row0, nrows, N, cr.ncoarse, cr.d_node, cr.d_pptr, cr.d_pcol, cr.d_pw);
}

void launch_zero_nodes(double *vec, int nrows, long N, const CoarseRows &cr, cudaStream_t s)
{
  const long n = (long)cr.ncoarse * nrows;
  if (n > 0) k_zero_nodes<<<nblk(n), 256, 0, s>>>(vec, nrows, N, cr.ncoarse, cr.d_node);
}

}  // namespace tgpu
