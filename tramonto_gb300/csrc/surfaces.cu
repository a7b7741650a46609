// Surfaces and their external fields on the GPU (set-up), described with tgpu_surface_spec in
// include/tramonto_gpu.h.  Three kernels, each a step of the reference's surface set-up:
//
//   k_surf_elements    one thread per element: the surface test of every wall at the element centre
//                      (setup_surface, src/dft_surfaces.c:236-420) gives each element a bit mask of the
//                      walls that own it; the box faces each wall touches are or-ed into a flag word
//                      (flag_wall_el, src/dft_surfaces.c:538-580).
//   k_surf_zero        one thread per node: zero density where, for some wall, no element around the
//                      node is fluid, or where one wall owns all of them (src/dft_mesh.c:1045-1145, the
//                      elements around a node as node_to_elem_return_dim, src/dft_mesh_lib.c:417-510).
//   k_vext_integrated  one warp per node: the LJ 12-6 wall-fluid potential of every wall of integrated
//                      type, integrated over the wall's elements, their images and their copies beyond
//                      IN_WALL / LAST_NODE faces (setup_integrated_LJ_walls, src/dft_vext.c:671-865;
//                      integrate_potential and get_wt_from_sten, src/dft_vext_integrated.c:42-200).
//
// The order of the field sum is the reference's, element by element in ascending element number,
// then image, then copy, because the sum of a node stops for good once it reaches vext_max: the warp
// walks the elements within reach of its node in that order (32 candidates per ballot), and spreads
// the Gauss points of one element over its lanes (a butterfly sum, which leaves every lane with the
// same value, so the clipped sum stays warp-uniform).  Positions, distances and rule choices are
// computed with the reference's operations in its order (no contraction, as in stencils.cu); the
// Gauss nodes are computed rather than tabulated, powers are products instead of pow(), and the
// Gauss points of an element are summed in a different order, so fields agree with the reference's
// to rounding.
//
// The reach test of an element reads r^2 < (max_cut + Esize_x[Ndim]) max_cut + Esize_x[Ndim] in the
// reference, one past the mesh sizes in 3-D: that entry is 0 in 1-D and 2-D, and the padding after
// the array in the reference build here, so the test is r^2 < max_cut^2, r measured from the
// element's lower corner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "tgpu_internal.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kRoff = 0.00000000001;   // the surface tests' tolerance (roff)
constexpr int kMaxImages = TGPU_SURF_MAXWALLS * 27;
constexpr int kWarpsPerBlock = 8;

enum { kModeId = 0, kModeAdd = 1, kModeSub = 2 };

// one image of a wall (WallPos_Images, src/dft_surfaces.c:120-200): how an element centre maps to
// its image per dimension, with the image and real wall centres
struct Image {
  int mode[3];
  double pic[3], prc[3];
  int ishift[3];   // lattice form: element e maps to e + ishift (periodic shift) or ishift - 1 - e (mirror)
  int lattice;     // 1 when every mapped corner is a lattice point (the offset table applies)
};

struct Mesh {
  int ndim, nodes[3], els[3];
  double size[3], esize[3];
  int bc[3][2];
  long nnodes, nels;
  double vol_el;
};

// the reference's Gauss rules of the integrated walls: ngp 6 / 3 / 3 per dimension, ngpu 20 / 12 / 6
// out of the plane, by the distance of the element (src/dft_vext.c:704-713); global memory rather than
// constant memory, since the lanes of a warp read different points
struct Rules {
  double g6x[6], g6w[6], g3x[3], g3w[3];
  double g20x[20], g20w[20], g12x[12], g12w[12], gu6x[6], gu6w[6];
};
__device__ Rules d_rules;

__host__ __device__ inline bool bc_face_wall(int b)
{
  return b == TGPU_BC_IN_WALL || b == TGPU_BC_LAST_NODE || b == TGPU_BC_LAST_NODE_RESTART;
}

// ---- surface tests (src/dft_surfaces_*.c, *_inSurfaceTest) ----------------------------------------

constexpr int kRoughBlocks = 100;          // MAX_ROUGH_BLOCK
constexpr unsigned kErrRoughBlock = 1u;    // a roughness patch index beyond the table (the reference exits)

// Roughness (src/dft_surfacesAdjust_roughness.c): the height of the patch of the table `rough`
// ([100][100] of this wall type) that holds the element centre x; w is the wall's position.
__device__ double rough_planar(const tgpu_surface_spec &s, const tgpu_wall_type &T, int orientation, const double *x,
                               const double *rough, unsigned *err)
{
  int rb[2] = {0, 0}, ib = 0;
  for (int d = 0; d < s.ndim; d++) {
    if (d == orientation) continue;
    rb[ib] = (int)((x[d] + 0.5 * s.size[d]) / T.rough_length);
    if (rb[ib] >= kRoughBlocks) { atomicOr(err, kErrRoughBlock); rb[ib] = 0; }
    ib++;
  }
  return rough[rb[0] * kRoughBlocks + rb[1]];
}

__device__ double rough_cylinder2d(const tgpu_wall_type &T, const double *x, const double *w, const double *rough,
                                   unsigned *err)
{
  const double angle_block = asin(T.rough_length / T.param[0]);
  double vec[2], rsq = 0.0;
  for (int d = 0; d < 2; d++) {
    vec[d] = x[d] - w[d];
    rsq += vec[d] * vec[d];
  }
  const double r = sqrt(rsq);
  double deg = 180. * acos(vec[0] / r) / kPi;
  if (x[1] < w[1]) deg = 360 - deg;
  const double angle = deg * kPi / 180.;
  int rb0 = (int)(angle / angle_block);
  if (rb0 >= kRoughBlocks) { atomicOr(err, kErrRoughBlock); rb0 = 0; }
  return rough[rb0 * kRoughBlocks];
}

__device__ double rough_cylinder3d(const tgpu_surface_spec &s, const tgpu_wall_type &T, const double *x,
                                   const double *w, const double *rough, unsigned *err)
{
  int dim[3], test_cos;
  const int o = T.orientation;
  if (o == 2) { dim[0] = 0; dim[1] = 1; dim[2] = 2; test_cos = 1; }
  else if (o == 1) { dim[0] = 2; dim[1] = 0; dim[2] = 1; test_cos = 0; }
  else { dim[0] = 1; dim[1] = 2; dim[2] = 0; test_cos = 2; }
  const double angle_block = asin(T.rough_length / T.param[0]);
  double vec[2], rsq = 0.0;
  for (int i = 0; i < 2; i++) {
    vec[i] = x[dim[i]] - w[dim[i]];
    rsq += vec[i] * vec[i];
  }
  const double r = sqrt(rsq);
  double deg = 180. * acos(vec[0] / r) / kPi;
  if (x[test_cos] < w[test_cos]) deg = 360 - deg;
  const double angle = kPi * deg / 180;
  int rb0 = (int)(angle / angle_block);
  int rb1 = (int)((x[o] + 0.5 * s.size[o]) / T.rough_length);
  if (rb0 >= kRoughBlocks || rb1 >= kRoughBlocks) { atomicOr(err, kErrRoughBlock); rb0 = rb1 = 0; }
  return rough[rb0 * kRoughBlocks + rb1];
}

// the roughness height of this surface at x (the fp_roughness choice of setup_surface,
// src/dft_surfaces.c:246-330; blocks use the planar patches with orientation 0, the orientation their
// geometry record leaves unset)
__device__ double rough_adjust(const tgpu_surface_spec &s, const tgpu_wall_type &T, const double *x, const double *w,
                               const double *rough, unsigned *err)
{
  if (!T.rough || s.ndim < 2) return 0.0;
  switch (T.surf_type) {
    case TGPU_SURF_PLANAR: return rough_planar(s, T, T.orientation, x, rough, err);
    case TGPU_SURF_BLOCK: return rough_planar(s, T, 0, x, rough, err);
    case TGPU_SURF_COLLOID:
    case TGPU_SURF_PORE: return s.ndim == 2 ? rough_cylinder2d(T, x, w, rough, err) : 0.0;
    case TGPU_SURF_FINITE_CYL: return rough_cylinder3d(s, T, x, w, rough, err);
    case TGPU_SURF_FINITE_PORE:
      return s.ndim == 3 ? rough_cylinder3d(s, T, x, w, rough, err) : rough_cylinder2d(T, x, w, rough, err);
    default: return 0.0;
  }
}

// the distance adjustment of the overlays the reference applies to this surface (the fp_periodic and
// fp_linear choices of setup_surface, src/dft_surfaces.c:246-330, and the forced orientations of
// src/dft_setup_params.c:681-790), after the roughness height dr
__device__ double overlay_adjust(const tgpu_wall_type &T, int ndim, const double *x, double dr)
{
  const int st = T.surf_type;
  bool per = false, lin = false, forced = false;
  if (st == TGPU_SURF_PLANAR) per = lin = ndim > 1;
  else if (st == TGPU_SURF_BLOCK) lin = true;
  else if (st == TGPU_SURF_FINITE_CYL) per = lin = forced = true;
  else if (st == TGPU_SURF_FINITE_PORE) lin = forced = true;
  double dp = 0.0, dl = 0.0;
  if (per && T.nperiodic > 0) {
    for (int i = 0; i < T.nperiodic; i++) {
      const int o = forced ? T.orientation : T.periodic_orient[i];
      dp += T.amplitude[i] * cos(2 * kPi * (x[o] - T.periodic_origin[i]) / T.wavelength[i]);
    }
  }
  if (lin && T.nlinear > 0) {
    for (int i = 0; i < T.nlinear; i++) {
      const int o = forced ? T.orientation : T.linear_orient[i];
      const double org = T.linear_origin[i], end = T.linear_end[i];
      if ((org < x[o] && x[o] <= end) || (org > x[o] && x[o] >= end)) dl += T.slope[i] * (x[o] - org);
    }
  }
  double adj = 0.0;
  adj += (dr + dp + dl);
  return adj;
}

// the cross-section distance r12 and the axial distance x12 of the cylinder tests (orientation o is
// the axis; the reference's dim[] permutation of src/dft_surfaces_cylindricalPore3D.c:60-80)
__device__ void cyl_dists(int o, const double *x, const double *w, double &r12, double &x12)
{
  int dim[3];
  if (o == 2) { dim[0] = 0; dim[1] = 1; dim[2] = 2; }
  else if (o == 1) { dim[0] = 2; dim[1] = 0; dim[2] = 1; }
  else { dim[0] = 1; dim[1] = 2; dim[2] = 0; }
  double s = 0.0;
  for (int i = 0; i < 2; i++) {
    const double dx = x[dim[i]] - w[dim[i]];
    s = s + dx * dx;
  }
  r12 = sqrt(s);
  x12 = fabs(w[dim[2]] - x[dim[2]]);
}

__device__ bool in_surface(const tgpu_wall_type &T, int ndim, const int *apply, const double *w, const double *x,
                           double adj)
{
  const int st = T.surf_type;
  if (st == TGPU_SURF_PLANAR) {
    double hw = T.param[0];
    hw += adj - kRoff;
    return fabs(w[T.orientation] - x[T.orientation]) <= hw;
  }
  if (st == TGPU_SURF_BLOCK) {
    bool in = true;
    for (int d = 0; d < ndim; d++) {
      const double hw = T.param[d] + adj - kRoff;
      if (fabs(w[d] - x[d]) > hw) in = false;
    }
    return in;
  }
  if (st == TGPU_SURF_COLLOID || st == TGPU_SURF_PORE) {
    const double radius = T.param[0] + adj - kRoff;
    double s = 0.0;
    for (int d = 0; d < ndim; d++) {
      const double x12 = w[d] - x[d];
      s += x12 * x12;
    }
    const double r12 = sqrt(s);
    return st == TGPU_SURF_COLLOID ? r12 <= radius : r12 >= radius;
  }
  // finite cylinder (3-D), finite cylindrical pore (3-D) or slit pore (2-D, orientation 1)
  const double radius = apply[0] ? T.param[0] + adj - kRoff : T.param[0] - kRoff;
  const double halflength = apply[1] ? T.param[1] + adj - kRoff : T.param[1] - kRoff;
  double r12, x12;
  if (ndim == 3) {
    cyl_dists(T.orientation, x, w, r12, x12);
  } else {
    const double dx = x[0] - w[0];
    r12 = sqrt(0.0 + dx * dx);
    x12 = fabs(w[1] - x[1]);
  }
  if (st == TGPU_SURF_FINITE_CYL) return r12 <= radius && x12 <= halflength;
  return r12 >= radius && x12 <= halflength;
}

// delx_vext of the surface tests: the distance from x to the surface (or, to_center, to its centre or
// axis) that the walls of Ipot_wf_n 2 and 3 use
__device__ double surface_dist(const tgpu_wall_type &T, int ndim, const int *apply, const double *w, const double *x,
                               double adj, bool to_center)
{
  const int st = T.surf_type;
  if (st == TGPU_SURF_PLANAR) {
    double hw = T.param[0];
    hw += adj - kRoff;
    const double x12 = fabs(w[T.orientation] - x[T.orientation]);
    return to_center ? x12 : x12 - hw;
  }
  if (st == TGPU_SURF_BLOCK) {
    bool in = true;
    double rs = 0.0, rc = 0.0;
    for (int d = 0; d < ndim; d++) {
      const double hw = T.param[d] + adj - kRoff;
      const double x12 = fabs(w[d] - x[d]);
      if (x12 > hw) in = false;
      const double xt = x12 - hw;
      if (xt > 0) {
        rs += xt * xt;
        rc += x12 * x12;
      }
    }
    if (in) return 0.0;
    return to_center ? sqrt(rc) : sqrt(rs);
  }
  if (st == TGPU_SURF_COLLOID || st == TGPU_SURF_PORE) {
    const double radius = T.param[0] + adj - kRoff;
    double q = 0.0;
    for (int d = 0; d < ndim; d++) {
      const double x12 = w[d] - x[d];
      q += x12 * x12;
    }
    const double r12 = sqrt(q);
    if (st == TGPU_SURF_PORE) return radius - r12;
    return to_center ? r12 : r12 - radius;
  }
  const double radius = apply[0] ? T.param[0] + adj - kRoff : T.param[0] - kRoff;
  const double halflength = apply[1] ? T.param[1] + adj - kRoff : T.param[1] - kRoff;
  double r12, x12;
  if (ndim == 3) {
    cyl_dists(T.orientation, x, w, r12, x12);
  } else {
    const double dx = x[0] - w[0];
    r12 = sqrt(0.0 + dx * dx);
    x12 = fabs(w[1] - x[1]);
  }
  double dsq = 0.0, csq = 0.0;
  if (st == TGPU_SURF_FINITE_CYL) {
    if (r12 > radius) dsq += (r12 - radius) * (r12 - radius);
    if (x12 > halflength) dsq += (x12 - halflength) * (x12 - halflength);
    if (r12 > radius) csq += r12 * r12;
    if (x12 > halflength) csq += x12 * x12;
    return to_center ? sqrt(csq) : sqrt(dsq);
  }
  if (x12 > halflength) dsq += (x12 - halflength) * (x12 - halflength);
  if (r12 < radius) dsq += (radius - r12) * (radius - r12);
  return sqrt(dsq);
}

// position of node index i along d (node_to_position, src/dft_mesh_lib.c:579-620)
__device__ __forceinline__ double node_pos(const Mesh &m, int d, int i)
{
  return -0.5 * m.size[d] + m.esize[d] * (double)i;
}

// the wedge test of an angle cutout (surface_angleCutout2D / surface_angleCutout3D_cyl): the angle of the
// element centre x about the wall centre w in the plane across axis `o` (3-D), in degrees over [0, 360)
__device__ bool angle_cutout(const tgpu_surface_spec &s, const tgpu_wall_type &T, const double *x, const double *w)
{
  double vec[2], rsq = 0.0;
  int test_cos = 1;
  if (s.ndim == 2) {
    for (int d = 0; d < 2; d++) {
      vec[d] = x[d] - w[d];
      rsq += vec[d] * vec[d];
    }
  } else {
    // spheres and spherical cavities keep the orientation their geometry record leaves at 0
    const int o = (T.surf_type == TGPU_SURF_FINITE_CYL || T.surf_type == TGPU_SURF_FINITE_PORE) ? T.orientation : 0;
    int dim[3];
    if (o == 2) { dim[0] = 0; dim[1] = 1; dim[2] = 2; test_cos = 1; }
    else if (o == 1) { dim[0] = 2; dim[1] = 0; dim[2] = 1; test_cos = 0; }
    else { dim[0] = 1; dim[1] = 2; dim[2] = 0; test_cos = 2; }
    for (int i = 0; i < 2; i++) {
      vec[i] = x[dim[i]] - w[dim[i]];
      rsq += vec[i] * vec[i];
    }
  }
  const double r = sqrt(rsq);
  double deg = 180. * acos(vec[0] / r) / kPi;
  if (x[test_cos] < w[test_cos]) deg = 360 - deg;
  if (T.angle_end > T.angle_start) return !(deg < T.angle_start || deg > T.angle_end);
  return deg > T.angle_start || deg < T.angle_end;
}

__device__ bool has_cutout(const tgpu_surface_spec &s, const tgpu_wall_type &T)
{
  // planar walls (2-D and 3-D), cylinders / spheres, finite cylinders and pores (src/dft_surfaces.c:246-330)
  return T.cutout && s.ndim > 1 && T.surf_type != TGPU_SURF_BLOCK &&
         !(T.surf_type == TGPU_SURF_PLANAR && s.ndim == 3);
}

// ---- k_surf_elements ------------------------------------------------------------------------------

__global__ void k_surf_elements(const tgpu_surface_spec *__restrict__ sp, Mesh m, const double *rough,
                                unsigned short *wall_el, unsigned *touch, unsigned *err)
{
  const tgpu_surface_spec &s = *sp;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < m.nels; e += (long)gridDim.x * blockDim.x) {
    int ijk[3] = {0, 0, 0};
    long r = e;
    for (int d = 0; d < m.ndim; d++) {
      ijk[d] = (int)(r % m.els[d]);
      r /= m.els[d];
    }
    double x[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < m.ndim; d++) x[d] = node_pos(m, d, ijk[d]) + 0.5 * m.esize[d];
    unsigned short bits = 0;
    for (int iw = 0; iw < s.nwalls; iw++) {
      const tgpu_wall_type &T = s.type[s.wall_type[iw]];
      const double dr = rough_adjust(s, T, x, s.wall_pos[iw], rough + (long)s.wall_type[iw] * kRoughBlocks * kRoughBlocks,
                                     err);
      const double adj = overlay_adjust(T, m.ndim, x, dr);
      if (!in_surface(T, m.ndim, s.apply_offset, s.wall_pos[iw], x, adj)) continue;
      if (has_cutout(s, T) && !angle_cutout(s, T, x, s.wall_pos[iw])) continue;
      bits |= (unsigned short)(1u << iw);
      unsigned t = 0;
      for (int d = 0; d < m.ndim; d++) {
        const int nadd = m.bc[d][1] == TGPU_BC_PERIODIC ? 0 : 1;
        if (ijk[d] == 0) t |= 1u << (2 * d);
        if (ijk[d] + nadd == m.nodes[d] - 1) t |= 1u << (2 * d + 1);
      }
      if (t) atomicOr(&touch[iw], t);
    }
    wall_el[e] = bits;
  }
}

// ---- k_surf_zero ----------------------------------------------------------------------------------

// the element at corner `loc` of node ijk (node_to_elem_return_dim with no reflection flags): its
// number, or -1 beyond an IN_WALL face (dimension and side returned), -2 beyond an IN_BULK face
__device__ long elem_around(const Mesh &m, const int *ijk_node, int loc, int &odim, int &oside)
{
  int ijk[3] = {ijk_node[0], ijk_node[1], ijk_node[2]};
  if (loc / 2 != (loc + 1) / 2) ijk[0]--;
  if (m.ndim > 1 && loc - 4 * (loc / 4) >= 2) ijk[1]--;
  if (m.ndim == 3 && loc >= 4) ijk[2]--;
  long code = 0;
  for (int d = 0; d < m.ndim; d++) {
    if (ijk[d] == -1) {
      const int b = m.bc[d][0];
      if (b == TGPU_BC_PERIODIC) ijk[d] = m.els[d] - 1;
      else if (b == TGPU_BC_REFLECT) ijk[d] = 0;
      else if (b == TGPU_BC_IN_BULK) code = -2;
      else if (b == TGPU_BC_IN_WALL) { code = -1; odim = d; oside = 0; }
      else ijk[d] = 0;   // LAST_NODE, LAST_NODE_RESTART
    } else if (ijk[d] == m.els[d]) {
      const int b = m.bc[d][1];
      if (b == TGPU_BC_PERIODIC) ijk[d] = 0;
      else if (b == TGPU_BC_REFLECT) ijk[d] = m.els[d] - 1;
      else if (b == TGPU_BC_IN_BULK) code = -2;
      else if (b == TGPU_BC_IN_WALL) { code = -1; odim = d; oside = 1; }
      else ijk[d] = m.els[d] - 1;
    }
  }
  if (code < 0) return code;
  long e = ijk[0];
  if (m.ndim > 1) e += (long)ijk[1] * m.els[0];
  if (m.ndim == 3) e += (long)ijk[2] * m.els[0] * m.els[1];
  return e;
}

__global__ void k_surf_zero(Mesh m, int nwalls, const unsigned short *wall_el, const unsigned *touch,
                            unsigned char *zero0)
{
  const int ncorner = 1 << m.ndim;
  for (long n = blockIdx.x * (long)blockDim.x + threadIdx.x; n < m.nnodes; n += (long)gridDim.x * blockDim.x) {
    int ijk[3] = {0, 0, 0};
    long r = n;
    for (int d = 0; d < m.ndim; d++) {
      ijk[d] = (int)(r % m.nodes[d]);
      r /= m.nodes[d];
    }
    int fluid[TGPU_SURF_MAXWALLS], countw[TGPU_SURF_MAXWALLS];
    for (int iw = 0; iw < nwalls; iw++) fluid[iw] = countw[iw] = 0;
    for (int loc = 0; loc < ncorner; loc++) {
      int odim = 0, oside = 0;
      const long e = elem_around(m, ijk, loc, odim, oside);
      if (e >= 0) {
        const unsigned short b = wall_el[e];
        for (int iw = 0; iw < nwalls; iw++) {
          if (!((b >> iw) & 1)) fluid[iw]++;
          if (b) countw[iw]++;
        }
      } else if (e == -2) {
        for (int iw = 0; iw < nwalls; iw++) fluid[iw]++;
      } else {
        for (int iw = 0; iw < nwalls; iw++)
          if ((touch[iw] >> (2 * odim + oside)) & 1) countw[iw]++;
      }
    }
    bool owned = false, zero = false;
    for (int iw = 0; iw < nwalls; iw++) owned |= countw[iw] == ncorner;
    for (int iw = 0; iw < nwalls; iw++) zero |= owned || fluid[iw] == 0;
    zero0[n] = zero ? 1 : 0;
  }
}

// ---- k_vext_integrated ----------------------------------------------------------------------------

// the cut-and-shifted LJ 12-6 potential (uLJ12_6_CS, src/dft_pairPot_LJ12_6.c:42-52); c6, c12 are
// (sigma/rcut)^6 and ^12
__device__ __forceinline__ double lj_cs(double r, double sigma, double eps, double rc, double c6, double c12)
{
  if (r <= rc) {
    const double q = sigma / r;
    const double q2 = q * q, q6 = q2 * q2 * q2, q12 = q6 * q6;
    return 4.0 * eps * ((q12 - c12) - (q6 - c6));
  }
  return 0.0;
}

struct PotParams {
  double sigma, eps, cut, c6, c12;
};

// get_wt_from_sten (src/dft_vext_integrated.c:160-200): r = distance / cut; in 1-D and 2-D the
// potential is integrated out of the mesh's dimensions with the ngpu-point rule
__device__ double wall_weight(int ndim, double r, const PotParams &P, int ngpu, const double *gu, const double *wu)
{
  if (r >= 1.0) return 0.0;
  if (ndim == 3) return lj_cs(r * P.cut, P.sigma, P.eps, P.cut, P.c6, P.c12);
  double temp = 0.0;
  const double zmax = sqrt(1.0 - r * r);
  for (int i = 0; i < ngpu; i++) {
    const double z = zmax * gu[i];
    const double rho = sqrt(r * r + z * z) * P.cut;
    if (ndim == 1) temp += wu[i] * z * lj_cs(rho, P.sigma, P.eps, P.cut, P.c6, P.c12);
    else temp += wu[i] * lj_cs(rho, P.sigma, P.eps, P.cut, P.c6, P.c12);
  }
  if (ndim == 1) return 2.0 * kPi * temp * P.cut * P.cut * zmax;
  return 2.0 * temp * P.cut * zmax;
}

// integrate_potential (src/dft_vext_integrated.c:42-155): the element with lower corner w seen from the
// node at f, the Gauss points t0, t0 + step, ... of the rule the distance class `near` selects
__device__ double integrate_points(const Mesh &m, const double *w, const double *f, const PotParams &P, int near,
                                   int t0, int step)
{
  const Rules &G = d_rules;
  const int ngp = near == 0 ? 6 : 3;
  const double *gp = near == 0 ? G.g6x : G.g3x, *gw = near == 0 ? G.g6w : G.g3w;
  const int ngpu = near == 0 ? 20 : (near == 1 ? 12 : 6);
  const double *gu = near == 0 ? G.g20x : (near == 1 ? G.g12x : G.gu6x);
  const double *wu = near == 0 ? G.g20w : (near == 1 ? G.g12w : G.gu6w);
  int total = ngp;
  if (m.ndim > 1) total *= ngp;
  if (m.ndim > 2) total *= ngp;
  double part = 0.0;
  for (int t = t0; t < total; t += step) {
    if (m.ndim == 3) {
      const int ig = t / (ngp * ngp), jg = (t / ngp) % ngp, kg = t % ngp;
      const double p0 = w[0] + gp[ig] * m.esize[0];
      const double p1 = w[1] + gp[jg] * m.esize[1];
      const double p2 = w[2] + gp[kg] * m.esize[2];
      double radius = sqrt((f[0] - p0) * (f[0] - p0) + (f[1] - p1) * (f[1] - p1) + (f[2] - p2) * (f[2] - p2));
      radius /= P.cut;
      const double weight = wall_weight(3, radius, P, ngpu, gu, wu);
      part += weight * gw[ig] * gw[jg] * gw[kg] * m.vol_el;
    } else if (m.ndim == 2) {
      const int ig = t / ngp, jg = t % ngp;
      const double p0 = w[0] + gp[ig] * m.esize[0];
      const double p1 = w[1] + gp[jg] * m.esize[1];
      double radius = sqrt((f[0] - p0) * (f[0] - p0) + (f[1] - p1) * (f[1] - p1));
      radius /= P.cut;
      const double weight = wall_weight(2, radius, P, ngpu, gu, wu);
      part += weight * gw[ig] * gw[jg] * m.vol_el;
    } else {
      const double p0 = w[0] + gp[t] * m.esize[0];
      double radius = fabs(f[0] - p0);
      radius /= P.cut;
      const double weight = wall_weight(1, radius, P, ngpu, gu, wu);
      part += weight * gw[t] * m.vol_el;
    }
  }
  return part;
}

// the same over the lanes of a warp; a butterfly sum leaves the element's value in every lane
__device__ double integrate_element_warp(const Mesh &m, const double *w, const double *f, const PotParams &P, int near,
                                         int lane)
{
  double part = integrate_points(m, w, f, P, near, lane, 32);
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  return part;
}

// ---- the offset table of an integrated wall type ---------------------------------------------------
// The element integral depends on the node and the element's lower corner only through their lattice
// offset delta (the corner of every image and face copy of an element is a lattice point when the
// images are periodic shifts or mirrors about the box faces).  One table per wall type holds, for
// every delta within (max_cut / Esize + 2) elements, a code and the integral per component:
//   code 0   beyond the reach test; 1..3 the Gauss rule of the distance class (r^2 < 4, < 16, else);
//   code 4   r^2 within 1e-9 (relative) of 4, 16 or max_cut^2: the reference's decision there depends
//            on the rounding of its absolute positions, so the table holds the integral under all three
//            rules and an item picks one (or none) by r^2 computed from the positions the reference
//            computes.
// Tabulated integrals are formed with the node at the origin; they differ from the reference's,
// formed at absolute positions, by rounding.  K is [rule][ncomp][n]: rule 0..2 (only the code's rule is
// filled for codes 1..3).
constexpr unsigned char kCodeSkip = 0, kCodeAmbiguous = 4;
constexpr double kAmbiguousTol = 1e-9;

struct OffTable {
  int R[3], W[3];
  long n;
  const unsigned char *code;
  const double *K;           // [3][ncomp][n]
  int ncomp;
};

__global__ void k_vext_table(Mesh m, PotParams P0, PotParams P1, PotParams P2, PotParams P3, int ncomp, double thr,
                             OffTable t, unsigned char *code, double *K)
{
  const int lane = threadIdx.x & 31;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  const PotParams P[4] = {P0, P1, P2, P3};
  for (long i = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5; i < t.n; i += nwarps) {
    long r = i;
    double w[3] = {0.0, 0.0, 0.0};
    const double f[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < 3; d++) {
      const int delta = (int)(r % t.W[d]) - t.R[d];
      r /= t.W[d];
      if (d < m.ndim) w[d] = delta * m.esize[d];
    }
    double r2 = 0.0;
    for (int d = 0; d < m.ndim; d++) r2 += (w[d] - f[d]) * (w[d] - f[d]);
    unsigned char c0;
    if (fabs(r2 - thr) <= kAmbiguousTol * thr || fabs(r2 - 4.0) <= kAmbiguousTol * 4.0 ||
        fabs(r2 - 16.0) <= kAmbiguousTol * 16.0) {
      c0 = kCodeAmbiguous;
    } else if (!(r2 < thr)) {
      c0 = kCodeSkip;
    } else {
      c0 = (unsigned char)(1 + (r2 < 4.0 ? 0 : (r2 < 16.0 ? 1 : 2)));
    }
    for (int rule = 0; rule < 3; rule++) {
      const bool want = c0 == kCodeAmbiguous || c0 == rule + 1;
      for (int c = 0; c < ncomp; c++) {
        const double v = want ? integrate_element_warp(m, w, f, P[c], rule, lane) : 0.0;
        if (lane == 0) K[((long)rule * ncomp + c) * t.n + i] = v;
      }
    }
    if (lane == 0) code[i] = c0;
  }
}

constexpr int kMaxIv = 28;

// the element coordinates along d whose image (any mode of the wall's images) lies within R elements
// of node coordinate i: sorted, merged intervals
__device__ int window(const Mesh &m, int d, int i, int R, const Image *img, int nimg, int *lo, int *hi)
{
  if (d >= m.ndim) {
    lo[0] = hi[0] = 0;
    return 1;
  }
  int n = 0;
  for (int k = 0; k < nimg && n < kMaxIv; k++) {
    const Image &I = img[k];
    long a, b;
    if (I.mode[d] == kModeId) {
      a = i - R; b = i + R;
    } else if (I.mode[d] == kModeAdd) {
      const long sh = llround((I.pic[d] - I.prc[d]) / m.esize[d]);
      a = i - sh - R; b = i - sh + R;
    } else {
      const long M = llround((I.pic[d] + I.prc[d] + m.size[d]) / m.esize[d]);
      a = M - 1 - i - R; b = M - 1 - i + R;
    }
    a = max(a - 1, 0L);
    b = min(b + 1, (long)m.els[d] - 1);
    if (a > b) continue;
    int j = n++;   // insertion by start
    while (j > 0 && lo[j - 1] > a) { lo[j] = lo[j - 1]; hi[j] = hi[j - 1]; j--; }
    lo[j] = (int)a; hi[j] = (int)b;
  }
  int out = 0;
  for (int k = 0; k < n; k++) {
    if (out > 0 && lo[k] <= hi[out - 1] + 1) {
      hi[out - 1] = max(hi[out - 1], hi[k]);
    } else {
      lo[out] = lo[k]; hi[out] = hi[k]; out++;
    }
  }
  return out;
}

struct NodeState {
  double V[TGPU_MAXC];
  bool live[TGPU_MAXC];   // not zero density
  int ncomp;
  double vmax;
  __device__ bool frozen() const
  {
    for (int c = 0; c < ncomp; c++)
      if (live[c] && (V[c] < vmax || V[c] == 0.0)) return false;
    return true;
  }
};

// The items of one wall element for one node — every image and face copy, in the reference's order
// (src/dft_vext.c:727-858) — summed in order per component, with the largest running sum: the node's
// clipped sum reaches vext_max inside this element exactly when its value before it plus that peak does.
__device__ void element_items(const Mesh &m, const int *ije, const Image *img, int nimg, double max_cut, double thr,
                              const PotParams *P, const NodeState &S, const int *ijk_f, const double *f,
                              const OffTable &t, double *sum, double *peak)
{
  for (int c = 0; c < S.ncomp; c++) {
    sum[c] = 0.0;
    peak[c] = -1.0e300;
  }
  // face copies: the reference tests |centre -/+ Esize/2 +/- Size/2| < 1e-6, i.e. the first or last element
  // along a dimension (Esize is far above 1e-6); the last dimension that holds decides
  int nghost = 0, gd = 0, gstep = 0;
  for (int d = 0; d < m.ndim; d++) {
    if (bc_face_wall(m.bc[d][0]) && ije[d] == 0) {
      nghost = (int)(max_cut / m.esize[d]);
      gd = d;
      gstep = -1;
    } else if (bc_face_wall(m.bc[d][1]) && ije[d] == m.els[d] - 1) {
      nghost = (int)(max_cut / m.esize[d]);
      gd = d;
      gstep = 1;
    }
  }
  for (int k = 0; k < nimg; k++) {
    const Image &I = img[k];
    int ci[3] = {0, 0, 0};
    for (int d = 0; d < m.ndim; d++)
      ci[d] = I.mode[d] == kModeId ? ije[d] : (I.mode[d] == kModeAdd ? ije[d] + I.ishift[d] : I.ishift[d] - 1 - ije[d]);
    for (int g = 0; g <= nghost; g++) {
      unsigned char code = kCodeAmbiguous;
      long idx = 0;
      if (I.lattice) {
        bool inside = true;
        for (int d = 2; d >= 0; d--) {
          const int delta = d < m.ndim ? ci[d] + (d == gd ? g * gstep : 0) - ijk_f[d] : 0;
          if (delta < -t.R[d] || delta > t.R[d]) inside = false;
          idx = idx * t.W[d] + (delta + t.R[d]);
        }
        if (!inside) continue;
        code = t.code[idx];
      }
      if (code == kCodeSkip) continue;
      int rule = code - 1;
      double w[3] = {0.0, 0.0, 0.0};
      if (code == kCodeAmbiguous) {
        // the item's lower corner as the reference computes it (src/dft_vext.c:741-790)
        for (int d = 0; d < m.ndim; d++) {
          const double center = node_pos(m, d, ije[d]) + 0.5 * m.esize[d];
          if (I.mode[d] == kModeId) {
            w[d] = center;
          } else {
            const double delta = center - I.prc[d];
            w[d] = I.mode[d] == kModeAdd ? I.pic[d] + delta : I.pic[d] - delta;
          }
          w[d] -= 0.5 * m.esize[d];
          if (g > 0 && d == gd) w[d] = w[d] + g * (gstep * m.esize[d]);
        }
        double r2 = 0.0;
        for (int d = 0; d < m.ndim; d++) r2 += (w[d] - f[d]) * (w[d] - f[d]);
        if (!(r2 < thr)) continue;
        rule = r2 < 4.0 ? 0 : (r2 < 16.0 ? 1 : 2);
      }
      for (int c = 0; c < S.ncomp; c++) {
        if (!S.live[c]) continue;
        // an image off the lattice (a wall mirrored about a face it lies beyond) is integrated here
        const double v = I.lattice ? t.K[((long)rule * t.ncomp + c) * t.n + idx] : integrate_points(m, w, f, P[c], rule, 0, 1);
        sum[c] += v;
        peak[c] = fmax(peak[c], sum[c]);
      }
    }
  }
}

// the 1-D wall forms (src/dft_vext_1D.c:40-230) and the LJ 12-6 pair potential at distance x
__device__ double wall_1d(const tgpu_wall_type &T, int c, double sigma_ff, double vmax, double x)
{
  const double sigma = T.sigma_wf[c], cut = T.cut_wf[c];
  if (T.type_vext == 1) {
    const double q = sigma / cut, q2 = q * q, q6 = q2 * q2 * q2;
    return lj_cs(x, sigma, T.eps_wf[c], cut, q6, q6 * q6);
  }
  const double prefac = T.eps_wf[c] * T.rho_w;
  const double s3 = sigma * sigma * sigma;
  auto p3 = [](double a) { return a * a * a; };
  switch (T.pot_id) {
    case TGPU_WALL1D_LJ93_CS:
      if (x > cut) return 0.0;
      return prefac * (2.0 * kPi / 3.0) * s3 *
             ((2.0 / 15.0) * (p3(p3(sigma / x)) - p3(p3(sigma / cut))) - (p3(sigma / x) - p3(sigma / cut)));
    case TGPU_WALL1D_LJ93_V2_CS:
      if (x > cut) return 0.0;
      return prefac * ((2.0 / 15.0) * (p3(p3(sigma / x)) - p3(p3(sigma / cut))) - (p3(sigma / x) - p3(sigma / cut)));
    case TGPU_WALL1D_LJ93_NOCS:
      if (x > cut) return 0.0;
      return prefac * (2.0 * kPi / 3.0) * ((2.0 / 15.0) * (p3(s3) * s3) / p3(p3(x)) - (s3 * s3) / p3(x));
    case TGPU_WALL1D_LJ93_SHIFTX_CS: {
      const double delta = 0.5 * (sigma_ff - 1);
      const double xmax = cut + delta, xmin = xmax - 0.5;
      if (x <= xmin) return vmax;
      if (x > xmax) return 0.0;
      const double q = sigma / (x - delta);
      return prefac * ((2.0 / 15.0) * (p3(p3(q)) - p3(p3(sigma / cut))) - (p3(q) - p3(sigma / cut)));
    }
    case TGPU_WALL1D_REPULSIVE9:
      if (x > cut) return 0.0;
      return prefac * (2.0 * kPi / 3.0) * s3 * ((2.0 / 15.0) * p3(p3(sigma / x)));
    default:   // TGPU_WALL1D_EXP_ATT
      if (x > cut) return 0.0;
      return -prefac * exp(-x / sigma);
  }
}

// setup_vext_XRSurf (src/dft_vext.c:364-436) for one real wall at one node: X_wall from the surface test at
// the node with the overlay adjustment of the element the reference tests the node from (its own lower
// corner element, the last element along a dimension for the far nodes; src/dft_surfaces.c:400-430)
__device__ void add_xr_wall(const tgpu_surface_spec &s, const Mesh &m, int iw, const int *ijk, const double *rough,
                            unsigned *err, NodeState &S)
{
  const tgpu_wall_type &T = s.type[s.wall_type[iw]];
  double xc[3] = {0.0, 0.0, 0.0}, xt[3] = {0.0, 0.0, 0.0};
  for (int d = 0; d < m.ndim; d++) {
    const int e = min(ijk[d], m.els[d] - 1);
    const double p = node_pos(m, d, e);
    xc[d] = p + 0.5 * m.esize[d];
    xt[d] = p + (ijk[d] - e) * m.esize[d];
  }
  const double dr = rough_adjust(s, T, xc, s.wall_pos[iw], rough + (long)s.wall_type[iw] * kRoughBlocks * kRoughBlocks,
                                 err);
  const double adj = overlay_adjust(T, m.ndim, xc, dr);
  const double delx = surface_dist(T, m.ndim, s.apply_offset, s.wall_pos[iw], xt, adj,
                                   T.ipot_wf == TGPU_VEXT_DIST_TO_CENTER);
  const double xw = delx > 0.0 ? fmin(delx, 1000.0) : 0.0;
  for (int c = 0; c < S.ncomp; c++) {
    if (!S.live[c]) continue;
    if (fabs(S.V[c] - S.vmax) > 1.e-6) {
      if (xw > 0.001) S.V[c] += wall_1d(T, c, s.sigma_ff[c], S.vmax, xw);
      else S.V[c] = S.vmax;
    }
    if (S.V[c] >= S.vmax) S.V[c] = S.vmax;
  }
}

struct Tables {
  OffTable t[TGPU_SURF_MAXTYPES];
};

// the wall-fluid parameters of component c of a wall type, with (sigma/cut)^6 and ^12 as products
__host__ __device__ inline PotParams pot_params(const tgpu_wall_type &T, int c)
{
  const double q = T.sigma_wf[c] / T.cut_wf[c], q2 = q * q, q6 = q2 * q2 * q2;
  return PotParams{T.sigma_wf[c], T.eps_wf[c], T.cut_wf[c], q6, q6 * q6};
}

__global__ void __launch_bounds__(32 * kWarpsPerBlock)
k_vext_integrated(const tgpu_surface_spec *__restrict__ sp, Mesh m, const Image *img, const int *img_first,
                  const int *img_count, Tables tabs, const double *rough, unsigned *err, const unsigned short *wall_el,
                  const unsigned char *zero0, double *vext, signed char *zero)
{
  const tgpu_surface_spec &s = *sp;
  const int lane = threadIdx.x & 31;
  const long nwarps = ((long)gridDim.x * blockDim.x) >> 5;
  for (long n = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5; n < m.nnodes; n += nwarps) {
    int ijk[3] = {0, 0, 0};
    long r = n;
    for (int d = 0; d < m.ndim; d++) {
      ijk[d] = (int)(r % m.nodes[d]);
      r /= m.nodes[d];
    }
    double f[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < m.ndim; d++) f[d] = node_pos(m, d, ijk[d]);
    NodeState S;
    S.ncomp = s.ncomp;
    S.vmax = s.vext_max;
    const bool z0 = zero0[n] != 0;
    for (int c = 0; c < s.ncomp; c++) {
      S.live[c] = !z0;
      S.V[c] = z0 ? s.vext_max : 0.0;
    }
    for (int iw = 0; iw < s.nwalls && !z0; iw++) {
      const tgpu_wall_type &T = s.type[s.wall_type[iw]];
      if (T.ipot_wf == TGPU_VEXT_DIST_TO_SURF || T.ipot_wf == TGPU_VEXT_DIST_TO_CENTER) {
        add_xr_wall(s, m, iw, ijk, rough, err, S);
        continue;
      }
      if (T.ipot_wf != TGPU_VEXT_INTEGRATED) continue;
      if (S.frozen()) continue;
      double max_cut = 0.0;
      PotParams P[TGPU_MAXC];
      for (int c = 0; c < s.ncomp; c++) {
        if (max_cut < T.cut_wf[c]) max_cut = T.cut_wf[c];
        P[c] = pot_params(T, c);
      }
      const OffTable &tab = tabs.t[s.wall_type[iw]];
      const double thr = (max_cut + 0.0) * max_cut + 0.0;
      const Image *wimg = img + img_first[iw];
      const int nimg = img_count[iw];
      int lo[3][kMaxIv], hi[3][kMaxIv], niv[3];
      for (int d = 0; d < 3; d++) {
        const int R = d < m.ndim ? (int)(max_cut / m.esize[d]) + 2 : 0;
        niv[d] = window(m, d, ijk[d], R, wimg, nimg, lo[d], hi[d]);
      }
      bool stop = false;
      for (int iz = 0; iz < niv[2] && !stop; iz++)
        for (int z = lo[2][iz]; z <= hi[2][iz] && !stop; z++)
          for (int iy = 0; iy < niv[1] && !stop; iy++)
            for (int y = lo[1][iy]; y <= hi[1][iy] && !stop; y++)
              for (int ix = 0; ix < niv[0] && !stop; ix++)
                for (int x0 = lo[0][ix]; x0 <= hi[0][ix] && !stop; x0 += 32) {
                  const int x = x0 + lane;
                  const long row = ((long)z * m.els[1] + y) * m.els[0];
                  const bool cand = x <= hi[0][ix] && ((wall_el[row + x] >> iw) & 1);
                  unsigned mask = __ballot_sync(0xffffffffu, cand);
                  if (!mask) continue;
                  double sum[TGPU_MAXC], peak[TGPU_MAXC];
                  if (cand) {
                    const int ije[3] = {x, y, z};
                    element_items(m, ije, wimg, nimg, max_cut, thr, P, S, ijk, f, tab, sum, peak);
                  }
                  // the elements of this chunk in ascending order
                  while (mask) {
                    const int b = __ffs(mask) - 1;
                    mask &= mask - 1;
                    for (int c = 0; c < s.ncomp; c++) {
                      const double sb = __shfl_sync(0xffffffffu, cand ? sum[c] : 0.0, b);
                      const double pb = __shfl_sync(0xffffffffu, cand ? peak[c] : 0.0, b);
                      if (!S.live[c] || !(S.V[c] < S.vmax || S.V[c] == 0.0)) continue;
                      if (S.V[c] + pb >= S.vmax) S.V[c] = S.vmax;
                      else S.V[c] += sb;
                    }
                  }
                  if (S.frozen()) stop = true;
                }
    }
    if (lane == 0) {
      for (int c = 0; c < s.ncomp; c++) {
        vext[(long)c * m.nnodes + n] = S.V[c];
        zero[(long)c * m.nnodes + n] = S.V[c] >= s.vext_max ? 1 : 0;
      }
    }
  }
}

}  // namespace

namespace {

// the mesh of the spec (set_up_mesh, src/dft_mesh.c:650-705); false when Size_x and Esize_x are not
// commensurate
bool make_mesh(const tgpu_surface_spec *s, Mesh &m)
{
  m.ndim = s->ndim;
  m.nnodes = m.nels = 1;
  m.vol_el = 1.0;
  for (int d = 0; d < 3; d++) {
    m.nodes[d] = m.els[d] = 1;
    m.size[d] = d < s->ndim ? s->size[d] : 0.0;
    m.esize[d] = d < s->ndim ? s->esize[d] : 0.0;
    m.bc[d][0] = d < s->ndim ? s->bc[d][0] : TGPU_BC_IN_BULK;
    m.bc[d][1] = d < s->ndim ? s->bc[d][1] : TGPU_BC_IN_BULK;
  }
  for (int d = 0; d < s->ndim; d++) {
    if (!(s->esize[d] > 0.0) || !(s->size[d] > 0.0)) return false;
    if (std::lround(std::fmod(s->size[d], s->esize[d])) != 0) return false;
    m.nodes[d] = (int)std::lround(s->size[d] / s->esize[d] + 1.);
    m.els[d] = m.nodes[d] - 1;
    if (s->bc[d][0] == TGPU_BC_PERIODIC && s->bc[d][1] == TGPU_BC_PERIODIC) m.nodes[d]--;
    if (m.els[d] < 1) return false;
    m.nnodes *= m.nodes[d];
    m.nels *= m.els[d];
    m.vol_el *= s->esize[d];
  }
  return true;
}

int check_spec(const tgpu_surface_spec *s)
{
  if (!s || s->ndim < 1 || s->ndim > 3 || s->ncomp < 1 || s->ncomp > TGPU_MAXC) return TGPU_ERR_ARG;
  if (s->nwalls < 0 || s->nwalls > TGPU_SURF_MAXWALLS || s->ntypes < 0 || s->ntypes > TGPU_SURF_MAXTYPES)
    return TGPU_ERR_ARG;
  if (!(s->vext_max > 0.0)) return TGPU_ERR_ARG;
  for (int d = 0; d < s->ndim; d++)
    for (int k = 0; k < 2; k++)
      if (s->bc[d][k] < TGPU_BC_IN_WALL || s->bc[d][k] > TGPU_BC_LAST_NODE_RESTART) return TGPU_ERR_ARG;
  for (int w = 0; w < s->nwalls; w++)
    if (s->wall_type[w] < 0 || s->wall_type[w] >= s->ntypes) return TGPU_ERR_ARG;
  for (int t = 0; t < s->ntypes; t++) {
    const tgpu_wall_type &T = s->type[t];
    if (T.nperiodic < 0 || T.nperiodic > TGPU_SURF_MAXFNC || T.nlinear < 0 || T.nlinear > TGPU_SURF_MAXFNC)
      return TGPU_ERR_ARG;
    for (int i = 0; i < T.nperiodic; i++)
      if (T.periodic_orient[i] < 0 || T.periodic_orient[i] >= s->ndim || T.wavelength[i] == 0.0) return TGPU_ERR_ARG;
    for (int i = 0; i < T.nlinear; i++)
      if (T.linear_orient[i] < 0 || T.linear_orient[i] >= s->ndim) return TGPU_ERR_ARG;
    switch (T.surf_type) {
      case TGPU_SURF_PLANAR:
        if (T.orientation < 0 || T.orientation >= s->ndim) return TGPU_ERR_ARG;
        break;
      case TGPU_SURF_BLOCK:
        break;
      case TGPU_SURF_COLLOID:
      case TGPU_SURF_PORE:
        if (s->ndim == 1) return TGPU_ERR_UNSUPPORTED;
        break;
      case TGPU_SURF_FINITE_CYL:
        if (s->ndim != 3) return TGPU_ERR_UNSUPPORTED;
        if (T.orientation < 0 || T.orientation > 2) return TGPU_ERR_ARG;
        break;
      case TGPU_SURF_FINITE_PORE:
        if (s->ndim == 1 || (s->ndim == 2 && T.orientation != 1)) return TGPU_ERR_UNSUPPORTED;
        if (T.orientation < 0 || T.orientation > 2) return TGPU_ERR_ARG;
        break;
      default:
        return TGPU_ERR_UNSUPPORTED;
    }
    if (T.cutout && !(T.angle_start != T.angle_end)) return TGPU_ERR_ARG;
    // the reference gives 3-D planar walls the 2-D wedge test, which writes past its 2-vector there
    if (T.cutout && T.surf_type == TGPU_SURF_PLANAR && s->ndim == 3) return TGPU_ERR_UNSUPPORTED;
    if (T.rough && s->ndim > 1) {
      if (!(T.rough_length > 0.0)) return TGPU_ERR_ARG;
      // the reference exits when a patch is longer than the radius (or a quarter of a cylinder's length)
      const bool cyl = T.surf_type == TGPU_SURF_FINITE_CYL || T.surf_type == TGPU_SURF_FINITE_PORE ||
                       ((T.surf_type == TGPU_SURF_COLLOID || T.surf_type == TGPU_SURF_PORE) && s->ndim == 2);
      if (cyl && T.rough_length > T.param[0]) return TGPU_ERR_ARG;
      if ((T.surf_type == TGPU_SURF_FINITE_CYL || (T.surf_type == TGPU_SURF_FINITE_PORE && s->ndim == 3)) &&
          T.rough_length > (T.param[1] - kRoff) / 2.)
        return TGPU_ERR_ARG;
    }
    if (T.ipot_wf != TGPU_VEXT_NONE && T.ipot_wf != TGPU_VEXT_HARD && T.ipot_wf != TGPU_VEXT_INTEGRATED &&
        T.ipot_wf != TGPU_VEXT_DIST_TO_SURF && T.ipot_wf != TGPU_VEXT_DIST_TO_CENTER)
      return TGPU_ERR_UNSUPPORTED;
    if (T.ipot_wf == TGPU_VEXT_INTEGRATED && (T.type_vext != 1 || T.pot_id != 0)) return TGPU_ERR_UNSUPPORTED;
    if ((T.ipot_wf == TGPU_VEXT_DIST_TO_SURF || T.ipot_wf == TGPU_VEXT_DIST_TO_CENTER) &&
        !(T.type_vext == 1 ? T.pot_id == 0 : (T.pot_id >= TGPU_WALL1D_LJ93_CS && T.pot_id <= TGPU_WALL1D_EXP_ATT)))
      return TGPU_ERR_UNSUPPORTED;
    // a component with sigma_wf = cut_wf = 0 (values a deck leaves unset) sees nothing of the wall, as in the
    // reference; negative or non-finite values are refused
    if (T.ipot_wf >= TGPU_VEXT_DIST_TO_SURF)
      for (int c = 0; c < s->ncomp; c++)
        if (!(T.cut_wf[c] >= 0.0) || !(T.sigma_wf[c] >= 0.0) || (T.cut_wf[c] > 0.0) != (T.sigma_wf[c] > 0.0))
          return TGPU_ERR_ARG;
  }
  return TGPU_OK;
}

// the images of every wall in the reference's order (find_wall_images and the loops of
// src/dft_surfaces.c:120-200), and how each maps an element centre per dimension
// (src/dft_vext.c:741-767); false where the reference would reuse a stale position
bool make_images(const tgpu_surface_spec *s, std::vector<Image> &out, std::vector<int> &first,
                 std::vector<int> &count)
{
  const int nd = s->ndim, nw = s->nwalls;
  std::vector<std::vector<double>> pos;
  std::vector<int> real;
  for (int w = 0; w < nw; w++) {
    pos.push_back({s->wall_pos[w][0], s->wall_pos[w][1], s->wall_pos[w][2]});
    real.push_back(w);
  }
  auto find_images = [&](int d, std::vector<double> p) {   // p by value: pos grows below
    for (int side = 0; side < 2; side++) {
      const double sign = side == 0 ? -1.0 : 1.0;
      const int b = s->bc[d][side];
      if (b != TGPU_BC_PERIODIC && b != TGPU_BC_REFLECT) continue;
      const double shift = b == TGPU_BC_PERIODIC ? s->size[d] : 2.0 * std::fabs(sign * 0.5 * s->size[d] - p[d]);
      std::vector<double> q = p;
      q[d] = p[d] + sign * shift;
      pos.push_back(q);
      real.push_back(-1);
    }
  };
  for (int w = 0; w < nw; w++) {
    for (int d = 0; d < nd; d++) {
      const int old = (int)pos.size();
      for (int i = 0; i < old; i++)
        if (real[i] == w) find_images(d, d == 0 ? pos[w] : pos[i]);
      for (int i = old; i < (int)pos.size(); i++) real[i] = w;
    }
  }
  first.assign(nw, 0);
  count.assign(nw, 0);
  out.clear();
  for (int w = 0; w < nw; w++) {
    first[w] = (int)out.size();
    for (int k = 0; k < (int)pos.size(); k++) {
      if (real[k] != w) continue;
      bool halfsurf = false;
      for (int j = 0; j < k; j++) {
        if (real[j] != w) continue;
        bool same = true;
        for (int d = 0; d < nd; d++)
          if (pos[k][d] != pos[j][d]) same = false;
        halfsurf = same;
        if (same) break;
      }
      if (k < nw) halfsurf = false;
      Image I{};
      for (int d = 0; d < nd; d++) {
        const double pic = pos[k][d], prc = pos[w][d];
        I.pic[d] = pic;
        I.prc[d] = prc;
        int side = -1;
        if (pic > prc || (halfsurf && std::fabs(pic - s->size[d] / 2.) < 1.e-5)) side = 1;
        else if (pic < prc || (halfsurf && std::fabs(pic + s->size[d] / 2.) < 1.e-5)) side = 0;
        if (side < 0) {
          I.mode[d] = kModeId;
        } else if (s->bc[d][side] == TGPU_BC_PERIODIC) {
          I.mode[d] = kModeAdd;
        } else if (s->bc[d][side] == TGPU_BC_REFLECT) {
          I.mode[d] = kModeSub;
        } else {
          return false;
        }
      }
      // the lattice form of the map: centre + (pic - prc) is element e + (pic - prc)/Esize; the mirror
      // (pic + prc) - centre has its lower corner at element (pic + prc + Size)/Esize - 1 - e
      I.lattice = 1;
      for (int d = 0; d < nd; d++) {
        if (I.mode[d] == kModeId) continue;
        const double q = I.mode[d] == kModeAdd ? (I.pic[d] - I.prc[d]) / s->esize[d]
                                               : (I.pic[d] + I.prc[d] + s->size[d]) / s->esize[d];
        const double qr = std::nearbyint(q);
        if (std::fabs(q - qr) > 1e-9 * std::max(1.0, std::fabs(q)) || std::fabs(qr) > 1e8) I.lattice = 0;
        I.ishift[d] = I.lattice ? (int)qr : 0;
      }
      out.push_back(I);
      count[w]++;
    }
  }
  return (int)out.size() <= kMaxImages;
}

// glibc's rand() after srand(seed): the additive feedback generator of random_r (TYPE_3, degree 31,
// separation 3).  The state starts from seed by r_i = 16807 r_{i-1} mod (2^31 - 1) (Schrage's method),
// i = 1..30, repeats r_0..r_2 as r_31..r_33, then runs r_i = r_{i-31} + r_{i-3} (mod 2^32); the first 310
// values are discarded and each later value gives r_i >> 1.
struct GlibcRand {
  std::vector<unsigned> r;
  size_t k = 0;
  explicit GlibcRand(unsigned seed)
  {
    if (seed == 0) seed = 1;
    r.resize(34);
    r[0] = seed;
    for (int i = 1; i < 31; i++) {
      const long hi = (long)(int)r[i - 1] / 127773, lo = (long)(int)r[i - 1] % 127773;
      long word = 16807 * lo - 2836 * hi;
      if (word < 0) word += 2147483647;
      r[i] = (unsigned)word;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    for (int i = 34; i < 344; i++) r.push_back(r[i - 31] + r[i - 3]);
    k = r.size();
  }
  int next()
  {
    const unsigned v = r[k - 31] + r[k - 3];
    r.push_back(v);
    k++;
    return (int)(v >> 1);
  }
};

// Rough_precalc[type][100][100] of src/dft_setup_params.c:303-331 (irand = rand() % (2^31 - 1))
std::vector<double> rough_tables(const tgpu_surface_spec *s)
{
  std::vector<double> out((size_t)std::max(s->ntypes, 1) * kRoughBlocks * kRoughBlocks, 0.0);
  bool any = false;
  for (int t = 0; t < s->ntypes; t++) any |= s->type[t].rough != 0;
  if (!any) return out;
  GlibcRand g(135649u);
  const int range = 2147483647;
  for (int t = 0; t < s->ntypes; t++)
    for (int i = 0; i < kRoughBlocks * kRoughBlocks; i++) {
      const int irand = g.next() % range;
      out[(size_t)t * kRoughBlocks * kRoughBlocks + i] = s->type[t].rough_max * (-0.5 + ((double)irand) / ((double)range));
    }
  return out;
}

void fill_rules(Rules &R)
{
  tgpu::gauss_rule01(6, R.g6x, R.g6w);
  tgpu::gauss_rule01(3, R.g3x, R.g3w);
  tgpu::gauss_rule01(20, R.g20x, R.g20w);
  tgpu::gauss_rule01(12, R.g12x, R.g12w);
  tgpu::gauss_rule01(6, R.gu6x, R.gu6w);
}

template <class T>
T *dev_alloc(std::vector<void *> &owned, size_t n)
{
  void *p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
  owned.push_back(p);
  return (T *)p;
}

int fail(int status, const char *text)
{
  tgpu::set_last_error(text);
  return status;
}

int surface_field(const tgpu_surface_spec *s, double *d_vext, signed char *d_zero, unsigned short *d_wall_el)
{
  int st = check_spec(s);
  if (st != TGPU_OK) return fail(st, "surface spec: an argument is out of range or an option is not built");
  Mesh m;
  if (!make_mesh(s, m)) return fail(TGPU_ERR_ARG, "surface spec: Size_x and Esize_x are not commensurate");
  std::vector<Image> img;
  std::vector<int> first, count;
  if (!make_images(s, img, first, count))
    return fail(TGPU_ERR_UNSUPPORTED, "surface spec: a wall image maps no element position (stale in the reference)");
  Rules R;
  fill_rules(R);
  std::vector<void *> owned;
  auto release = [&]() {
    for (void *p : owned) cudaFree(p);
  };
  unsigned short *wall_el = d_wall_el ? d_wall_el : dev_alloc<unsigned short>(owned, m.nels);
  unsigned *touch = dev_alloc<unsigned>(owned, TGPU_SURF_MAXWALLS + 1);   // [nwalls] face flags, then the error word
  unsigned *err = touch ? touch + TGPU_SURF_MAXWALLS : nullptr;
  const std::vector<double> rtab = rough_tables(s);
  double *rough = dev_alloc<double>(owned, rtab.size());
  unsigned char *zero0 = dev_alloc<unsigned char>(owned, m.nnodes);
  tgpu_surface_spec *dspec = dev_alloc<tgpu_surface_spec>(owned, 1);
  Image *dimg = dev_alloc<Image>(owned, img.size());
  int *dfirst = dev_alloc<int>(owned, TGPU_SURF_MAXWALLS), *dcount = dev_alloc<int>(owned, TGPU_SURF_MAXWALLS);
  if (!wall_el || !touch || !zero0 || !dimg || !dfirst || !dcount || !rough || !dspec) {
    release();
    return fail(TGPU_ERR_CUDA, "surface field: device allocation failed");
  }
  bool ok = cudaMemset(touch, 0, (TGPU_SURF_MAXWALLS + 1) * sizeof(unsigned)) == cudaSuccess;
  ok = ok && cudaMemcpy(dspec, s, sizeof(tgpu_surface_spec), cudaMemcpyHostToDevice) == cudaSuccess;
  ok = ok && cudaMemcpy(rough, rtab.data(), rtab.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!img.empty())
    ok = ok && cudaMemcpy(dimg, img.data(), img.size() * sizeof(Image), cudaMemcpyHostToDevice) == cudaSuccess;
  if (s->nwalls > 0) {
    ok = ok && cudaMemcpy(dfirst, first.data(), s->nwalls * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
    ok = ok && cudaMemcpy(dcount, count.data(), s->nwalls * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  ok = ok && cudaMemcpyToSymbol(d_rules, &R, sizeof(Rules)) == cudaSuccess;
  // the offset tables of the integrated wall types that some wall uses
  Tables tabs{};
  for (int t = 0; t < s->ntypes && ok; t++) {
    const tgpu_wall_type &T = s->type[t];
    bool used = false;
    for (int w = 0; w < s->nwalls; w++) used |= s->wall_type[w] == t;
    if (!used || T.ipot_wf != TGPU_VEXT_INTEGRATED) continue;
    double max_cut = 0.0;
    PotParams P[4] = {};
    for (int c = 0; c < s->ncomp; c++) {
      if (max_cut < T.cut_wf[c]) max_cut = T.cut_wf[c];
      P[c] = pot_params(T, c);
    }
    OffTable &tb = tabs.t[t];
    tb.n = 1;
    for (int d = 0; d < 3; d++) {
      tb.R[d] = d < m.ndim ? (int)(max_cut / m.esize[d]) + 2 : 0;
      tb.W[d] = 2 * tb.R[d] + 1;
      tb.n *= tb.W[d];
    }
    unsigned char *code = dev_alloc<unsigned char>(owned, tb.n);
    double *K = dev_alloc<double>(owned, (size_t)tb.n * s->ncomp * 3);
    tb.ncomp = s->ncomp;
    if (!code || !K) {
      release();
      return fail(TGPU_ERR_CUDA, "surface field: device allocation failed");
    }
    tb.code = code;
    tb.K = K;
    const double thr = (max_cut + 0.0) * max_cut + 0.0;
    const long bt = std::min<long>((tb.n + kWarpsPerBlock - 1) / kWarpsPerBlock, 152L * 64);
    k_vext_table<<<(int)bt, 32 * kWarpsPerBlock>>>(m, P[0], P[1], P[2], P[3], s->ncomp, thr, tb, code, K);
  }
  if (ok) {
    const int tb = 256;
    const long be = std::min<long>((m.nels + tb - 1) / tb, 152L * 16);
    const long bn = std::min<long>((m.nnodes + tb - 1) / tb, 152L * 16);
    k_surf_elements<<<(int)be, tb>>>(dspec, m, rough, wall_el, touch, err);
    k_surf_zero<<<(int)bn, tb>>>(m, s->nwalls, wall_el, touch, zero0);
    const long bw = std::min<long>((m.nnodes + kWarpsPerBlock - 1) / kWarpsPerBlock, 152L * 64);
    k_vext_integrated<<<(int)bw, 32 * kWarpsPerBlock>>>(dspec, m, dimg, dfirst, dcount, tabs, rough, err, wall_el,
                                                        zero0, d_vext, d_zero);
    ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  }
  unsigned herr = 0;
  if (ok) ok = cudaMemcpy(&herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost) == cudaSuccess;
  if (ok && herr) {
    release();
    return fail(TGPU_ERR_ARG, "surface field: a roughness patch index reaches 100 (MAX_ROUGH_BLOCK)");
  }
  release();
  return ok ? TGPU_OK : fail(TGPU_ERR_CUDA, "surface field: a CUDA call failed");
}

}  // namespace

extern "C" {

int tgpu_surface_mesh(const tgpu_surface_spec *s, int *nodes, int *elements)
{
  if (!s || !nodes || !elements || s->ndim < 1 || s->ndim > 3) return TGPU_ERR_ARG;
  Mesh m;
  if (!make_mesh(s, m)) return TGPU_ERR_ARG;
  for (int d = 0; d < 3; d++) {
    nodes[d] = m.nodes[d];
    elements[d] = m.els[d];
  }
  return TGPU_OK;
}

int tgpu_surface_rough_table(const tgpu_surface_spec *s, double *out)
{
  if (!s || !out || s->ntypes < 0 || s->ntypes > TGPU_SURF_MAXTYPES) return TGPU_ERR_ARG;
  const std::vector<double> t = rough_tables(s);
  std::copy(t.begin(), t.begin() + (size_t)s->ntypes * kRoughBlocks * kRoughBlocks, out);
  return TGPU_OK;
}

int tgpu_surface_field_device(const tgpu_surface_spec *s, double *d_vext, signed char *d_zero,
                              unsigned short *d_wall_el)
{
  if (!d_vext || !d_zero) return TGPU_ERR_ARG;
  return surface_field(s, d_vext, d_zero, d_wall_el);
}

int tgpu_surface_field_host(const tgpu_surface_spec *s, double *vext, signed char *zero, unsigned short *wall_el)
{
  if (!vext || !zero) return TGPU_ERR_ARG;
  int st = check_spec(s);
  if (st != TGPU_OK) return st;
  Mesh m;
  if (!make_mesh(s, m)) return TGPU_ERR_ARG;
  std::vector<void *> owned;
  double *dv = dev_alloc<double>(owned, (size_t)s->ncomp * m.nnodes);
  signed char *dz = dev_alloc<signed char>(owned, (size_t)s->ncomp * m.nnodes);
  unsigned short *de = wall_el ? dev_alloc<unsigned short>(owned, m.nels) : nullptr;
  if (!dv || !dz || (wall_el && !de)) {
    for (void *p : owned) cudaFree(p);
    return TGPU_ERR_CUDA;
  }
  st = surface_field(s, dv, dz, de);
  if (st == TGPU_OK) {
    bool ok = cudaMemcpy(vext, dv, (size_t)s->ncomp * m.nnodes * sizeof(double), cudaMemcpyDeviceToHost) == cudaSuccess;
    ok = ok && cudaMemcpy(zero, dz, (size_t)s->ncomp * m.nnodes, cudaMemcpyDeviceToHost) == cudaSuccess;
    if (wall_el) ok = ok && cudaMemcpy(wall_el, de, m.nels * sizeof(unsigned short), cudaMemcpyDeviceToHost) == cudaSuccess;
    if (!ok) st = TGPU_ERR_CUDA;
  }
  for (void *p : owned) cudaFree(p);
  return st;
}

}  // extern "C"
