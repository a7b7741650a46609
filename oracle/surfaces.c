/* CPU restatement of the reference's surface set-up: wall elements, zero-density nodes and the
 * integrated LJ 12-6 wall field.  Test infrastructure (the oracle of tgpu_surface_field_*), never
 * part of the product.  The loops follow the reference's nesting so that every field sum is formed
 * in the reference's order:
 *   setup_surface              src/dft_surfaces.c:39-420 (images :120-200, element tests :236-420)
 *   find_wall_images           src/dft_surfaces.c:508-536
 *   flag_wall_el               src/dft_surfaces.c:538-580 (touched faces)
 *   surface tests              src/dft_surfaces_{planar,block,sphere,cylinder2D,cylinder3D,
 *                              cylindricalPore2D,cylindricalPore3D,sphericalCavity3D,slitPore2D}.c
 *   overlays                   src/dft_surfacesAdjust_{linear,periodic}.c
 *   zero-density nodes         src/dft_mesh.c:1045-1145, node_to_elem_return_dim src/dft_mesh_lib.c:417-510
 *   setup_external_field_n     src/dft_vext.c:38-200 (setup_vext_max, setup_zero: :240-310)
 *   setup_integrated_LJ_walls  src/dft_vext.c:671-865
 *   integrate_potential, get_wt_from_sten   src/dft_vext_integrated.c:42-200
 *   uLJ12_6_CS                 src/dft_pairPot_LJ12_6.c:42-52
 * Gauss-Legendre nodes are computed here by Newton iteration on the Legendre recurrence.  The reach
 * test's Esize_x[Ndim] term is 0 (see the product's surfaces.cu). */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/tramonto_gpu.h"

#define OR_PI 3.14159265358979323846
#define OR_ROFF 0.00000000001

typedef struct {
  int ndim, nodes[3], els[3];
  long nnodes, nels;
  double vol_el;
} or_mesh;

static int or_make_mesh(const tgpu_surface_spec *s, or_mesh *m)
{
  int d;
  m->ndim = s->ndim;
  m->nnodes = m->nels = 1;
  m->vol_el = 1.0;
  for (d = 0; d < 3; d++) m->nodes[d] = m->els[d] = 1;
  for (d = 0; d < s->ndim; d++) {
    if (lround(fmod(s->size[d], s->esize[d])) != 0) return 0;
    m->nodes[d] = (int)floor(s->size[d] / s->esize[d] + 1. + 0.5);
    m->els[d] = m->nodes[d] - 1;
    if (s->bc[d][0] == TGPU_BC_PERIODIC && s->bc[d][1] == TGPU_BC_PERIODIC) m->nodes[d]--;
    m->nnodes *= m->nodes[d];
    m->nels *= m->els[d];
    m->vol_el *= s->esize[d];
  }
  return 1;
}

/* Gauss-Legendre on [0,1] */
static void or_gauss(int n, double *x, double *w)
{
  int i, k, it;
  for (i = 0; i < n; i++) {
    double z = cos(OR_PI * (i + 0.75) / (n + 0.5)), p0, p1, p2, dp = 1.0;
    for (it = 0; it < 200; it++) {
      p0 = 1.0;
      p1 = z;
      for (k = 2; k <= n; k++) {
        p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      {
        double dz = p1 / dp;
        z -= dz;
        if (fabs(dz) < 1e-17) break;
      }
    }
    p0 = 1.0;
    p1 = z;
    for (k = 2; k <= n; k++) {
      p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1.0);
    x[i] = (z + 1.0) / 2.0;
    w[i] = 2.0 / ((1.0 - z * z) * dp * dp) / 2.0;
  }
}

static void or_node_pos(const tgpu_surface_spec *s, const or_mesh *m, long inode, double *p)
{
  long r = inode;
  int d;
  for (d = 0; d < 3; d++) p[d] = 0.0;
  for (d = 0; d < m->ndim; d++) {
    int i = (int)(r % m->nodes[d]);
    r /= m->nodes[d];
    p[d] = -0.5 * s->size[d] + s->esize[d] * i;
  }
}

/* Rough_precalc (src/dft_setup_params.c:303-331): the C library's rand() after srand(135649), every wall
 * type in order; [ntypes][100][100] */
#define OR_ROUGH 100
static double *or_rough_tables(const tgpu_surface_spec *s)
{
  int t, i, any = 0;
  double *tab = calloc((size_t)(s->ntypes > 0 ? s->ntypes : 1) * OR_ROUGH * OR_ROUGH, sizeof(double));
  for (t = 0; t < s->ntypes; t++) any |= s->type[t].rough;
  if (!any) return tab;
  srand(135649);
  for (t = 0; t < s->ntypes; t++)
    for (i = 0; i < OR_ROUGH * OR_ROUGH; i++) {
      int irand = rand() % 2147483647;
      tab[(size_t)t * OR_ROUGH * OR_ROUGH + i] = s->type[t].rough_max * (-0.5 + (((double)irand) / ((double)2147483647)));
    }
  return tab;
}

/* surface_planar_roughness, surface_cylinder2D_roughness, surface_cylinder3D_roughness
 * (src/dft_surfacesAdjust_roughness.c:38-180); returns 0 and sets *bad for a patch index >= 100 */
static double or_rough(const tgpu_surface_spec *s, const tgpu_wall_type *T, const double *x, const double *wp,
                       const double *tab, int *bad)
{
  int st = T->surf_type, nd = s->ndim, rb[2] = {0, 0}, idim, ib = 0;
  if (!T->rough || nd < 2) return 0.0;
  if (st == TGPU_SURF_PLANAR || st == TGPU_SURF_BLOCK) {
    int orientation = st == TGPU_SURF_PLANAR ? T->orientation : 0;
    for (idim = 0; idim < nd; idim++) {
      if (idim != orientation) {
        rb[ib] = (int)((x[idim] + 0.5 * s->size[idim]) / T->rough_length);
        if (rb[ib] >= OR_ROUGH) { *bad = 1; return 0.0; }
        ib++;
      }
    }
  } else if (nd == 2 && (st == TGPU_SURF_COLLOID || st == TGPU_SURF_PORE || st == TGPU_SURF_FINITE_PORE)) {
    double vecB[2], rsq = 0.0, r, angle, angle_deg, angle_block = asin(T->rough_length / T->param[0]);
    for (idim = 0; idim < nd; idim++) {
      vecB[idim] = x[idim] - wp[idim];
      rsq += vecB[idim] * vecB[idim];
    }
    r = sqrt(rsq);
    angle = acos(vecB[0] / r);
    angle_deg = 180. * angle / OR_PI;
    if (x[1] < wp[1]) angle_deg = 360 - angle_deg;
    angle = angle_deg * OR_PI / 180.;
    rb[0] = (int)(angle / angle_block);
  } else if (nd == 3 && (st == TGPU_SURF_FINITE_CYL || st == TGPU_SURF_FINITE_PORE)) {
    double xtest[3], vecB[3], rsq = 0.0, r, angle, angle_deg, angle_block;
    int dim[3], test_cos;
    switch (T->orientation) {
      case 2: xtest[0] = x[0]; dim[0] = 0; xtest[1] = x[1]; dim[1] = 1; xtest[2] = x[2]; dim[2] = 2; test_cos = 1; break;
      case 1: xtest[0] = x[2]; dim[0] = 2; xtest[1] = x[0]; dim[1] = 0; xtest[2] = x[1]; dim[2] = 1; test_cos = 0; break;
      default: xtest[0] = x[1]; dim[0] = 1; xtest[1] = x[2]; dim[1] = 2; xtest[2] = x[0]; dim[2] = 0; test_cos = 2; break;
    }
    angle_block = asin(T->rough_length / T->param[0]);
    for (idim = 0; idim < nd - 1; idim++) {
      vecB[idim] = xtest[idim] - wp[dim[idim]];
      rsq += vecB[idim] * vecB[idim];
    }
    r = sqrt(rsq);
    angle = acos(vecB[0] / r);
    angle_deg = 180. * angle / OR_PI;
    if (x[test_cos] < wp[test_cos]) angle_deg = 360 - angle_deg;
    angle = OR_PI * angle_deg / 180;
    rb[0] = (int)(angle / angle_block);
    rb[1] = (int)((x[T->orientation] + 0.5 * s->size[T->orientation]) / T->rough_length);
  } else {
    return 0.0;
  }
  if (rb[0] >= OR_ROUGH || rb[1] >= OR_ROUGH) { *bad = 1; return 0.0; }
  return tab[rb[0] * OR_ROUGH + rb[1]];
}

/* surface_angleCutout2D / surface_angleCutout3D_cyl (src/dft_surfacesAdjust_angleCutout.c:40-139) with
 * the choice of setup_surface (src/dft_surfaces.c:246-330); spheres and spherical cavities have no
 * orientation set (0) */
static int or_angle_test(const tgpu_surface_spec *s, const tgpu_wall_type *T, const double *x, const double *wp)
{
  int nd = s->ndim, idim, angle_test = 1, dim[3], idim_testCos = 1, orientation;
  double vecB[3], xtest[3], rsq = 0.0, r, angle, angle_deg;
  if (!T->cutout || nd < 2 || T->surf_type == TGPU_SURF_BLOCK) return 1;
  if (nd == 2) {
    for (idim = 0; idim < nd; idim++) {
      vecB[idim] = x[idim] - wp[idim];
      rsq += vecB[idim] * vecB[idim];
    }
  } else {
    orientation = (T->surf_type == TGPU_SURF_FINITE_CYL || T->surf_type == TGPU_SURF_FINITE_PORE) ? T->orientation : 0;
    switch (orientation) {
      case 2: xtest[0] = x[0]; dim[0] = 0; xtest[1] = x[1]; dim[1] = 1; idim_testCos = 1; break;
      case 1: xtest[0] = x[2]; dim[0] = 2; xtest[1] = x[0]; dim[1] = 0; idim_testCos = 0; break;
      default: xtest[0] = x[1]; dim[0] = 1; xtest[1] = x[2]; dim[1] = 2; idim_testCos = 2; break;
    }
    for (idim = 0; idim < nd - 1; idim++) {
      vecB[idim] = xtest[idim] - wp[dim[idim]];
      rsq += vecB[idim] * vecB[idim];
    }
  }
  r = sqrt(rsq);
  angle = acos(vecB[0] / r);
  angle_deg = 180. * angle / OR_PI;
  if (x[idim_testCos] < wp[idim_testCos]) angle_deg = 360 - angle_deg;
  if (T->angle_end > T->angle_start) {
    angle_test = 1;
    if (angle_deg < T->angle_start || angle_deg > T->angle_end) angle_test = 0;
  } else if (T->angle_end < T->angle_start) {
    angle_test = 0;
    if (angle_deg > T->angle_start || angle_deg < T->angle_end) angle_test = 1;
  }
  return angle_test;
}

static double or_overlay(const tgpu_wall_type *T, int ndim, const double *x, double dist_roughness)
{
  double dist_periodic = 0.0, dist_linear = 0.0, adj = 0.0;
  int i, use_per = 0, use_lin = 0, forced = 0;
  switch (T->surf_type) {
    case TGPU_SURF_PLANAR: use_per = use_lin = ndim > 1; break;
    case TGPU_SURF_BLOCK: use_lin = 1; break;
    case TGPU_SURF_FINITE_CYL: use_per = use_lin = forced = 1; break;
    case TGPU_SURF_FINITE_PORE: use_lin = forced = 1; break;
    default: break;
  }
  if (use_per && T->nperiodic > 0) {
    double offset = 0.0;
    for (i = 0; i < T->nperiodic; i++) {
      int o = forced ? T->orientation : T->periodic_orient[i];
      offset += T->amplitude[i] * cos(2 * OR_PI * (x[o] - T->periodic_origin[i]) / T->wavelength[i]);
    }
    dist_periodic = offset;
  }
  if (use_lin && T->nlinear > 0) {
    double offset = 0.0;
    for (i = 0; i < T->nlinear; i++) {
      int o = forced ? T->orientation : T->linear_orient[i];
      if ((T->linear_origin[i] < x[o] && x[o] <= T->linear_end[i]) ||
          (T->linear_origin[i] > x[o] && x[o] >= T->linear_end[i]))
        offset += T->slope[i] * (x[o] - T->linear_origin[i]);
    }
    dist_linear = offset;
  }
  adj += (dist_roughness + dist_periodic + dist_linear);
  return adj;
}

static int or_in_surface(const tgpu_surface_spec *s, const tgpu_wall_type *T, const double *wp, const double *xt,
                         double adj)
{
  int nd = s->ndim, idim;
  double radius, halflength, r12, x12, sq;
  switch (T->surf_type) {
    case TGPU_SURF_PLANAR: {
      double halfwidth = T->param[0];
      halfwidth += adj - OR_ROFF;
      x12 = fabs(wp[T->orientation] - xt[T->orientation]);
      return x12 <= halfwidth;
    }
    case TGPU_SURF_BLOCK: {
      int in = 1;
      for (idim = 0; idim < nd; idim++) {
        double halfwidth = T->param[idim] + adj - OR_ROFF;
        x12 = fabs(wp[idim] - xt[idim]);
        if (x12 > halfwidth) in = 0;
      }
      return in;
    }
    case TGPU_SURF_COLLOID:
    case TGPU_SURF_PORE:
      radius = T->param[0] + adj - OR_ROFF;
      sq = 0.0;
      for (idim = 0; idim < nd; idim++) {
        x12 = wp[idim] - xt[idim];
        sq += x12 * x12;
      }
      r12 = sqrt(sq);
      return T->surf_type == TGPU_SURF_COLLOID ? r12 <= radius : r12 >= radius;
    default: {
      double xtest[3];
      int dim[3];
      if (s->apply_offset[0]) radius = T->param[0] + adj - OR_ROFF;
      else radius = T->param[0] - OR_ROFF;
      if (s->apply_offset[1]) halflength = T->param[1] + adj - OR_ROFF;
      else halflength = T->param[1] - OR_ROFF;
      if (nd == 3) {
        switch (T->orientation) {
          case 2: dim[0] = 0; dim[1] = 1; dim[2] = 2; break;
          case 1: dim[0] = 2; dim[1] = 0; dim[2] = 1; break;
          default: dim[0] = 1; dim[1] = 2; dim[2] = 0; break;
        }
      } else {
        dim[0] = 0; dim[1] = 1; dim[2] = 1;
      }
      for (idim = 0; idim < 3; idim++) xtest[idim] = xt[dim[idim]];
      sq = 0.0;
      for (idim = 0; idim < nd - 1; idim++) {
        double dx = xtest[idim] - wp[dim[idim]];
        sq = sq + dx * dx;
      }
      r12 = sqrt(sq);
      x12 = fabs(wp[dim[nd - 1]] - xtest[nd - 1]);
      if (T->surf_type == TGPU_SURF_FINITE_CYL) return r12 <= radius && x12 <= halflength;
      return r12 >= radius && x12 <= halflength;
    }
  }
}

/* delx_vext of the surface tests (the same src/dft_surfaces_*.c functions) */
static double or_surface_dist(const tgpu_surface_spec *s, const tgpu_wall_type *T, const double *wp, const double *xt,
                              double adj, int flag_X_to_center)
{
  int nd = s->ndim, idim;
  double radius, halflength, r12, x12, sq;
  switch (T->surf_type) {
    case TGPU_SURF_PLANAR: {
      double halfwidth = T->param[0];
      halfwidth += adj - OR_ROFF;
      x12 = fabs(wp[T->orientation] - xt[T->orientation]);
      return flag_X_to_center ? x12 : x12 - halfwidth;
    }
    case TGPU_SURF_BLOCK: {
      int in = 1;
      double rsq_surface = 0.0, rsq_center = 0.0;
      for (idim = 0; idim < nd; idim++) {
        double halfwidth = T->param[idim] + adj - OR_ROFF, xtest;
        x12 = fabs(wp[idim] - xt[idim]);
        if (x12 > halfwidth) in = 0;
        xtest = x12 - halfwidth;
        if (xtest > 0) {
          rsq_surface += xtest * xtest;
          rsq_center += x12 * x12;
        }
      }
      if (in) return 0.0;
      return flag_X_to_center ? sqrt(rsq_center) : sqrt(rsq_surface);
    }
    case TGPU_SURF_COLLOID:
    case TGPU_SURF_PORE:
      radius = T->param[0] + adj - OR_ROFF;
      sq = 0.0;
      for (idim = 0; idim < nd; idim++) {
        x12 = wp[idim] - xt[idim];
        sq += x12 * x12;
      }
      r12 = sqrt(sq);
      if (T->surf_type == TGPU_SURF_PORE) return radius - r12;
      return flag_X_to_center ? r12 : r12 - radius;
    default: {
      double xtest[3], delr_sq = 0.0, delr_sq_center = 0.0;
      int dim[3];
      if (s->apply_offset[0]) radius = T->param[0] + adj - OR_ROFF;
      else radius = T->param[0] - OR_ROFF;
      if (s->apply_offset[1]) halflength = T->param[1] + adj - OR_ROFF;
      else halflength = T->param[1] - OR_ROFF;
      if (nd == 3) {
        switch (T->orientation) {
          case 2: dim[0] = 0; dim[1] = 1; dim[2] = 2; break;
          case 1: dim[0] = 2; dim[1] = 0; dim[2] = 1; break;
          default: dim[0] = 1; dim[1] = 2; dim[2] = 0; break;
        }
      } else {
        dim[0] = 0; dim[1] = 1; dim[2] = 1;
      }
      for (idim = 0; idim < 3; idim++) xtest[idim] = xt[dim[idim]];
      sq = 0.0;
      for (idim = 0; idim < nd - 1; idim++) {
        double dx = xtest[idim] - wp[dim[idim]];
        sq = sq + dx * dx;
      }
      r12 = sqrt(sq);
      x12 = fabs(wp[dim[nd - 1]] - xtest[nd - 1]);
      if (T->surf_type == TGPU_SURF_FINITE_CYL) {
        if (r12 > radius) delr_sq += (r12 - radius) * (r12 - radius);
        if (x12 > halflength) delr_sq += (x12 - halflength) * (x12 - halflength);
        if (r12 > radius) delr_sq_center += (r12) * (r12);
        if (x12 > halflength) delr_sq_center += (x12) * (x12);
        return flag_X_to_center ? sqrt(delr_sq_center) : sqrt(delr_sq);
      }
      if (x12 > halflength) delr_sq += (x12 - halflength) * (x12 - halflength);
      if (r12 < radius) delr_sq += (radius - r12) * (radius - r12);
      return sqrt(delr_sq);
    }
  }
}

static double or_ulj(double r, double sigma, double eps, double rcut);

/* Vext_1D (src/dft_switch_vext1D.c:42-80 with src/dft_vext_1D.c) or the LJ 12-6 pair potential */
static double or_vext_1d(const tgpu_surface_spec *s, const tgpu_wall_type *T, int icomp, double x)
{
  double prefac = T->eps_wf[icomp] * T->rho_w, sigma = T->sigma_wf[icomp], cut = T->cut_wf[icomp];
  if (T->type_vext == 1) return or_ulj(x, sigma, T->eps_wf[icomp], cut);
  switch (T->pot_id) {
    case TGPU_WALL1D_LJ93_CS:
      if (x <= cut)
        return prefac * (2.0 * OR_PI / 3.0) * (pow(sigma, 3)) *
               ((2.0 / 15.0) * (pow(sigma / x, 9) - pow(sigma / cut, 9)) - (pow(sigma / x, 3) - pow(sigma / cut, 3)));
      return 0.0;
    case TGPU_WALL1D_LJ93_V2_CS:
      if (x <= cut)
        return prefac * ((2.0 / 15.0) * (pow(sigma / x, 9) - pow(sigma / cut, 9)) - (pow(sigma / x, 3) - pow(sigma / cut, 3)));
      return 0.0;
    case TGPU_WALL1D_LJ93_NOCS:
      if (x <= cut)
        return prefac * (2.0 * OR_PI / 3.0) * ((2.0 / 15.0) * pow(sigma, 12) / pow(x, 9) - pow(sigma, 6) / pow(x, 3));
      return 0.0;
    case TGPU_WALL1D_LJ93_SHIFTX_CS: {
      double delta = 0.5 * (s->sigma_ff[icomp] - 1), xmax = cut + delta, xmin = xmax - 0.5;
      if (x <= xmin) return s->vext_max;
      if (x <= xmax)
        return prefac * ((2.0 / 15.0) * (pow(sigma / (x - delta), 9) - pow(sigma / cut, 9)) -
                         (pow(sigma / (x - delta), 3) - pow(sigma / cut, 3)));
      return 0.0;
    }
    case TGPU_WALL1D_REPULSIVE9:
      if (x <= cut) return prefac * (2.0 * OR_PI / 3.0) * pow(sigma, 3) * ((2.0 / 15.0) * pow(sigma / x, 9));
      return 0.0;
    default:
      if (x <= cut) return -prefac * exp(-x / sigma);
      return 0.0;
  }
}

static double or_ulj(double r, double sigma, double eps, double rcut)
{
  double u;
  if (r <= rcut) u = (pow(sigma / r, 12) - pow(sigma / rcut, 12)) - (pow(sigma / r, 6) - pow(sigma / rcut, 6));
  else u = 0.0;
  return 4.0 * eps * u;
}

static double or_wt(int ndim, double r, double sigma, double eps, double rcut, int ngpu, const double *gpu,
                    const double *gwu)
{
  double temp, zmax, z, rho;
  int i;
  if (r >= 1.0) return 0.0;
  if (ndim == 1) {
    temp = 0.0;
    zmax = sqrt(1.0 - r * r);
    for (i = 0; i < ngpu; i++) {
      z = zmax * gpu[i];
      rho = sqrt(r * r + z * z) * rcut;
      temp += gwu[i] * z * or_ulj(rho, sigma, eps, rcut);
    }
    return 2.0 * OR_PI * temp * rcut * rcut * zmax;
  }
  if (ndim == 2) {
    temp = 0.0;
    zmax = sqrt(1 - r * r);
    for (i = 0; i < ngpu; i++) {
      z = zmax * gpu[i];
      rho = sqrt(r * r + z * z) * rcut;
      temp += gwu[i] * or_ulj(rho, sigma, eps, rcut);
    }
    return 2.0 * temp * rcut * zmax;
  }
  rho = r * rcut;
  return or_ulj(rho, sigma, eps, rcut);
}

static double or_integrate(const tgpu_surface_spec *s, double vol_el, double sigma, double eps, double cut, int ngp,
                           int ngpu, const double *gp, const double *gpu, const double *gw, const double *gwu,
                           const double *npos, const double *fpos)
{
  int ig, jg, kg;
  double vext = 0.0, radius, point[3], weight;
  const double *E = s->esize;
  if (s->ndim == 1) {
    for (ig = 0; ig < ngp; ig++) {
      point[0] = npos[0] + gp[ig] * E[0];
      radius = fabs(fpos[0] - point[0]);
      radius /= cut;
      weight = or_wt(1, radius, sigma, eps, cut, ngpu, gpu, gwu);
      vext += weight * gw[ig] * vol_el;
    }
  } else if (s->ndim == 2) {
    for (ig = 0; ig < ngp; ig++) {
      point[0] = npos[0] + gp[ig] * E[0];
      for (jg = 0; jg < ngp; jg++) {
        point[1] = npos[1] + gp[jg] * E[1];
        radius = sqrt((fpos[0] - point[0]) * (fpos[0] - point[0]) + (fpos[1] - point[1]) * (fpos[1] - point[1]));
        radius /= cut;
        weight = or_wt(2, radius, sigma, eps, cut, ngpu, gpu, gwu);
        vext += weight * gw[ig] * gw[jg] * vol_el;
      }
    }
  } else {
    for (ig = 0; ig < ngp; ig++) {
      point[0] = npos[0] + gp[ig] * E[0];
      for (jg = 0; jg < ngp; jg++) {
        point[1] = npos[1] + gp[jg] * E[1];
        for (kg = 0; kg < ngp; kg++) {
          point[2] = npos[2] + gp[kg] * E[2];
          radius = sqrt((fpos[0] - point[0]) * (fpos[0] - point[0]) + (fpos[1] - point[1]) * (fpos[1] - point[1]) +
                        (fpos[2] - point[2]) * (fpos[2] - point[2]));
          radius /= cut;
          weight = or_wt(3, radius, sigma, eps, cut, ngpu, gpu, gwu);
          vext += weight * gw[ig] * gw[jg] * gw[kg] * vol_el;
        }
      }
    }
  }
  return vext;
}

/* element ielement's number around node inode at corner loc (node_to_elem_return_dim, no reflection
 * flags): -1 beyond an IN_WALL face (*idim_return, *iside), -2 beyond an IN_BULK face */
static long or_node_to_elem(const tgpu_surface_spec *s, const or_mesh *m, long inode, int loc, int *idim_return,
                            int *iside)
{
  int ijk[3] = {0, 0, 0}, idim;
  long r = inode, iel = 0;
  for (idim = 0; idim < m->ndim; idim++) {
    ijk[idim] = (int)(r % m->nodes[idim]);
    r /= m->nodes[idim];
  }
  if (loc / 2 != (loc + 1) / 2) ijk[0]--;
  if (m->ndim > 1 && loc - 4 * (loc / 4) >= 2) ijk[1]--;
  if (m->ndim == 3 && loc >= 4) ijk[2]--;
  for (idim = 0; idim < m->ndim; idim++) {
    if (ijk[idim] == -1) {
      if (s->bc[idim][0] == TGPU_BC_PERIODIC) ijk[idim] = m->els[idim] - 1;
      else if (s->bc[idim][0] == TGPU_BC_REFLECT) ijk[idim] = 0;
      else if (s->bc[idim][0] == TGPU_BC_IN_BULK) iel = -2;
      else if (s->bc[idim][0] == TGPU_BC_IN_WALL) { iel = -1; *idim_return = idim; *iside = 0; }
      else ijk[idim] = 0;
    } else if (ijk[idim] == m->els[idim]) {
      if (s->bc[idim][1] == TGPU_BC_PERIODIC) ijk[idim] = 0;
      else if (s->bc[idim][1] == TGPU_BC_REFLECT) ijk[idim] = m->els[idim] - 1;
      else if (s->bc[idim][1] == TGPU_BC_IN_BULK) iel = -2;
      else if (s->bc[idim][1] == TGPU_BC_IN_WALL) { iel = -1; *idim_return = idim; *iside = 1; }
      else ijk[idim] = m->els[idim] - 1;
    }
  }
  if (iel >= 0) {
    iel = ijk[0];
    if (m->ndim > 1) iel += (long)ijk[1] * m->els[0];
    if (m->ndim == 3) iel += (long)ijk[2] * m->els[0] * m->els[1];
  }
  return iel;
}

static void or_find_wall_images(const tgpu_surface_spec *s, int idim, int *image, double (*image_pos)[3],
                                const double *pos)
{
  int iside, jdim;
  double sign, shift = 0;
  for (iside = 0; iside < 2; iside++) {
    sign = iside == 0 ? -1.0 : 1.0;
    if (s->bc[idim][iside] == TGPU_BC_PERIODIC || s->bc[idim][iside] == TGPU_BC_REFLECT) {
      if (s->bc[idim][iside] == TGPU_BC_PERIODIC) shift = s->size[idim];
      else shift = 2.0 * fabs(sign * 0.5 * s->size[idim] - pos[idim]);
      for (jdim = 0; jdim < s->ndim; jdim++)
        image_pos[*image][jdim] = jdim == idim ? pos[jdim] + sign * shift : pos[jdim];
      (*image)++;
    }
  }
}

/* vext, zero [ncomp][nnodes]; wall_el [nels] bit masks (may be NULL).  Returns 0, or -1 for what the
 * restatement does not cover. */
int oracle_surface_field(const tgpu_surface_spec *s, double *vext, signed char *zero, unsigned short *wall_el_out)
{
  or_mesh m;
  int nd = s->ndim, nw = s->nwalls, iwall, idim, i, icomp, ncorner;
  int nimg, k_img, *real, (*touch)[3][2];
  double (*wpos)[3], *xwall, *rough;
  int bad_rough = 0;
  unsigned short *wall_el;
  long iel, inode;
  signed char *zero0;
  double gp1[6], gw1[6], gp2[3], gw2[3], gp3[3], gw3[3], gpu1[20], gwu1[20], gpu2[12], gwu2[12], gpu3[6], gwu3[6];
  if (!or_make_mesh(s, &m)) return -1;
  ncorner = 1 << nd;
  or_gauss(6, gp1, gw1);
  or_gauss(3, gp2, gw2);
  or_gauss(3, gp3, gw3);
  or_gauss(20, gpu1, gwu1);
  or_gauss(12, gpu2, gwu2);
  or_gauss(6, gpu3, gwu3);

  /* images: real walls first, then per wall its images in x, y, z */
  wpos = calloc((size_t)nw * 27 + 1, sizeof(*wpos));
  real = calloc((size_t)nw * 27 + 1, sizeof(int));
  for (iwall = 0; iwall < nw; iwall++) {
    for (idim = 0; idim < 3; idim++) wpos[iwall][idim] = s->wall_pos[iwall][idim];
    real[iwall] = iwall;
  }
  nimg = nw;
  for (iwall = 0; iwall < nw; iwall++) {
    for (idim = 0; idim < nd; idim++) {
      int image_old = nimg;
      for (i = 0; i < image_old; i++) {
        if (real[i] == iwall) {
          double pos[3];
          int k;
          for (k = 0; k < 3; k++) pos[k] = idim == 0 ? wpos[iwall][k] : wpos[i][k];
          or_find_wall_images(s, idim, &nimg, wpos, pos);
        }
      }
      for (i = image_old; i < nimg; i++) real[i] = iwall;
    }
  }

  rough = or_rough_tables(s);
  /* wall elements and touched faces; X_wall when a wall type is distance-based */
  wall_el = calloc((size_t)m.nels, sizeof(unsigned short));
  touch = calloc((size_t)nw + 1, sizeof(*touch));
  xwall = NULL;
  for (i = 0; i < s->ntypes; i++)
    if (s->type[i].ipot_wf == TGPU_VEXT_DIST_TO_SURF || s->type[i].ipot_wf == TGPU_VEXT_DIST_TO_CENTER) {
      long k;
      xwall = malloc((size_t)m.nnodes * nw * sizeof(double));
      for (k = 0; k < m.nnodes * nw; k++) xwall[k] = 1000.0;
      break;
    }
  for (iwall = 0; iwall < nw; iwall++) {
    const tgpu_wall_type *T = &s->type[s->wall_type[iwall]];
    for (iel = 0; iel < m.nels; iel++) {
      int ijk[3] = {0, 0, 0};
      double xtest[3] = {0.0, 0.0, 0.0}, adj;
      long r = iel;
      for (idim = 0; idim < nd; idim++) {
        ijk[idim] = (int)(r % m.els[idim]);
        r /= m.els[idim];
        xtest[idim] = (-0.5 * s->size[idim] + s->esize[idim] * ijk[idim]) + 0.5 * s->esize[idim];
      }
      adj = or_overlay(T, nd, xtest,
                       or_rough(s, T, xtest, s->wall_pos[iwall], rough + (size_t)s->wall_type[iwall] * OR_ROUGH * OR_ROUGH,
                                &bad_rough));
      if (xwall) {   /* X_wall from the nodes of this element (src/dft_surfaces.c:400-430) */
        int imax[3] = {1, 1, 1}, ix[3];
        for (idim = 0; idim < nd; idim++)
          if (ijk[idim] == m.nodes[idim] - 2 && s->bc[idim][1] != TGPU_BC_PERIODIC) imax[idim] = 2;
        for (ix[2] = 0; ix[2] < imax[2]; ix[2]++)
          for (ix[1] = 0; ix[1] < imax[1]; ix[1]++)
            for (ix[0] = 0; ix[0] < imax[0]; ix[0]++) {
              double xt[3] = {0.0, 0.0, 0.0}, delx;
              long node = 0, stride = 1;
              for (idim = 0; idim < nd; idim++) {
                xt[idim] = (-0.5 * s->size[idim] + s->esize[idim] * ijk[idim]) + ix[idim] * s->esize[idim];
                node += (ijk[idim] + ix[idim]) * stride;
                stride *= m.nodes[idim];
              }
              delx = or_surface_dist(s, T, s->wall_pos[iwall], xt, adj, T->ipot_wf == TGPU_VEXT_DIST_TO_CENTER);
              if (delx > 0.0) xwall[node * nw + iwall] = delx < xwall[node * nw + iwall] ? delx : xwall[node * nw + iwall];
              else xwall[node * nw + iwall] = 0.0;
            }
      }
      if (or_in_surface(s, T, s->wall_pos[iwall], xtest, adj) && or_angle_test(s, T, xtest, s->wall_pos[iwall])) {
        wall_el[iel] |= (unsigned short)(1u << iwall);
        for (idim = 0; idim < nd; idim++) {
          int nadd = s->bc[idim][1] == TGPU_BC_PERIODIC ? 0 : 1;
          if (ijk[idim] == 0) touch[iwall][idim][0] = 1;
          if (ijk[idim] + nadd == m.nodes[idim] - 1) touch[iwall][idim][1] = 1;
        }
      }
    }
  }

  /* zero density from the elements around each node */
  zero0 = calloc((size_t)m.nnodes, 1);
  for (inode = 0; inode < m.nnodes && nw > 0; inode++) {
    int n_fluid[TGPU_SURF_MAXWALLS], countw[TGPU_SURF_MAXWALLS], loc, iw;
    for (iw = 0; iw < nw; iw++) n_fluid[iw] = countw[iw] = 0;
    for (loc = 0; loc < ncorner; loc++) {
      int odim = 0, oside = 0;
      long e = or_node_to_elem(s, &m, inode, loc, &odim, &oside);
      for (iw = 0; iw < nw; iw++) {
        if (e >= 0) {
          if (!((wall_el[e] >> iw) & 1)) n_fluid[iw]++;
          if (wall_el[e]) countw[iw]++;
        } else if (e == -2) {
          n_fluid[iw]++;
        } else if (touch[iw][odim][oside]) {
          countw[iw]++;
        }
      }
    }
    for (iw = 0; iw < nw; iw++)
      if (countw[iw] == ncorner)
        for (i = 0; i < nw; i++) n_fluid[i] = 0;
    for (iw = 0; iw < nw; iw++)
      if (n_fluid[iw] == 0) zero0[inode] = 1;
  }

  /* setup_vext_max / setup_zero */
  for (icomp = 0; icomp < s->ncomp; icomp++)
    for (inode = 0; inode < m.nnodes; inode++)
      vext[icomp * m.nnodes + inode] = zero0[inode] ? s->vext_max : 0.0;

  /* the walls and their images in image order (setup_external_field_n, src/dft_vext.c:108-140):
   * setup_vext_XRSurf for every image of a distance-based type, setup_integrated_LJ_walls for every real
   * wall of integrated type */
  for (k_img = 0; k_img < nimg; k_img++) {
    const tgpu_wall_type *T = &s->type[s->wall_type[real[k_img]]];
    double max_cut = 0.0;
    iwall = k_img;
    if (T->ipot_wf == TGPU_VEXT_DIST_TO_SURF || T->ipot_wf == TGPU_VEXT_DIST_TO_CENTER) {
      for (icomp = 0; icomp < s->ncomp; icomp++)
        for (inode = 0; inode < m.nnodes; inode++) {
          double *V = &vext[icomp * m.nnodes + inode], xORr;
          if (zero0[inode]) continue;
          xORr = k_img < nw ? xwall[inode * nw + k_img] : 1000.0;
          if (fabs(*V - s->vext_max) > 1.e-6) {
            if (xORr > 0.001) *V += or_vext_1d(s, T, icomp, xORr);
            else *V = s->vext_max;
          }
          if (*V >= s->vext_max) *V = s->vext_max;
        }
      continue;
    }
    if (T->ipot_wf != TGPU_VEXT_INTEGRATED || k_img >= nw) continue;
    for (icomp = 0; icomp < s->ncomp; icomp++)
      if (max_cut < T->cut_wf[icomp]) max_cut = T->cut_wf[icomp];
    for (iel = 0; iel < m.nels; iel++) {
      int nghost = 0, ghost_dim = 0, iwall_images, ijk[3] = {0, 0, 0};
      double node_pos[3] = {0.0, 0.0, 0.0}, del_ghost = 0.0;
      long r = iel;
      if (!((wall_el[iel] >> iwall) & 1)) continue;
      for (idim = 0; idim < nd; idim++) {
        ijk[idim] = (int)(r % m.els[idim]);
        r /= m.els[idim];
        node_pos[idim] = -0.5 * s->size[idim] + s->esize[idim] * ijk[idim];
      }
      for (idim = 0; idim < nd; idim++) node_pos[idim] += 0.5 * s->esize[idim];
      for (iwall_images = 0; iwall_images < nimg; iwall_images++) {
        double node_pos_w[3] = {0.0, 0.0, 0.0}, node_pos_w_save[3], delta[3];
        int halfsurf = 0, jwall, ighost;
        if (real[iwall_images] != iwall) continue;
        for (idim = 0; idim < nd; idim++) delta[idim] = node_pos[idim] - wpos[iwall][idim];
        for (jwall = 0; jwall < iwall_images; jwall++) {
          if (real[jwall] == iwall) {
            halfsurf = 1;
            for (idim = 0; idim < nd; idim++)
              if (wpos[iwall_images][idim] != wpos[jwall][idim]) halfsurf = 0;
            if (halfsurf) jwall = iwall_images;
          }
        }
        if (iwall_images < nw) halfsurf = 0;
        for (idim = 0; idim < nd; idim++) {
          double pic = wpos[iwall_images][idim], prc = wpos[iwall][idim];
          if (pic > prc || (halfsurf && fabs(pic - s->size[idim] / 2.) < 1.e-5)) {
            if (s->bc[idim][1] == TGPU_BC_PERIODIC) node_pos_w[idim] = pic + delta[idim];
            else if (s->bc[idim][1] == TGPU_BC_REFLECT) node_pos_w[idim] = pic - delta[idim];
            else return -1;
          } else if (pic < prc || (halfsurf && fabs(pic + s->size[idim] / 2.) < 1.e-5)) {
            if (s->bc[idim][0] == TGPU_BC_PERIODIC) node_pos_w[idim] = pic + delta[idim];
            else if (s->bc[idim][0] == TGPU_BC_REFLECT) node_pos_w[idim] = pic - delta[idim];
            else return -1;
          } else {
            node_pos_w[idim] = node_pos[idim];
          }
          if ((s->bc[idim][0] == TGPU_BC_IN_WALL || s->bc[idim][0] == TGPU_BC_LAST_NODE ||
               s->bc[idim][0] == TGPU_BC_LAST_NODE_RESTART) &&
              fabs(node_pos[idim] - 0.5 * s->esize[idim] + s->size[idim] / 2.) < 1.e-6) {
            nghost = (int)(max_cut / s->esize[idim]);
            del_ghost = -s->esize[idim];
            ghost_dim = idim;
          } else if ((s->bc[idim][1] == TGPU_BC_IN_WALL || s->bc[idim][1] == TGPU_BC_LAST_NODE ||
                      s->bc[idim][1] == TGPU_BC_LAST_NODE_RESTART) &&
                     fabs(node_pos[idim] + 0.5 * s->esize[idim] - s->size[idim] / 2) < 1.e-6) {
            nghost = (int)(max_cut / s->esize[idim]);
            del_ghost = s->esize[idim];
            ghost_dim = idim;
          }
        }
        for (idim = 0; idim < nd; idim++) {
          node_pos_w[idim] -= 0.5 * s->esize[idim];
          node_pos_w_save[idim] = node_pos_w[idim];
        }
        for (inode = 0; inode < m.nnodes; inode++) {
          for (ighost = 0; ighost <= nghost; ighost++) {
            if (ighost > 0) node_pos_w[ghost_dim] = node_pos_w_save[ghost_dim] + ighost * del_ghost;
            for (icomp = 0; icomp < s->ncomp; icomp++) {
              double *V = &vext[icomp * m.nnodes + inode], fpos[3], r_center_sq = 0.0;
              if (zero0[inode]) continue;
              if (!(*V < s->vext_max || *V == 0.0)) continue;
              or_node_pos(s, &m, inode, fpos);
              for (idim = 0; idim < nd; idim++)
                r_center_sq += (node_pos_w[idim] - fpos[idim]) * (node_pos_w[idim] - fpos[idim]);
              if (r_center_sq < (max_cut + 0.0) * max_cut + 0.0) {
                int ngp, ngpu;
                const double *gp, *gpu, *gw, *gwu;
                if (r_center_sq < 4.0) { ngp = 6; ngpu = 20; gp = gp1; gpu = gpu1; gw = gw1; gwu = gwu1; }
                else if (r_center_sq < 16.0) { ngp = 3; ngpu = 12; gp = gp2; gpu = gpu2; gw = gw2; gwu = gwu2; }
                else { ngp = 3; ngpu = 6; gp = gp3; gpu = gpu3; gw = gw3; gwu = gwu3; }
                *V += or_integrate(s, m.vol_el, T->sigma_wf[icomp], T->eps_wf[icomp], T->cut_wf[icomp], ngp, ngpu, gp,
                                   gpu, gw, gwu, node_pos_w, fpos);
                if (*V >= s->vext_max) *V = s->vext_max;
              }
            }
          }
          for (idim = 0; idim < nd; idim++) node_pos_w[idim] = node_pos_w_save[idim];
        }
      }
    }
  }
  for (icomp = 0; icomp < s->ncomp; icomp++)
    for (inode = 0; inode < m.nnodes; inode++)
      zero[icomp * m.nnodes + inode] = vext[icomp * m.nnodes + inode] >= s->vext_max ? 1 : 0;
  if (wall_el_out) memcpy(wall_el_out, wall_el, (size_t)m.nels * sizeof(unsigned short));
  free(wall_el);
  free(touch);
  free(xwall);
  free(rough);
  if (bad_rough) return -1;
  free(zero0);
  free(wpos);
  free(real);
  return 0;
}
