"""Surfaces and their external fields, built on the GPU (tgpu_surface_field_*, csrc/surfaces.cu).

A reference user describes walls in the input deck (dft_input.dat: mesh, boundaries, the surface
and wall-fluid sections) and their positions in dft_surfaces.dat.  :func:`read_deck` reads those
sections into a :class:`SurfaceSpec`; :func:`surface_field` returns the external field V_ext/kT
[ncomp][nodes], the zero-density flags [ncomp][nodes] and the walls of every element, as the
reference's set-up computes them (setup_surface, src/dft_surfaces.c:39; setup_external_field_n,
src/dft_vext.c:38; setup_integrated_LJ_walls, src/dft_vext.c:671).  :func:`problem_fields` gives
them in the layout build_problem takes.

The deck is read by the labels of its '@' lines, as the reference's input reader reads fields in
order (src/dft_input.c): the wall-fluid parameters follow its mixing rules (Lorentz-Berthelot for
Mix_type 0, src/dft_potential_params.c:120-125; the deck's values for Mix_type 1).  Parts of the
deck this path does not build (Lhard_surf, the charged and Yukawa 1-D wall forms, pair potentials other
than LJ 12-6, a positive Temp or Length_ref) raise NotImplementedError.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

from . import native

MAXC, MAXWALLS, MAXTYPES, MAXFNC = 4, 16, 16, 4
SURF_PLANAR, SURF_BLOCK, SURF_COLLOID, SURF_FINITE_CYL, SURF_PORE, SURF_FINITE_PORE = 0, 1, 2, 5, 7, 8
VEXT_NONE, VEXT_HARD, VEXT_DIST_TO_SURF, VEXT_DIST_TO_CENTER, VEXT_INTEGRATED = 0, 1, 2, 3, 5
WALL1D_LJ93_CS, WALL1D_LJ93_V2_CS, WALL1D_LJ93_NOCS, WALL1D_LJ93_SHIFTX_CS, WALL1D_REPULSIVE9, WALL1D_EXP_ATT = range(6)
BC_IN_WALL, BC_IN_BULK, BC_PERIODIC, BC_REFLECT, BC_LAST_NODE, BC_LAST_NODE_RESTART = -1, 0, 1, 2, 3, 4


class WallType(C.Structure):
    _fields_ = [("surf_type", C.c_int), ("orientation", C.c_int), ("param", C.c_double * 3),
                ("nperiodic", C.c_int), ("periodic_orient", C.c_int * MAXFNC), ("amplitude", C.c_double * MAXFNC),
                ("wavelength", C.c_double * MAXFNC), ("periodic_origin", C.c_double * MAXFNC),
                ("nlinear", C.c_int), ("linear_orient", C.c_int * MAXFNC), ("slope", C.c_double * MAXFNC),
                ("linear_origin", C.c_double * MAXFNC), ("linear_end", C.c_double * MAXFNC),
                ("cutout", C.c_int), ("angle_start", C.c_double), ("angle_end", C.c_double),
                ("rough", C.c_int), ("rough_max", C.c_double), ("rough_length", C.c_double),
                ("ipot_wf", C.c_int), ("type_vext", C.c_int), ("pot_id", C.c_int), ("rho_w", C.c_double),
                ("sigma_wf", C.c_double * MAXC), ("eps_wf", C.c_double * MAXC), ("cut_wf", C.c_double * MAXC)]


class SurfaceSpec(C.Structure):
    """tgpu_surface_spec (include/tramonto_gpu.h)."""
    _fields_ = [("ndim", C.c_int), ("size", C.c_double * 3), ("esize", C.c_double * 3),
                ("bc", (C.c_int * 2) * 3), ("ncomp", C.c_int), ("vext_max", C.c_double),
                ("sigma_ff", C.c_double * MAXC), ("apply_offset", C.c_int * 3), ("ntypes", C.c_int), ("type", WallType * MAXTYPES),
                ("nwalls", C.c_int), ("wall_type", C.c_int * MAXWALLS), ("wall_pos", (C.c_double * 3) * MAXWALLS)]

    def mesh(self):
        """(nodes[3], elements[3]) of the spec's mesh (unused dimensions 1)."""
        lib = native.load()
        nodes, els = (C.c_int * 3)(), (C.c_int * 3)()
        native._check(lib.tgpu_surface_mesh(C.byref(self), nodes, els), lib)
        return list(nodes), list(els)


def make_spec(ndim, size, esize, bc, ncomp, walls, types, vext_max=10.0, apply_offset=(0, 0, 0), sigma_ff=None):
    """A SurfaceSpec from plain values: bc [(lo, hi)] per dimension; types a list of dicts (surf_type,
    orientation, param, ipot_wf, type_vext (default 1 for integrated walls, else 0), pot_id, rho_w, sigma_wf,
    eps_wf, cut_wf per component, optional periodic / linear lists of (orientation, amplitude, wavelength,
    origin) / (orientation, slope, origin, end)); walls a list of (type index, position); sigma_ff the
    fluid diameters Sigma_ff[i][i]."""
    s = SurfaceSpec()
    s.ndim, s.ncomp, s.vext_max = int(ndim), int(ncomp), float(vext_max)
    for c in range(ncomp):
        s.sigma_ff[c] = float(sigma_ff[c]) if sigma_ff is not None else 1.0
    for d in range(3):
        s.size[d] = float(size[d]) if d < ndim else 0.0
        s.esize[d] = float(esize[d]) if d < ndim else 0.0
        lo, hi = bc[d] if d < ndim else (BC_IN_BULK, BC_IN_BULK)
        s.bc[d][0], s.bc[d][1] = int(lo), int(hi)
        s.apply_offset[d] = int(apply_offset[d])
    if len(types) > MAXTYPES or len(walls) > MAXWALLS or ncomp > MAXC:
        raise ValueError("too many wall types, walls or components")
    s.ntypes = len(types)
    for t, T in enumerate(types):
        o = s.type[t]
        o.surf_type, o.orientation = int(T["surf_type"]), int(T.get("orientation", 0))
        for k, v in enumerate(T.get("param", (0.0, 0.0, 0.0))[:3]):
            o.param[k] = float(v)
        per = T.get("periodic", [])
        lin = T.get("linear", [])
        if len(per) > MAXFNC or len(lin) > MAXFNC:
            raise ValueError("too many overlay functions")
        o.nperiodic = len(per)
        for i, (ori, amp, wl, org) in enumerate(per):
            o.periodic_orient[i], o.amplitude[i], o.wavelength[i], o.periodic_origin[i] = int(ori), amp, wl, org
        o.nlinear = len(lin)
        for i, (ori, sl, org, end) in enumerate(lin):
            o.linear_orient[i], o.slope[i], o.linear_origin[i], o.linear_end[i] = int(ori), sl, org, end
        o.cutout = int(T.get("cutout", 0))
        o.angle_start = float(T.get("angle_start", 0.0))
        o.angle_end = float(T.get("angle_end", 0.0))
        o.rough = int(T.get("rough", 0))
        o.rough_max = float(T.get("rough_max", 0.0))
        o.rough_length = float(T.get("rough_length", 0.0))
        o.ipot_wf = int(T.get("ipot_wf", VEXT_HARD))
        o.type_vext = int(T.get("type_vext", 1 if o.ipot_wf == VEXT_INTEGRATED else 0))
        o.pot_id = int(T.get("pot_id", 0))
        o.rho_w = float(T.get("rho_w", 1.0))
        for c in range(ncomp):
            o.sigma_wf[c] = float(T.get("sigma_wf", [0.0] * ncomp)[c])
            o.eps_wf[c] = float(T.get("eps_wf", [0.0] * ncomp)[c])
            o.cut_wf[c] = float(T.get("cut_wf", [0.0] * ncomp)[c])
    s.nwalls = len(walls)
    for w, (t, pos) in enumerate(walls):
        s.wall_type[w] = int(t)
        for d in range(3):
            s.wall_pos[w][d] = float(pos[d]) if d < len(pos) else 0.0
    return s


def surface_field(spec: SurfaceSpec):
    """V_ext/kT [ncomp][nodes], zero-density flags [ncomp][nodes] (int8) and the wall bit mask of every
    element [elements] (uint16), computed on the GPU."""
    nodes, els = spec.mesh()
    n, ne = int(np.prod(nodes)), int(np.prod(els))
    vext = np.zeros((spec.ncomp, n))
    zero = np.zeros((spec.ncomp, n), np.int8)
    wall_el = np.zeros(ne, np.uint16)
    lib = native.load()
    native._check(lib.tgpu_surface_field_host(C.byref(spec), vext.ctypes.data, zero.ctypes.data,
                                              wall_el.ctypes.data), lib)
    return vext, zero, wall_el


# ---- reading the surface part of a reference input deck ----------------------------------------------

def _deck_fields(text):
    """[(values, label)] of the '@' records: the text from one '@' to the next (the reference's reader
    continues a list of values onto the following lines); values are the leading numeric tokens (n/a as
    None), the label the rest."""
    out = []
    records = []
    for line in text.splitlines():
        if line.startswith("@"):
            records.append(line[1:])
        elif records:
            records[-1] += " " + line
    for rec in records:
        toks = rec.split()
        vals, k = [], 0
        for k, t in enumerate(toks):
            if t.lower() == "n/a":
                vals.append(None)
                continue
            try:
                vals.append(float(t))
            except ValueError:
                break
        else:
            k = len(toks)
        out.append((vals, " ".join(toks[k:])))
    return out


class _Deck:
    def __init__(self, text):
        self.fields = _deck_fields(text)

    def get(self, key, n=None):
        """the values of the one line whose label starts with key (or, for a key in parentheses, holds it)"""
        if key.startswith("("):
            hits = [v for v, lab in self.fields if key[1:-1] in lab]
        else:
            hits = [v for v, lab in self.fields if lab.startswith(key)]
        if len(hits) != 1:
            raise KeyError(f"deck label {key!r} matched {len(hits)} lines")
        return self._take(hits[0], n)

    @staticmethod
    def _take(v, n):
        # a line with fewer values than asked for: the reference's reads of the missing ones fail and leave
        # its zero-initialised arrays unchanged
        if n is None:
            return v
        v = [0.0 if x is None else x for x in v[:n]]
        return v + [0.0] * (n - len(v))

    def after(self, key, k, n):
        """the values of the k-th '@' line after the one labelled key: the reference reads these lines in
        order, and some decks leave them unlabelled"""
        idx = [i for i, (_, lab) in enumerate(self.fields) if lab.startswith(key)]
        if len(idx) != 1:
            raise KeyError(f"deck label {key!r} matched {len(idx)} lines")
        return self._take(self.fields[idx[0] + k][0], n)


def read_deck(input_path, surfaces_path=None):
    """A SurfaceSpec from a reference input deck (dft_input.dat) and its wall positions
    (dft_surfaces.dat beside it unless surfaces_path is given)."""
    with open(input_path) as f:
        dk = _Deck(f.read())
    if surfaces_path is None:
        surfaces_path = os.path.join(os.path.dirname(os.path.abspath(input_path)), "dft_surfaces.dat")
    length_ref, _, temp, _, vext_max = dk.get("Length_ref", 5)
    if (length_ref is not None and length_ref > 0) or (temp is not None and temp > 0):
        raise NotImplementedError("dimensioned units (Length_ref or Temp > 0)")
    ndim = int(dk.get("Ndim", 1)[0])
    size = dk.get("Size_x", ndim)
    esize = dk.get("Esize_x", ndim)
    bc = [tuple(int(v) for v in dk.get(f"Type_bc(x{d}", 2)) for d in range(ndim)]
    ntypes, nwalls, _, auto_center, auto_size = (int(v) for v in dk.get("Nwall_types Nwall", 5))
    if auto_size:
        raise NotImplementedError("Lauto_size")
    surf = [int(v) for v in dk.get("Surf_type", ntypes)]
    orient = [int(v) for v in dk.get("Orientation[iwall_type]", ntypes)]
    p1 = dk.get("WallParam[", ntypes)
    p2 = dk.get("WallParam2", ntypes)
    p3 = dk.get("WallParam3", ntypes)
    apply = [int(v) for v in dk.get("Lapply_of", 3)]
    rough = [int(v) for v in dk.get("Lrough_surf", ntypes)]
    rough_max = dk.get("rough_param_max", ntypes) if any(rough) else [0.0] * ntypes
    rough_len = dk.get("Rough_length", ntypes) if any(rough) else [0.0] * ntypes
    nper = [int(v) for v in dk.get("Nperiodic_overlay", ntypes)]
    nlin = [int(v) for v in dk.get("Nlinear_overlay", ntypes)]
    cutout = [int(v) for v in dk.get("LangleCutout", ntypes)]
    a_start = dk.get("Angle_start", ntypes) if any(cutout) else [0.0] * ntypes
    a_end = dk.get("Angle_end", ntypes) if any(cutout) else [0.0] * ntypes

    def per_type(key, counts):
        if sum(counts) == 0:
            return [[] for _ in counts]
        vals = dk.get(key, sum(counts))
        out, k = [], 0
        for c in counts:
            out.append(vals[k:k + c])
            k += c
        return out

    p_or = per_type("OrientationPeriodic", nper)
    p_amp = per_type("Amplitude[", nper)
    p_wl = per_type("Period[", nper)
    p_org = per_type("Origin[iwall_type]", nper)
    l_or = per_type("OrientationLinear", nlin)
    l_sl = per_type("Slope[", nlin)
    l_org = per_type("Origin_linear", nlin)
    l_end = per_type("Endpoint_linear", nlin)
    ipot = [int(v) for v in dk.get("(Ipot_wf_n)", ntypes)]
    if int(dk.get("Lhard_surf", 1)[0]):
        raise NotImplementedError("Lhard_surf")
    tvext = [int(v) for v in dk.get("Type_vext[", ntypes)]
    potid = [int(v) for v in dk.get("Vext_PotentialID", ntypes)]
    ncomp, mix = (int(v) for v in dk.get("Ncomp Mix_type", 2))
    for t in range(ntypes):
        if ipot[t] not in (VEXT_NONE, VEXT_HARD, VEXT_DIST_TO_SURF, VEXT_DIST_TO_CENTER, VEXT_INTEGRATED):
            raise NotImplementedError(f"Ipot_wf_n = {ipot[t]}")
        if ipot[t] == VEXT_INTEGRATED and (tvext[t] != 1 or potid[t] != 0):
            raise NotImplementedError("integrated walls other than the LJ 12-6 pair potential")
        if ipot[t] in (VEXT_DIST_TO_SURF, VEXT_DIST_TO_CENTER) and (potid[t] != 0 if tvext[t] == 1 else potid[t] > 5):
            raise NotImplementedError("distance-based walls other than the 1-D forms 0-5 and the LJ 12-6 pair potential")
    nff = ncomp if mix == 0 else ncomp * ncomp
    nww = ntypes if mix == 0 else ntypes * ntypes
    sff_all = dk.get("Sigma_ff", nff)
    sigma_ff = [sff_all[i] if mix == 0 else sff_all[i * ncomp + i] for i in range(ncomp)]
    rho_w = dk.get("Rho_w", ntypes)
    # after Rho_w: Sigma_ww, Eps_ww, Cut_ww, EpsYukawa_ww, YukawaK_ww, Sigma_wf, Eps_wf, Cut_wf (src/dft_input.c)
    if mix == 0:
        sff = dk.get("Sigma_ff", nff)
        eff = dk.get("Eps_ff", nff)
        cff = dk.get("Cut_ff", nff)
        sww = dk.after("Rho_w", 1, nww)
        eww = dk.after("Rho_w", 2, nww)
        cww = dk.after("Rho_w", 3, nww)
        # Lorentz-Berthelot (src/dft_potential_params.c:120-125)
        swf = [[0.5 * (sff[i] + sww[t]) for i in range(ncomp)] for t in range(ntypes)]
        ewf = [[math.sqrt(eff[i] * eww[t]) for i in range(ncomp)] for t in range(ntypes)]
        cwf = [[0.5 * (cff[i] + cww[t]) for i in range(ncomp)] for t in range(ntypes)]
    else:
        nwf = ncomp * ntypes
        s_in, e_in, c_in = dk.after("Rho_w", 6, nwf), dk.after("Rho_w", 7, nwf), dk.after("Rho_w", 8, nwf)
        swf = [[s_in[i * ntypes + t] for i in range(ncomp)] for t in range(ntypes)]
        ewf = [[e_in[i * ntypes + t] for i in range(ncomp)] for t in range(ntypes)]
        cwf = [[c_in[i * ntypes + t] for i in range(ncomp)] for t in range(ntypes)]
    types = []
    for t in range(ntypes):
        types.append(dict(surf_type=surf[t], orientation=orient[t], param=(p1[t], p2[t], p3[t]), ipot_wf=ipot[t],
                          type_vext=tvext[t], pot_id=potid[t], rho_w=rho_w[t], rough=rough[t],
                          cutout=cutout[t], angle_start=a_start[t], angle_end=a_end[t],
                          rough_max=rough_max[t], rough_length=rough_len[t],
                          sigma_wf=swf[t], eps_wf=ewf[t], cut_wf=cwf[t],
                          periodic=[(int(p_or[t][i]), p_amp[t][i], p_wl[t][i], p_org[t][i]) for i in range(nper[t])],
                          linear=[(int(l_or[t][i]), l_sl[t][i], l_org[t][i], l_end[t][i]) for i in range(nlin[t])]))
    with open(surfaces_path) as f:
        toks = f.read().split()
    walls, k = [], 0
    for _ in range(nwalls):
        wt = int(toks[k])
        pos = [float(toks[k + 2 + d]) for d in range(ndim)]
        walls.append((wt, pos))
        k += 2 + ndim + 1          # type, link, position, Elec_param_w
    if auto_center:
        lo = [min(w[1][d] for w in walls) for d in range(ndim)]
        hi = [max(w[1][d] for w in walls) for d in range(ndim)]
        walls = [(t, [p[d] - 0.5 * (hi[d] + lo[d]) for d in range(ndim)]) for t, p in walls]
    return make_spec(ndim, size, esize, bc, ncomp, walls, types, vext_max=vext_max, apply_offset=apply,
                     sigma_ff=sigma_ff)


def rough_table(spec: SurfaceSpec):
    """The roughness patch heights [ntypes][100][100] the builder uses (Rough_precalc)."""
    out = np.zeros((max(spec.ntypes, 1), 100, 100))
    lib = native.load()
    native._check(lib.tgpu_surface_rough_table(C.byref(spec), out.ctypes.data), lib)
    return out[:spec.ntypes]


def problem_fields(spec: SurfaceSpec):
    """(vext, zero_density) for build_problem: V_ext/kT [ncomp][nodes] and int8 flags."""
    vext, zero, _ = surface_field(spec)
    return vext, zero


def spec_arrays(spec: SurfaceSpec) -> dict:
    """The spec as named numpy arrays (for storing next to results); spec_from_arrays inverts it."""
    nt, nw = spec.ntypes, spec.nwalls
    a = {"ndim": np.int32(spec.ndim), "size": np.array(spec.size[:]), "esize": np.array(spec.esize[:]),
         "bc": np.array([[spec.bc[d][0], spec.bc[d][1]] for d in range(3)], np.int32),
         "ncomp": np.int32(spec.ncomp), "vext_max": np.float64(spec.vext_max),
         "apply_offset": np.array(spec.apply_offset[:], np.int32),
         "wall_type": np.array(spec.wall_type[:nw], np.int32),
         "wall_pos": np.array([spec.wall_pos[w][:] for w in range(nw)]).reshape(nw, 3)}
    a["sigma_ff"] = np.array(spec.sigma_ff[:])
    for f in ("surf_type", "orientation", "nperiodic", "nlinear", "ipot_wf", "type_vext", "pot_id", "rough",
              "cutout"):
        a["t_" + f] = np.array([getattr(spec.type[t], f) for t in range(nt)], np.int32)
    for f in ("rho_w", "rough_max", "rough_length", "angle_start", "angle_end"):
        a["t_" + f] = np.array([getattr(spec.type[t], f) for t in range(nt)])
    for f in ("periodic_orient", "linear_orient"):
        a["t_" + f] = np.array([getattr(spec.type[t], f)[:] for t in range(nt)], np.int32).reshape(nt, MAXFNC)
    for f, n in (("param", 3), ("amplitude", MAXFNC), ("wavelength", MAXFNC), ("periodic_origin", MAXFNC),
                 ("slope", MAXFNC), ("linear_origin", MAXFNC), ("linear_end", MAXFNC), ("sigma_wf", MAXC),
                 ("eps_wf", MAXC), ("cut_wf", MAXC)):
        a["t_" + f] = np.array([getattr(spec.type[t], f)[:] for t in range(nt)]).reshape(nt, n)
    return a


def spec_from_arrays(a) -> SurfaceSpec:
    s = SurfaceSpec()
    s.ndim, s.ncomp, s.vext_max = int(a["ndim"]), int(a["ncomp"]), float(a["vext_max"])
    for d in range(3):
        s.size[d], s.esize[d] = float(a["size"][d]), float(a["esize"][d])
        s.bc[d][0], s.bc[d][1] = int(a["bc"][d][0]), int(a["bc"][d][1])
        s.apply_offset[d] = int(a["apply_offset"][d])
    for c, v in enumerate(a["sigma_ff"] if "sigma_ff" in a else [1.0] * MAXC):
        s.sigma_ff[c] = float(v)
    nt = len(a["t_surf_type"])
    s.ntypes = nt
    for t in range(nt):
        o = s.type[t]
        for f in ("surf_type", "orientation", "nperiodic", "nlinear", "ipot_wf"):
            setattr(o, f, int(a["t_" + f][t]))
        # arrays stored before the distance-based walls: integrated LJ 12-6 walls (Type_vext 1, potential 0)
        o.type_vext = int(a["t_type_vext"][t]) if "t_type_vext" in a else 1
        o.pot_id = int(a["t_pot_id"][t]) if "t_pot_id" in a else 0
        o.rho_w = float(a["t_rho_w"][t]) if "t_rho_w" in a else 1.0
        o.cutout = int(a["t_cutout"][t]) if "t_cutout" in a else 0
        o.angle_start = float(a["t_angle_start"][t]) if "t_angle_start" in a else 0.0
        o.angle_end = float(a["t_angle_end"][t]) if "t_angle_end" in a else 0.0
        o.rough = int(a["t_rough"][t]) if "t_rough" in a else 0
        o.rough_max = float(a["t_rough_max"][t]) if "t_rough_max" in a else 0.0
        o.rough_length = float(a["t_rough_length"][t]) if "t_rough_length" in a else 0.0
        for f in ("periodic_orient", "linear_orient", "param", "amplitude", "wavelength", "periodic_origin", "slope",
                  "linear_origin", "linear_end", "sigma_wf", "eps_wf", "cut_wf"):
            arr = getattr(o, f)
            for i, v in enumerate(a["t_" + f][t]):
                arr[i] = v
    nw = len(a["wall_type"])
    s.nwalls = nw
    for w in range(nw):
        s.wall_type[w] = int(a["wall_type"][w])
        for d in range(3):
            s.wall_pos[w][d] = float(a["wall_pos"][w][d])
    return s
