"""ctypes binding of the C restatement oracle (oracle.c); test infrastructure.

``build()`` compiles oracle.c with the host C compiler into oracle/_build.
``Oracle(problem)`` takes any object with the problem attributes used by the
product (see tramonto_gb300.problem.Problem: geometry, constants, fields and
stencil tables) and exposes the oracle's residual, Jacobian products and
Schur product on numpy arrays shaped [unknown][node].
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
MAXC = 4
MAXZ = 5


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, "oracle.c"), os.path.join(HERE, "surfaces.c")]
    deps = srcs + [os.path.join(HERE, "oracle.h"), os.path.join(HERE, "..", "include", "tramonto_gpu.h")]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(f) for f in deps):
        os.makedirs(BUILD, exist_ok=True)
        tmp = LIB + f".tmp{os.getpid()}"
        # no contraction of multiply-adds: the surface restatement keeps the reference's operations
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c99", "-ffp-contract=off", "-o", tmp, *srcs, "-lm"],
                       check=True)
        os.replace(tmp, LIB)
    return LIB


def surface_field(spec):
    """The restatement of the reference's surface set-up (oracle/surfaces.c) for a tramonto_gb300.surfaces
    SurfaceSpec: (V_ext [ncomp][nodes], zero flags [ncomp][nodes] int8, element wall masks uint16)."""
    lib = C.CDLL(build())
    nodes, els = [1, 1, 1], [1, 1, 1]
    for d in range(spec.ndim):
        nodes[d] = int(np.floor(spec.size[d] / spec.esize[d] + 1.0 + 0.5))
        els[d] = nodes[d] - 1
        if spec.bc[d][0] == 1 and spec.bc[d][1] == 1:
            nodes[d] -= 1
    n, ne = int(np.prod(nodes)), int(np.prod(els))
    vext = np.zeros((spec.ncomp, n))
    zero = np.zeros((spec.ncomp, n), np.int8)
    wall_el = np.zeros(ne, np.uint16)
    fn = lib.oracle_surface_field
    fn.argtypes = [C.c_void_p] * 4
    fn.restype = C.c_int
    if fn(C.addressof(spec), vext.ctypes.data, zero.ctypes.data, wall_el.ctypes.data) != 0:
        raise ValueError("the surface restatement does not cover this spec")
    return vext, zero, wall_el


class _Problem(C.Structure):
    _fields_ = [
        ("ndim", C.c_int), ("nx", C.c_int * 3), ("esize", C.c_double * 3), ("bc", (C.c_int * 2) * 3),
        ("ncomp", C.c_int), ("functional", C.c_int), ("attraction", C.c_int), ("att_in_a22", C.c_int),
        ("single_size", C.c_int), ("hard_surf", C.c_int), ("nlists_hw", C.c_int),
        ("first_rho", C.c_int), ("first_rb", C.c_int), ("first_mf", C.c_int), ("nunk", C.c_int),
        ("rho_b", C.c_double * MAXC), ("betamu_hs_ex", C.c_double * MAXC), ("betamu_att", C.c_double * MAXC),
        ("inv_rad", C.c_double * MAXC), ("inv_4pir", C.c_double * MAXC), ("inv_4pirsq", C.c_double * MAXC),
        ("fac_overlap", C.c_double * MAXC), ("dphi_bulk", C.c_double * 4), ("vext_max", C.c_double),
        ("vext", C.POINTER(C.c_double)), ("zero_density", C.POINTER(C.c_int8)),
        ("boundary_nodes", C.POINTER(C.c_int)), ("fluid_masks", C.POINTER(C.c_int16)),
        ("sten_len", (C.c_int * (MAXC * MAXC)) * 3),
        ("sten_off", (C.POINTER(C.c_int16) * (MAXC * MAXC)) * 3),
        ("sten_w", (C.POINTER(C.c_double) * (MAXC * MAXC)) * 3),
        ("sten_hw", (C.POINTER(C.c_double) * (MAXC * MAXC)) * 3),
        ("interface", C.c_int), ("rho_b_lbb", C.c_double * MAXC), ("rho_b_rtf", C.c_double * MAXC),
        ("dphi_lbb", C.c_double * 4), ("dphi_rtf", C.c_double * 4), ("betamu", C.c_double * MAXC),
        ("pin_node", C.c_long), ("pin_value", C.c_double),
        ("nzone", C.c_int), ("mesh_coarsening", C.c_int), ("coarser_jac", C.c_int), ("nwall", C.c_int),
        ("zone_flag", C.POINTER(C.c_int)),
        ("zsten_len", ((C.c_int * (MAXC * MAXC)) * 3) * MAXZ),
        ("zsten_off", ((C.POINTER(C.c_int16) * (MAXC * MAXC)) * 3) * MAXZ),
        ("zsten_w", ((C.POINTER(C.c_double) * (MAXC * MAXC)) * 3) * MAXZ),
        ("zsten_hw", ((C.POINTER(C.c_double) * (MAXC * MAXC)) * 3) * MAXZ),
        ("rhobar_bc", C.c_double * 10),
        ("l1d_bc", C.c_int), ("dim_1dbc", C.c_int),
        ("rhobar_lbb", C.c_double * 10), ("rhobar_rtf", C.c_double * 10),
    ]


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    def __init__(self, prob):
        self.lib = C.CDLL(build())
        for fn in ("orc_resid", "orc_jv", "orc_jtv", "orc_schur", "orc_dphi", "orc_resid_rows"):
            getattr(self.lib, fn).restype = C.c_int
        self.prob = prob
        self._keep = []
        s = _Problem()
        s.ndim = prob.ndim
        for d in range(3):
            s.nx[d] = int(prob.nx[d]) if d < prob.ndim else 1
            s.esize[d] = float(prob.esize[d]) if d < prob.ndim else 0.0
            for k in range(2):
                s.bc[d][k] = int(prob.bc[d][k]) if d < prob.ndim else 0
        for name in ("ncomp", "functional", "attraction", "att_in_a22", "single_size", "hard_surf", "nlists_hw",
                     "first_rho", "first_rb", "first_mf", "nunk"):
            setattr(s, name, int(getattr(prob, name)))
        for name in ("rho_b", "betamu_hs_ex", "betamu_att", "inv_rad", "inv_4pir", "inv_4pirsq", "fac_overlap"):
            arr = getattr(s, name)
            vals = np.asarray(getattr(prob, name), np.float64)
            for i in range(min(len(vals), MAXC)):
                arr[i] = vals[i]
        for i in range(4):
            s.dphi_bulk[i] = float(prob.dphi_bulk[i])
        s.vext_max = float(prob.vext_max)
        s.interface = int(getattr(prob, "interface", 0))
        s.pin_node = -1
        if s.interface:
            for name, src in (("rho_b_lbb", prob.rho_b_lbb), ("rho_b_rtf", prob.rho_b_rtf), ("dphi_lbb", prob.dphi_lbb),
                              ("dphi_rtf", prob.dphi_rtf), ("betamu", prob.betamu_if)):
                arr = getattr(s, name)
                for i, v in enumerate(np.asarray(src, np.float64)[:4]):
                    arr[i] = float(v)
            s.pin_node = int(prob.pin_node)
            s.pin_value = float(prob.pin_value)
        self.N = int(np.prod([prob.nx[d] for d in range(prob.ndim)]))
        vext = np.ascontiguousarray(prob.vext, np.float64)
        zd = np.ascontiguousarray(prob.zero_density, np.int8)
        self._keep += [vext, zd]
        s.vext = _dp(vext)
        s.zero_density = zd.ctypes.data_as(C.POINTER(C.c_int8))
        if prob.hard_surf:
            bn = np.ascontiguousarray(prob.boundary_nodes, np.int32)
            fm = np.ascontiguousarray(prob.fluid_masks, np.int16)
            self._keep += [bn, fm]
            s.boundary_nodes = bn.ctypes.data_as(C.POINTER(C.c_int))
            s.fluid_masks = fm.ctypes.data_as(C.POINTER(C.c_int16))
        for (stype, idx), (off, w, hw) in prob.stencils.items():
            off = np.ascontiguousarray(off, np.int16)
            w = np.ascontiguousarray(w, np.float64)
            self._keep += [off, w]
            s.sten_len[stype][idx] = len(w)
            s.sten_off[stype][idx] = off.ctypes.data_as(C.POINTER(C.c_int16))
            s.sten_w[stype][idx] = _dp(w)
            if hw is not None:
                hw = np.ascontiguousarray(hw, np.float64)
                self._keep.append(hw)
                s.sten_hw[stype][idx] = _dp(hw)
        s.nzone = int(getattr(prob, "nzone", 1))
        s.mesh_coarsening, s.coarser_jac = int(getattr(prob, "mesh_coarsening", 0)), int(getattr(prob, "coarser_jac", 0))
        s.nwall = int(getattr(prob, "nwall", 0))
        s.l1d_bc, s.dim_1dbc = int(getattr(prob, "l1d_bc", 0)), int(getattr(prob, "dim_1dbc", 0))
        if getattr(prob, "zone_flag", None) is not None:
            zf = np.ascontiguousarray(prob.zone_flag, np.int32)
            self._keep.append(zf)
            s.zone_flag = zf.ctypes.data_as(C.POINTER(C.c_int))
        for zone, tabs in (getattr(prob, "zone_stencils", None) or {}).items():
            for (stype, idx), (off, w, hw) in tabs.items():
                off = np.ascontiguousarray(off, np.int16)
                w = np.ascontiguousarray(w, np.float64)
                self._keep += [off, w]
                s.zsten_len[zone][stype][idx] = len(w)
                s.zsten_off[zone][stype][idx] = off.ctypes.data_as(C.POINTER(C.c_int16))
                s.zsten_w[zone][stype][idx] = _dp(w)
                if hw is not None:
                    hw = np.ascontiguousarray(hw, np.float64)
                    self._keep.append(hw)
                    s.zsten_hw[zone][stype][idx] = _dp(hw)
        rbc = getattr(prob, "rhobar_bc", None)
        if rbc is not None:
            for i, v in enumerate(np.asarray(rbc, np.float64)[:10]):
                s.rhobar_bc[i] = float(v)
        if s.interface == 2:
            # Rhobar_b_LBB / _RTF (rhobar_icomp of the two bulk states, src/dft_thermo_hs.c:292-311)
            for dst, rho in ((s.rhobar_lbb, prob.rho_b_lbb), (s.rhobar_rtf, prob.rho_b_rtf)):
                for ic in range(prob.ncomp):
                    d = float(prob.hs_diam[ic])
                    vol, area = np.pi * d * d * d / 6.0, np.pi * d * d
                    f = float(prob.fac_overlap[ic]) * float(rho[ic])
                    dst[0] += f * vol
                    dst[1] += f * area
                    dst[2] += f * area * float(prob.inv_4pir[ic])
                    dst[3] += f * area * float(prob.inv_4pirsq[ic])
        self.s = s

    def _vec(self, x, rows=None):
        x = np.ascontiguousarray(x, np.float64)
        return x

    def resid(self, x):
        x = self._vec(x)
        R = np.zeros((self.prob.nunk, self.N))
        assert self.lib.orc_resid(C.byref(self.s), _dp(x), _dp(R)) == 0
        return R

    def resid_rows(self, x, begin, end):
        x = self._vec(x)
        R = np.zeros((self.prob.nunk, self.N))
        assert self.lib.orc_resid_rows(C.byref(self.s), _dp(x), _dp(R), C.c_long(begin), C.c_long(end)) == 0
        return R

    def jv(self, x, v):
        x, v = self._vec(x), self._vec(v)
        out = np.zeros((self.prob.nunk, self.N))
        assert self.lib.orc_jv(C.byref(self.s), _dp(x), _dp(v), _dp(out)) == 0
        return out

    def jtv(self, x, w):
        x, w = self._vec(x), self._vec(w)
        out = np.zeros((self.prob.nunk, self.N))
        assert self.lib.orc_jtv(C.byref(self.s), _dp(x), _dp(w), _dp(out)) == 0
        return out

    def schur(self, x, v2):
        x, v2 = self._vec(x), self._vec(v2)
        out = np.zeros((self.prob.ncomp, self.N))
        assert self.lib.orc_schur(C.byref(self.s), _dp(x), _dp(v2), _dp(out)) == 0
        return out

    def dphi(self, x):
        x = self._vec(x)
        out = np.zeros((4 + 2 * self.prob.ndim, self.N))
        assert self.lib.orc_dphi(C.byref(self.s), _dp(x), _dp(out)) == 0
        return out
