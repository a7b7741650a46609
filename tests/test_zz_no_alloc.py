"""Allocation-free stencil sum (tgpu_stencil_sum_noalloc) on the GPU.

The entry point serves callers that cannot allocate device memory where they
need a weighted-density sum (its scratch lives in fixed arrays inside the
library).  Its output must equal what the handle-based fill (tgpu_fill, the
existing entry point) computes for the same sums: with the weighted density n3
and the mean field set to zero, the fill's residual rows for them are exactly
the theta-stencil and attraction-stencil sums of the density.  Three calls in
a row (theta, attraction, theta again) check that a call does not depend on
what the previous one left in the shared scratch.  Further cases run the
other boundary rules and dimensions: a 1-D box with an in-wall side and a
reflecting side (the HS3 deck's geometry, hs1d_reflect, without its hard-wall
weights) and a 2-D box reflecting on one x side, in-bulk on the other and
periodic in y, each against the fill's theta and delta (n2) rows, two calls
in a row.  Tolerance: the absolute 1e-12 the other fill tests use."""
import ctypes as C

import numpy as np
import pytest

from goldens import RESID_ATOL, load

pytestmark = pytest.mark.gpu


def _lib():
    from tramonto_gb300 import native
    lib = native.load()
    lib.tgpu_stencil_sum_noalloc.restype = C.c_int
    lib.tgpu_stencil_sum_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.tgpu_noalloc_last_error.restype = C.c_char_p
    return lib


def _noalloc_sum(lib, p, stype, field, out):
    nx = np.array(list(p.nx[:p.ndim]) + [1] * (3 - p.ndim), np.int32)
    bc = np.array([b for pair in p.bc[:p.ndim] for b in pair], np.int32)
    off, w, _ = p.stencils[(stype, 0)]
    off = np.ascontiguousarray(off, np.int16)
    w = np.ascontiguousarray(w, np.float64)
    rc = lib.tgpu_stencil_sum_noalloc(p.ndim, nx.ctypes.data, bc.ctypes.data, float(p.rho_b[0]), len(w),
                                      off.ctypes.data, w.ctypes.data, C.c_void_p(field.data_ptr()),
                                      C.c_void_p(out.data_ptr()), None)
    assert rc == 0, lib.tgpu_noalloc_last_error()


def test_noalloc_stencil_sum_matches_fill():
    import torch
    from tramonto_gb300 import native
    from tramonto_gb300.problem import THETA, UATT

    lib = _lib()

    z, p = load("fmt1_wca_3d")
    k = len(z["states"]) - 1
    x = np.array(z[f"x{k}"], copy=True)
    x[p.first_rb] = 0.0          # n3 row: R = -0 + theta sum
    x[p.first_mf] = 0.0          # mean-field row: R = -0 + attraction sum
    s = native.Solver(p)
    R = s.fill(x, mode=1)
    s.close()
    expected = {THETA: R[p.first_rb], UATT: R[p.first_mf]}

    nx = np.array(p.nx[:3], np.int32)
    bc = np.array([b for pair in p.bc[:3] for b in pair], np.int32)
    field = torch.tensor(x[p.first_rho], dtype=torch.float64, device="cuda")
    out = torch.full_like(field, float("nan"))
    for stype in (THETA, UATT, THETA):
        off, w, _ = p.stencils[(stype, 0)]
        off = np.ascontiguousarray(off, np.int16)
        w = np.ascontiguousarray(w, np.float64)
        rc = lib.tgpu_stencil_sum_noalloc(p.ndim, nx.ctypes.data, bc.ctypes.data, float(p.rho_b[0]), len(w),
                                          off.ctypes.data, w.ctypes.data, C.c_void_p(field.data_ptr()),
                                          C.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.tgpu_noalloc_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        err = np.abs(got - expected[stype]).max()
        assert err <= RESID_ATOL, (stype, err)


def _without_hard_walls(p):
    import dataclasses
    st = {k: (o, w, None) for k, (o, w, _h) in p.stencils.items()}
    return dataclasses.replace(p, hard_surf=0, boundary_nodes=None, fluid_masks=None, stencils=st)


def _box_2d():
    from tramonto_gb300 import setup
    from tramonto_gb300.problem import BC_IN_BULK, BC_PERIODIC, BC_REFLECT
    return setup.build_problem(2, (60, 40), (0.05, 0.05), ((BC_REFLECT, BC_IN_BULK), (BC_PERIODIC, BC_PERIODIC)),
                               hs_diam=[1.0], rho_b=[0.6])


@pytest.mark.parametrize("case", ["hs1d_reflect", "box2d_reflect"])
def test_noalloc_other_boundaries_and_dimensions(case):
    """Reflecting, in-wall, in-bulk and periodic sides in 1-D and 2-D against the fill's theta and delta (n2)
    rows (n3 and n2 set to zero, so each row is its stencil sum of the density)."""
    import torch
    from tramonto_gb300 import native
    from tramonto_gb300.problem import DELTA, THETA

    if case == "hs1d_reflect":
        z, p = load(case)
        p = _without_hard_walls(p)
        x = np.array(z["x_newton"], copy=True)
    else:
        p = _box_2d()
        rng = np.random.default_rng(11)
        x = np.zeros((p.nunk, p.nnodes))
        x[p.first_rho] = 0.6 * (1.0 + 0.3 * rng.uniform(-1.0, 1.0, p.nnodes))
    x[p.first_rb] = 0.0          # n3 row: R = theta sum
    x[p.first_rb + 1] = 0.0      # n2 row: R = delta sum (one component: n2 carries the delta weights as they are)
    s = native.Solver(p)
    R = s.fill(x, mode=1)
    s.close()
    lib = _lib()
    field = torch.tensor(x[p.first_rho], dtype=torch.float64, device="cuda")
    out = torch.full_like(field, float("nan"))
    for stype, row in ((THETA, p.first_rb), (DELTA, p.first_rb + 1)) * 2:
        _noalloc_sum(lib, p, stype, field, out)
        torch.cuda.synchronize()
        err = np.abs(out.cpu().numpy() - R[row]).max()
        assert err <= RESID_ATOL, (case, stype, err)


def test_noalloc_rejects_oversized_boxes():
    lib = _lib()
    nx = np.array([256, 256, 256], np.int32)
    bc = np.array([1, 1, 1, 1, 1, 1], np.int32)
    off = np.zeros((1, 3), np.int16)
    w = np.ones(1)
    rc = lib.tgpu_stencil_sum_noalloc(3, C.c_void_p(nx.ctypes.data), C.c_void_p(bc.ctypes.data), C.c_double(0.0), 1,
                                      C.c_void_p(off.ctypes.data), C.c_void_p(w.ctypes.data), C.c_void_p(16),
                                      C.c_void_p(16), None)
    assert rc == -1 and b"TGPU_NOALLOC_MAX_PADDED" in lib.tgpu_noalloc_last_error()
