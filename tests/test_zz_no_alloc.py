"""Allocation-free stencil sum (tgpu_stencil_sum_noalloc) on the GPU.

The entry point serves callers that cannot allocate device memory where they
need a weighted-density sum (its scratch lives in fixed arrays inside the
library).  Its output must equal what the handle-based fill (tgpu_fill, the
existing entry point) computes for the same sums: with the weighted density n3
and the mean field set to zero, the fill's residual rows for them are exactly
the theta-stencil and attraction-stencil sums of the density.  Three calls in
a row (theta, attraction, theta again) check that a call does not depend on
what the previous one left in the shared scratch.  Tolerance: the absolute
1e-12 the other fill tests use."""
import ctypes as C

import numpy as np
import pytest

from goldens import RESID_ATOL, load

pytestmark = pytest.mark.gpu


def test_noalloc_stencil_sum_matches_fill():
    import torch
    from tramonto_gb300 import native
    from tramonto_gb300.problem import THETA, UATT

    lib = native.load()
    lib.tgpu_stencil_sum_noalloc.restype = C.c_int
    lib.tgpu_stencil_sum_noalloc.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.tgpu_noalloc_last_error.restype = C.c_char_p

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


def test_noalloc_rejects_oversized_boxes():
    from tramonto_gb300 import native
    lib = native.load()
    lib.tgpu_stencil_sum_noalloc.restype = C.c_int
    lib.tgpu_noalloc_last_error.restype = C.c_char_p
    nx = np.array([256, 256, 256], np.int32)
    bc = np.array([1, 1, 1, 1, 1, 1], np.int32)
    off = np.zeros((1, 3), np.int16)
    w = np.ones(1)
    rc = lib.tgpu_stencil_sum_noalloc(3, C.c_void_p(nx.ctypes.data), C.c_void_p(bc.ctypes.data), C.c_double(0.0), 1,
                                      C.c_void_p(off.ctypes.data), C.c_void_p(w.ctypes.data), C.c_void_p(16),
                                      C.c_void_p(16), None)
    assert rc == -1 and b"TGPU_NOALLOC_MAX_PADDED" in lib.tgpu_noalloc_last_error()
