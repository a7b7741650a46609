"""Failure statuses of the C ABI, each provoked on the host (no GPU fault, trap or hang is involved):

- TGPU_ERR_DOMAIN: a state with n3 = 1.2 at one node, or a density <= 0 on a live Euler-Lagrange row, where the fill
  would take log(1 - n3), 1/(1 - n3)^k or log(rho) (the reference evaluates them unguarded: calc_FMT_derivatives
  src/dft_fill_FMT.c:362-366, fill_EL_ideal_gas src/dft_fill_EL.c:358); a zero density on a zero-density row is
  the reference's own solution there and passes;
- TGPU_ERR_NONFINITE: NaN in the external field at set-up, NaN in one density of a Newton state, a NaN right-hand
  side of the Schur solve;
- TGPU_ERR_NOCONV: the GMRES cap (one iteration to 1e-14) and the Newton cap (one iteration to 1e-14; the
  reference's newton_solver returns -iter when Max_NL_iter is reached, src/dft_newton.c:186-192);
- TGPU_ERR_CUDA from the tensor-core stencil sum when its pipeline's mbarrier waits are limited to one attempt
  (tgpu_set_tc_wait_limit): the waits run out, the kernel drains the copies and MMAs it started (those waits keep
  their default limit), frees its tensor memory and leaves a flag that the product reports.

After each failure the handle stays usable: the next fill of the fixture's state equals the reference's residual.
"""
import ctypes as C

import numpy as np
import pytest

from goldens import RESID_ATOL, load

pytestmark = pytest.mark.gpu

ERR_NOCONV, ERR_NONFINITE, ERR_DOMAIN = -5, -6, -7


def _still_usable(s, z):
    R = s.fill(z["x0"], mode=1)
    assert np.abs(R - z["R0"]).max() <= RESID_ATOL


def _status(fn):
    from tramonto_gb300.native import TgpuError
    with pytest.raises(TgpuError) as e:
        fn()
    return e.value.status, str(e.value)


@pytest.mark.parametrize("case", ["lj1d_mf", "fmt1_wca_3d"])
def test_domain_n3_at_or_above_one(case):
    from tramonto_gb300 import native
    z, p = load(case)
    s = native.Solver(p)
    x = np.array(z["x0"], copy=True)
    x[p.first_rb, p.nnodes // 2] = 1.2
    st, msg = _status(lambda: s.fill(x, mode=0))
    assert st == ERR_DOMAIN and "n3 >= 1" in msg
    st, _ = _status(lambda: s.newton_solve(x, max_iter=3))
    assert st == ERR_DOMAIN
    _still_usable(s, z)
    s.close()


def test_domain_nonpositive_density_on_a_live_row():
    from tramonto_gb300 import native
    z, p = load("hs1d_wall")
    s = native.Solver(p)
    live = np.flatnonzero((np.asarray(p.zero_density)[0] == 0) & (np.asarray(p.vext)[0] < p.vext_max))
    zero_rows = np.flatnonzero(np.asarray(p.zero_density)[0] != 0)
    assert len(zero_rows) > 0 and len(live) > 0
    x = np.array(z["x0"], copy=True)
    x[p.first_rho, zero_rows] = 0.0          # allowed: the zero-density rows are R = rho
    s.fill(x, mode=1)
    x[p.first_rho, live[len(live) // 2]] = -1e-3
    st, msg = _status(lambda: s.fill(x, mode=1))
    assert st == ERR_DOMAIN and "density <= 0" in msg
    _still_usable(s, z)
    s.close()


def test_nonfinite_inputs():
    import torch
    from tramonto_gb300 import native
    z, p = load("lj1d_mf")
    s = native.Solver(p)
    v = np.array(p.vext, copy=True)
    v[0, p.nnodes // 3] = np.nan
    st, msg = _status(lambda: s.set_vext(v))
    assert st == ERR_NONFINITE and "NaN" in msg
    x = np.array(z["x0"], copy=True)
    x[p.first_rho, p.nnodes // 2] = np.nan
    st, msg = _status(lambda: s.newton_solve(x, max_iter=5))
    assert st == ERR_NONFINITE and "non-finite" in msg
    # a NaN right-hand side of the Schur solve, through the device entry point
    s.fill(z["x0"], mode=0)
    b = torch.zeros((p.nunk, p.nnodes), dtype=torch.float64, device="cuda")
    b[p.first_rho, 5] = float("nan")
    dx = torch.zeros_like(b)
    st, msg = _status(lambda: s.solve_device(b, dx, tol=1e-10, max_iter=50))
    assert st == ERR_NONFINITE
    _still_usable(s, z)
    s.close()


def test_iteration_caps():
    from tramonto_gb300 import native
    z, p = load("lj1d_mf")
    s = native.Solver(p)
    x1 = np.array(z["x1"], copy=True)      # the perturbed fixture state: |R| ~ 1e-1
    s.fill(x1, mode=0)
    b = -s.fill(x1, mode=1)
    dx = np.empty_like(b)
    it, rr = C.c_int(0), C.c_double(0.0)
    st = s.lib.tgpu_solve(s.h, C.c_void_p(b.ctypes.data), C.c_void_p(dx.ctypes.data), 1e-14, 1, C.byref(it),
                         C.byref(rr))
    assert st == ERR_NOCONV and it.value == 1 and rr.value > 1e-14
    st, msg = _status(lambda: s.newton_solve(x1, resid_tol=1e-14, max_iter=1))
    assert st == ERR_NOCONV
    _still_usable(s, z)
    s.close()


def test_tensor_core_waits_that_run_out_are_reported():
    import ctypes as C
    from tramonto_gb300 import native, setup
    from goldens import rel_err
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    s.set_fft32_policy(0)          # the direct tensor-core sum, not the FP32 FFT
    x = setup.initial_state(s, p)
    s.fill(x, mode=0)
    v2 = np.random.default_rng(6).standard_normal((p.ncomp, p.nnodes))
    ref = s.schur(v2)              # FP64
    s.set_precision(native.FP16TC)
    ok = s.schur(v2)
    assert rel_err(ok, ref) <= 1e-4
    assert s.lib.tgpu_set_tc_wait_limit(s.h, C.c_long(1)) == 0
    st, msg = _status(lambda: s.schur(v2))
    assert st == -2 and "bounded wait ran out" in msg
    assert s.lib.tgpu_set_tc_wait_limit(s.h, C.c_long(0)) == 0
    again = s.schur(v2)            # default limit: the context and the handle still work
    assert rel_err(again, ref) <= 1e-4 and np.abs(again - ok).max() <= 1e-12 * np.abs(ok).max()
    s.close()
