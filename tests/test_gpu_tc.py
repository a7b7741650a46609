"""Tensor-core attraction sums (tcgen05, FP16 inputs scaled by powers of two, FP32 accumulation).

The 3-D attraction (WCA) stencil sums of the Jacobian / Schur products run on
the tensor cores in TGPU_FP16TC.  Checked against the FP64 sums:
- the mean-field rows of J v (= the attraction sums of v) for a random v:
  within 2e-5 of max |S| (FP16 rounding of independent values averages out
  over the ~7e4-point stencil);
- the same for the smooth density field itself, where the rounding errors
  are correlated: within 1e-3 of max |S|;
- Schur products within 1e-4 relative;
- a mixed Newton solve with these products reaches ||R||_2 <= 1e-8 (FP64
  residual) and its density is within 1e-6 of the FP64 solve's.
The FP32 FFT sums win the timed choice at these sizes, so every handle here fixes the direct kernels
(tgpu_set_fft32_policy 0): the tensor-core kernel is what runs.
"""
import numpy as np
import pytest

from goldens import rel_err

pytestmark = pytest.mark.gpu


def _attraction_sums(s, p, v):
    full = np.zeros((p.nunk, p.nnodes))
    full[p.first_rho:p.first_rho + p.ncomp] = v
    return s.jv(full)[p.first_mf:p.first_mf + p.ncomp]


@pytest.fixture(scope="module")
def case64():
    from tramonto_gb300 import native, setup
    p, meta = setup.config2(n=64)
    s = native.Solver(p)
    s.set_fft32_policy(0)
    x = setup.initial_state(s, p)
    s.fill(x, mode=0)
    yield p, s, x
    s.close()


def test_tc_attraction_sum_of_random_field(case64):
    from tramonto_gb300 import native
    p, s, x = case64
    v = np.random.default_rng(3).standard_normal((p.ncomp, p.nnodes))
    s.set_precision(native.FP64)
    ref = _attraction_sums(s, p, v)
    s.set_precision(native.FP16TC)
    got = _attraction_sums(s, p, v)
    s.set_precision(native.FP64)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print("random field: max error / max |S| =", err)
    assert err <= 2e-5


def test_tc_attraction_sum_of_density(case64):
    from tramonto_gb300 import native
    p, s, x = case64
    v = x[p.first_rho:p.first_rho + p.ncomp]
    s.set_precision(native.FP64)
    ref = _attraction_sums(s, p, v)
    s.set_precision(native.FP16TC)
    got = _attraction_sums(s, p, v)
    s.set_precision(native.FP64)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    print("density field: max error / max |S| =", err)
    assert err <= 1e-3


def test_tc_schur_product(case64):
    from tramonto_gb300 import native
    p, s, x = case64
    v2 = np.random.default_rng(4).standard_normal((p.ncomp, p.nnodes))
    s.set_precision(native.FP64)
    ref = s.schur(v2)
    s.set_precision(native.FP16TC)
    got = s.schur(v2)
    s.set_precision(native.FP64)
    print("Schur product relative error:", rel_err(got, ref))
    assert rel_err(got, ref) <= 1e-4


def test_tc_mixed_newton_reaches_fp64_target():
    from tramonto_gb300 import native, setup
    p, meta = setup.config2(n=40)
    s = native.Solver(p)
    s.set_fft32_policy(0)
    x0 = setup.initial_state(s, p)
    x64, it64, r64, _ = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-10)
    s.set_precision(native.FP16TC)
    s.set_fill_arithmetic(native.FILL_MIXED, switch_norm=0.1)
    xtc, ittc, rtc, li = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-6)
    s.close()
    print("FP64:", it64, r64, " FP16TC products:", ittc, rtc, li)
    assert rtc <= 1e-8
    assert np.abs(xtc[p.first_rho] - x64[p.first_rho]).max() <= 1e-6
