"""Mixed-precision form: FP32 stencil sums in the Schur products, FP64 residual.

The FP32 Schur product must agree with the FP64 one to FP32-level accuracy, and
a Newton solve whose Schur-GMRES uses FP32 products must converge to the FP64
solution (residual 1e-8, density error <= 1e-6 relative) because the residual
stays FP64."""
import numpy as np
import pytest

from goldens import load, rel_err

pytestmark = pytest.mark.gpu

FP32_PRODUCT_RTOL = 2e-5


def test_fp32_schur_product_close_to_fp64():
    from tramonto_gb300 import native
    z, p = load("fmt1_wca_3d")
    s = native.Solver(p)
    x = z["x0"]
    s.fill(x)
    rng = np.random.default_rng(11)
    v2 = rng.standard_normal((p.ncomp, p.nnodes))
    y64 = s.schur(v2)
    s.set_precision(native.FP32)
    y32 = s.schur(v2)
    s.close()
    assert rel_err(y32, y64) <= FP32_PRODUCT_RTOL


def test_refined_fill_matches_fp64_fill():
    """FP64 sums of a reference state + FP32 sums of a small change = the FP64 residual."""
    from tramonto_gb300 import native
    z, p = load("fmt1_wca_3d")
    s = native.Solver(p)
    x0 = z["x0"]
    rng = np.random.default_rng(5)
    x1 = x0 * (1.0 + 1e-4 * rng.uniform(-1, 1, x0.shape))
    R64 = s.fill(x1)
    s.set_fill_arithmetic(native.FILL_REFINED, tau=1e-3)
    s.fill(x0)                         # sets the FP64 reference
    s.reset_stats()
    Rref = s.fill(x1)                  # change 1e-4 < tau: FP32 sums of the change only
    st = s.stats()
    s.set_fill_arithmetic(native.FILL_FP32)
    R32 = s.fill(x1)
    s.close()
    assert st["fp64_refreshes"] == 0
    # FP32 sums of a change of relative size 1e-4: their rounding is ~1e-7 of the change's sums (FP32 FFT sums
    # carry it relative to the sums' max norm, ~3e-7), against residual terms of O(1..10)
    assert np.abs(Rref - R64).max() <= 3e-10, np.abs(Rref - R64).max()
    assert np.abs(R32 - R64).max() > np.abs(Rref - R64).max()


@pytest.mark.parametrize("fill", ["fp64", "refined"])
def test_mixed_newton_matches_fp64_solution(fill):
    from tramonto_gb300 import native, setup
    p, meta = setup.config2(n=40)
    s = native.Solver(p, precision=native.FP64)
    x0 = setup.initial_state(s, p)
    x64, it64, r64 = s.newton(x0, max_iter=40, lin_tol=1e-8, lin_max_iter=300)
    s.set_precision(native.FP32)
    if fill == "refined":
        s.set_fill_arithmetic(native.FILL_REFINED)
    x32, it32, r32 = s.newton(x0, max_iter=40, lin_tol=1e-6, lin_max_iter=300)
    s.set_fill_arithmetic(native.FILL_FP64)
    R = s.fill(x32, mode=1)
    s.close()
    rho64, rho32 = x64[0], x32[0]
    err = np.abs(rho32 - rho64).max() / np.abs(rho64).max()
    assert np.abs(R).max() < 1e-8, np.abs(R).max()
    assert err <= 1e-6, (err, it64, it32)


def test_mixed_newton_solve_reaches_fp64_residual_target():
    """Residual-targeted solve: FP32 residual sums far from the solution, FP64 near it,
    FP32 Schur products throughout; the result must have an FP64 residual <= 1e-8 and
    match the plain FP64 solve's density to 1e-6."""
    from tramonto_gb300 import native, setup
    p, meta = setup.config2(n=40)
    s = native.Solver(p, precision=native.FP64)
    x0 = setup.initial_state(s, p)
    x64, it64, r64, _ = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-10)
    s.set_precision(native.FP32)
    s.set_fill_arithmetic(native.FILL_MIXED, switch_norm=0.1)
    x32, it32, r32, li = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-6)
    s.set_fill_arithmetic(native.FILL_FP64)
    R = s.fill(x32, mode=1)
    s.close()
    assert r64 <= 1e-8 and r32 <= 1e-8
    assert np.sqrt((R ** 2).sum()) <= 1e-8
    err = np.abs(x32[0] - x64[0]).max() / np.abs(x64[0]).max()
    assert err <= 1e-6, (err, it64, it32)
