"""Float-float 3-D stencil sums (TGPU_FILL_FF): FP64-accurate residual fills from FP32 pairs.

- At the fixture states of fmt1_wca_3d the TGPU_FILL_FF residual equals the reference's to the 1e-12
  of the FP64 parity tests;
- on the 64^3 configuration-2 problem it equals the FP64 fill to 5e-12 at the initial state (|R| up to
  7.5; both sums carry ~1e-12 of rounding over ~7e4-point stencils, in different orders);
- a TGPU_FILL_MIXED_FF Newton solve reaches ||R||_2 <= 1e-8, its residual re-evaluated in FP64 is
  below 1e-8 too, and its density equals the FP64 solve's to 1e-9.
"""
import numpy as np
import pytest

from goldens import RESID_ATOL, load

pytestmark = pytest.mark.gpu


def test_ff_fill_matches_reference_fixture():
    from tramonto_gb300 import native
    z, p = load("fmt1_wca_3d")
    s = native.Solver(p)
    s.set_fill_arithmetic(native.FILL_FF)
    for k in range(len(z["states"])):
        R = s.fill(z[f"x{k}"], mode=1)
        err = np.abs(R - z[f"R{k}"]).max()
        print("fixture state", k, "max |R_ff - R_ref|", err)
        assert err <= RESID_ATOL
    s.close()


def test_ff_fill_matches_fp64_fill():
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=64)
    s = native.Solver(p)
    x = setup.initial_state(s, p)
    R64 = s.fill(x, mode=1)
    s.set_fill_arithmetic(native.FILL_FF)
    Rff = s.fill(x, mode=1)
    err = np.abs(Rff - R64).max()
    print("64^3: max |R_ff - R_fp64|", err, "max |R|", np.abs(R64).max())
    assert err <= 5e-12
    s.close()


def test_mixed_ff_newton_solve():
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    x64, _, _, _ = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-10)
    s.set_precision(native.FP16TC)
    s.set_fill_arithmetic(native.FILL_MIXED_FF, switch_norm=0.1)
    xff, it, rn, li = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-6)
    assert rn <= 1e-8
    s.set_fill_arithmetic(native.FILL_FP64)
    r64 = np.linalg.norm(s.fill(xff, mode=1))
    print("mixed-FF solve:", it, "iterations, ||R||_2", rn, "re-evaluated in FP64", r64)
    assert r64 <= 1e-8
    assert np.abs(xff[p.first_rho] - x64[p.first_rho]).max() <= 1e-9
    s.close()
