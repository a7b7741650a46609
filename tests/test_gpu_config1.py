"""Configuration 1 on the GPU: the reference's HS5 hard-sphere wall problem at
L = 20 sigma, dx = 0.01 sigma (2000 elements), rho_b = 0.7, solved from the
bulk density by the FP64 Newton of the reference (tgpu_newton: damping,
clamps and update-norm test of src/dft_newton.c) and by the residual-targeted
Newton to ||R||_2 <= 1e-10.

Against the reference's own solve of the same deck (fixture hs1d_c1: the
reference converged in 8 iterations to a residual of 8.7e-13): the converged
densities agree to 1e-8, the surface excess free energy and the excess
adsorption to 1e-9, and the iteration count of the reference-criterion Newton
is within the +-4 the reference's own result checker allows.
"""
import numpy as np
import pytest

from goldens import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def c1():
    from tramonto_gb300 import native, setup
    z, p = load("hs1d_c1")
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    yield z, p, s, x0
    s.close()


def test_config1_reference_newton_matches_reference_solve(c1):
    z, p, s, x0 = c1
    x, it, rn = s.newton(x0, rel_tol=1e-6, abs_tol=1e-10, update_floor=0.1, max_iter=50, lin_tol=1e-12,
                         lin_max_iter=500)
    ref_it = int(z["newton_iters"])
    print("tgpu_newton iterations", it, "reference", ref_it, "final |R|", rn)
    assert abs(it - ref_it) <= 4
    rho = x[p.first_rho]
    assert np.abs(rho - z["x_newton"][p.first_rho]).max() <= 1e-8


def test_config1_residual_target_and_objectives(c1):
    z, p, s, x0 = c1
    x, it, rn, li = s.newton_solve(x0, resid_tol=1e-10, lin_tol=1e-12, lin_max_iter=500, max_iter=50)
    assert rn <= 1e-10
    ref = z["x_newton"]
    assert np.abs(x[p.first_rho] - ref[p.first_rho]).max() <= 1e-8
    om, gam = s.objectives(x)
    ref_om = float(z["omega_s0"])
    ref_gam = float(z["ads0"][0] - z["ads_b0"][0])
    print("Omega_s", om, "reference", ref_om, "Gamma_ex", gam[0], "reference", ref_gam, "iterations", it)
    assert abs(om - ref_om) <= 1e-9 * max(1.0, abs(ref_om))
    assert abs(gam[0] - ref_gam) <= 1e-9 * max(1.0, abs(ref_gam))
