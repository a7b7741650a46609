"""The four hard-sphere functionals on the GPU and the two forms of their second derivatives.

FMT2 and FMT4 residuals, J v, J^T w and Schur products are pinned to the reference's own
fixtures by the golden-case tests (tests/test_gpu_parity.py, tests/test_gpu_adjoint.py run
over hs1d_fmt2, hs1d_fmt4, mix1d_fmt4, rough3d_fmt2, rough3d_fmt4).  This file covers what
the fixtures cannot:

* TGPU_JAC_EXACT gives the same products as the reference's tables for FMT1 and FMT3;
* for FMT2 and FMT4 the exact form is the derivative of the residual (central differences,
  1e-6 relative) while the reference's tables differ from it in 3-D;
* Newton with the exact form converges to the same state as with the reference's form;
* the V_ext sensitivity of Omega_s for FMT4 (adjoint, always with the exact form) matches
  central differences of re-converged states (1e-5 of the gradient's scale).
"""
import numpy as np
import pytest

from goldens import PROD_RTOL, load, probe, rel_err

pytestmark = pytest.mark.gpu


def _solver(name, form):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    s.set_jacobian_form(form)
    return z, p, s


@pytest.mark.parametrize("name", ["fmt1_wca_3d", "mix1d_fmt3", "hs1d_reflect"])
def test_exact_form_equals_reference_tables_for_fmt1_fmt3(name):
    from tramonto_gb300 import native
    z, p, s = _solver(name, native.JAC_EXACT)
    N = p.nunk * p.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        s.fill(x)
        Jv = s.jv(probe(N, 0).reshape(x.shape))
        assert rel_err(Jv, z[f"Jv{k}"]) <= PROD_RTOL, (name, k)
    s.close()


def _fd_directional(s, x, v, h=1e-6):
    rp = s.fill(x + h * v)
    rm = s.fill(x - h * v)
    return (rp - rm) / (2 * h)


@pytest.mark.parametrize("name", ["hs1d_fmt2", "hs1d_fmt4", "mix1d_fmt4", "rough3d_fmt2", "rough3d_fmt4"])
def test_exact_form_is_the_derivative_of_the_residual(name):
    from tramonto_gb300 import native
    z, p, s = _solver(name, native.JAC_EXACT)
    k = len(z["states"]) - 1
    x = np.array(z[f"x{k}"])
    # a relative perturbation keeps every density and 1 - n3 positive
    v = x * probe(x.size, 5).reshape(x.shape)
    fd = _fd_directional(s, x, v)
    s.fill(x)
    je = s.jv(v)
    err_exact = rel_err(je, fd)
    assert err_exact <= 1e-6, (name, err_exact)
    s.set_jacobian_form(native.JAC_REFERENCE)
    s.fill(x)
    jr = s.jv(v)
    err_ref = rel_err(jr, fd)
    if name == "hs1d_fmt2":
        # one dimension: the reference's FMT2 tables are the Hessian
        assert rel_err(jr, je) <= PROD_RTOL, (name, rel_err(jr, je))
    elif name in ("rough3d_fmt2", "rough3d_fmt4", "hs1d_fmt4", "mix1d_fmt4"):
        assert err_ref > 100 * err_exact, (name, err_ref, err_exact)
    s.close()


@pytest.mark.parametrize("name", ["rough3d_fmt2", "rough3d_fmt4"])
def test_newton_with_exact_form_reaches_the_reference_solution(name):
    from tramonto_gb300 import native
    z, p, s = _solver(name, native.JAC_EXACT)
    x0 = z["x0"]
    x, it_exact, rn, _ = s.newton_solve(x0, resid_tol=1e-11, lin_tol=1e-12, lin_max_iter=1000, max_iter=60)
    assert rn <= 1e-11
    s.set_jacobian_form(native.JAC_REFERENCE)
    xr, it_ref, rnr, _ = s.newton_solve(x0, resid_tol=1e-11, lin_tol=1e-12, lin_max_iter=1000, max_iter=60)
    assert rnr <= 1e-11
    rho = slice(p.first_rho, p.first_rho + p.ncomp)
    assert np.abs(x[rho] - xr[rho]).max() <= 1e-9 * np.abs(x[rho]).max()
    ref = z["x_newton"]
    assert np.abs(x[rho] - ref[rho]).max() <= 1e-7 * np.abs(ref[rho]).max()
    assert it_exact <= it_ref, (name, it_exact, it_ref)
    s.close()


def test_fmt4_vext_sensitivity_matches_finite_differences():
    from tramonto_gb300 import native
    z, p, s = _solver("rough3d_fmt4", native.JAC_EXACT)
    vext0 = np.array(p.vext, dtype=np.float64).reshape(p.ncomp, p.nnodes)

    def converge(v, x0):
        s.set_vext(v)
        x, _, rn, _ = s.newton_solve(x0, resid_tol=1e-12, lin_tol=1e-12, lin_max_iter=1000, max_iter=60,
                                     allow_noconv=True)
        assert rn <= 1e-11, rn
        return x

    x0 = converge(vext0, z["x0"])
    # the adjoint uses the exact form even when the reference's tables are selected
    s.set_jacobian_form(native.JAC_REFERENCE)
    s.set_vext(vext0)
    g = s.grad_vext(x0, kind=0, tol=1e-13, max_iter=2000)
    s.set_jacobian_form(native.JAC_EXACT)
    live = np.nonzero((np.asarray(p.zero_density).reshape(-1) == 0) & (vext0.reshape(-1) < p.vext_max))[0]
    u = np.zeros(vext0.size)
    u[live] = np.cos(0.37 * np.arange(live.size))
    dirs = [u, np.eye(1, vext0.size, live[live.size // 3]).reshape(-1)]
    h = 1e-6
    for d in dirs:
        d = d.reshape(vext0.shape)
        om_p = s.objectives(converge(vext0 + h * d, x0))[0]
        om_m = s.objectives(converge(vext0 - h * d, x0))[0]
        fd = (om_p - om_m) / (2 * h)
        adj = float(np.sum(g * d))
        scale = max(abs(fd), float(np.abs(g).max() * np.abs(d).max()))
        assert abs(adj - fd) <= 1e-5 * scale, (adj, fd)
    s.close()
