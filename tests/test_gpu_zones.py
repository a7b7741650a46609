"""Quadrature zones and mesh coarsening on the GPU (the reference's HS6 and HS7 decks).

hs1d_zones: four zones at 2, 4 and 5 sigma from the wall; the nodes off each zone's coarse lattice have
averaged rows.  hs1d_jaczones: the same residual with the reference's Jacobian one zone coarser near the
wall (Coarser_jac = 1), an approximation of its assembled matrix; the GPU products are the residual's own
derivative, checked against the oracle with Coarser_jac = 0 and against central differences.

* J^T w against the reference's transpose (hs1d_zones) and the oracle (1e-12), <u, J v> = <J^T u, v>;
* J v is the derivative of the residual (central differences, 1e-7 relative);
* a Newton step solved on the other nodes satisfies the full system J dx = b (1e-9) when b vanishes on
  the coarsened nodes: the interpolated values satisfy the averaged rows;
* the adjoint of that step: dOmega_s/dV_ext against central differences of re-converged states (a V_ext
  change at a coarsened node does not move the solution: its rows carry no field).
The fill, J v and the Newton solution against the fixtures are in tests/test_gpu_parity.py.
"""
import copy

import numpy as np
import pytest

import orc
from goldens import PROD_RTOL, coarsened, load, probe, rel_err

pytestmark = pytest.mark.gpu

ZCASES = ["hs1d_zones", "hs1d_jaczones"]


def _solver(name):
    from tramonto_gb300 import native
    z, p = load(name)
    assert coarsened(p)
    return z, p, native.Solver(p)


def _oracle_residual_jacobian(p):
    q = copy.copy(p)
    q.coarser_jac = 0
    return orc.Oracle(q)


@pytest.mark.parametrize("name", ZCASES)
def test_jtv_matches_reference_and_oracle(name):
    z, p, s = _solver(name)
    o = _oracle_residual_jacobian(p)
    N = p.nunk * p.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        s.fill(x)
        w = probe(N, 1).reshape(x.shape)
        got = s.jtv(w)
        assert rel_err(got, o.jtv(x, w)) <= PROD_RTOL, (name, k)
        if not p.coarser_jac:
            assert rel_err(got, z[f"JTw{k}"]) <= PROD_RTOL, (name, k)
    s.close()


@pytest.mark.parametrize("name", ZCASES)
def test_jtv_is_the_adjoint_of_jv(name):
    z, p, s = _solver(name)
    x = z["x0"]
    s.fill(x)
    rng = np.random.default_rng(5)
    for _ in range(3):
        u, v = rng.standard_normal(x.shape), rng.standard_normal(x.shape)
        Jv = s.jv(v)
        lhs, rhs = float(np.sum(u * Jv)), float(np.sum(s.jtv(u) * v))
        assert abs(lhs - rhs) <= 1e-12 * float(np.abs(u * Jv).sum()), (name, lhs, rhs)
    s.close()


@pytest.mark.parametrize("name", ZCASES)
def test_jv_is_the_derivative_of_the_residual(name):
    z, p, s = _solver(name)
    x = np.array(z["x0"])
    v = x * probe(x.size, 6).reshape(x.shape)   # relative perturbation: densities stay positive
    h = 1e-6
    fd = (s.fill(x + h * v) - s.fill(x - h * v)) / (2 * h)
    s.fill(x)
    assert rel_err(s.jv(v), fd) <= 1e-7, name
    s.close()


@pytest.mark.parametrize("name", ZCASES)
def test_step_on_the_other_nodes_solves_the_full_system(name):
    z, p, s = _solver(name)
    x = z[f"x{len(z['states']) - 1}"]
    s.fill(x)
    b = probe(p.nunk * p.nnodes, 4).reshape(x.shape)
    b[:, np.asarray(p.zone_flag) < 0] = 0.0
    dx, it, rr = s.solve(b, tol=1e-12, max_iter=1000)
    r = s.jv(dx) - b
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(b), (name, it, rr, np.linalg.norm(r))
    s.close()


def test_vext_sensitivity_matches_finite_differences():
    """The adjoint of the step on the other nodes: dOmega_s/dV_ext against central differences of
    re-converged states (1e-5 of the gradient's scale)."""
    z, p, s = _solver("hs1d_zones")
    vext0 = np.array(p.vext, dtype=np.float64).reshape(p.ncomp, p.nnodes)

    def converge(v, x0):
        s.set_vext(v)
        x, _, rn, _ = s.newton_solve(x0, resid_tol=1e-12, lin_tol=1e-12, lin_max_iter=1000, max_iter=60,
                                     allow_noconv=True)
        assert rn <= 1e-11, rn
        return x

    x0 = converge(vext0, z["x_newton"])
    g = s.grad_vext(x0, kind=0, tol=1e-13, max_iter=2000)
    live = np.nonzero((np.asarray(p.zero_density).reshape(-1) == 0) & (vext0.reshape(-1) < p.vext_max))[0]
    coarse = np.asarray(p.zone_flag)[live % p.nnodes] < 0
    u = np.zeros(vext0.size)
    u[live] = np.cos(0.37 * np.arange(live.size))
    dirs = [u, np.eye(1, vext0.size, live[~coarse][10]).reshape(-1), np.eye(1, vext0.size, live[coarse][5]).reshape(-1)]
    h = 1e-5
    for d in dirs:
        d = d.reshape(vext0.shape)
        om_p = s.objectives(converge(vext0 + h * d, x0))[0]
        om_m = s.objectives(converge(vext0 - h * d, x0))[0]
        fd = (om_p - om_m) / (2 * h)
        adj = float(np.sum(g * d))
        scale = max(abs(fd), float(np.abs(g).max() * np.abs(d).max()))
        assert abs(adj - fd) <= 1e-5 * scale, (adj, fd)
    s.close()
