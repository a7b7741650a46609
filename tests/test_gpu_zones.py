"""Quadrature zones and mesh coarsening on the GPU (the reference's HS6 and HS7 decks).

hs1d_zones: four zones at 2, 4 and 5 sigma from the wall; the nodes off each zone's coarse lattice have
averaged rows.  hs1d_jaczones: the same residual with the reference's Jacobian one zone coarser near the
wall (Coarser_jac = 1), an approximation of its assembled matrix; the GPU products are the residual's own
derivative, checked against the oracle with Coarser_jac = 0 and against central differences.

* J^T w against the reference's transpose (hs1d_zones) and the oracle (1e-12), <u, J v> = <J^T u, v>;
* J v is the derivative of the residual (central differences, 1e-7 relative);
* a Newton step solved on the other nodes satisfies the full system J dx = b (1e-9) when b vanishes on
  the coarsened nodes: the interpolated values satisfy the averaged rows;
* the adjoint entry points refuse coarsened problems.
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


def test_adjoint_entry_points_refuse_coarsened_problems():
    from tramonto_gb300 import native
    z, p, s = _solver("hs1d_zones")
    s.fill(z["x0"])
    with pytest.raises(native.TgpuError):
        s.adjoint_solve(np.ones(z["x0"].shape), tol=1e-10, max_iter=10)
    s.close()
