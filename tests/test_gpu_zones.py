"""Quadrature zones, mesh coarsening and the other Mesh_coarsen_flag rows on the GPU.

hs1d_zones (the reference's HS6 deck): four zones at 2, 4 and 5 sigma from the wall; the nodes off each
zone's coarse lattice have averaged rows.  hs1d_jaczones (HS7): the same residual with the reference's
Jacobian one zone coarser near the wall (Coarser_jac = 1), an approximation of its assembled matrix; the GPU
products are the residual's own derivative, checked against the oracle with Coarser_jac = 0 and against
central differences.  lj1d_zones / lj1d_zones_a22: the LJ1 fluid (FMT1 + WCA) with HS6's zones, the mean field
as its own unknown and summed into the Euler-Lagrange rows (ATTInA22Block = 1).  fmt1_wca_3d_1dbc: L1D_bc,
the nodes within 1 sigma of either x end copying the line y = z = 0.  BULK_ZONE / PB_ZONE (Mesh_coarsening
2 / 3, flags -888 / -777 on every node of a zone above 0): no example deck uses them and the reference's
weighted-density rows at those nodes index its stencil table with the negative flag, so they are checked
against the oracle (zone 0's stencils there).

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

ZCASES = ["hs1d_zones", "hs1d_jaczones", "lj1d_zones", "lj1d_zones_a22", "fmt1_wca_3d_1dbc"]


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


def _bulk_pb(kind):
    """lj1d_zones with the flags of Mesh_coarsening 2 (BULK_ZONE) or 3 (PB_ZONE): every node of a zone above 0
    flagged -888 / -777 (set_mesh_coarsen_flag, src/dft_mesh.c:2816-2824), no averaged rows."""
    z, p = load("lj1d_zones")
    q = copy.copy(p)
    f = np.asarray(p.zone_flag)
    q.zone_flag = np.where(f != 0, -888 if kind == "bulk" else -777, 0).astype(np.int32)
    q.mesh_coarsening = 2 if kind == "bulk" else 3
    return z, q


@pytest.mark.parametrize("kind", ["bulk", "pb"])
def test_bulk_and_pb_zone_rows_match_the_oracle(kind):
    """Fill, J v and J^T w with BULK_ZONE / PB_ZONE rows against the oracle (1e-12) on the fixture's states."""
    from tramonto_gb300 import native
    z, q = _bulk_pb(kind)
    s = native.Solver(q)
    o = orc.Oracle(q)
    N = q.nunk * q.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        R = s.fill(x)
        want = o.resid(x)
        assert np.max(np.abs(R - want)) <= 1e-12 * max(1.0, float(np.abs(want).max())), (kind, k)
        v = probe(N, 0).reshape(x.shape)
        assert rel_err(s.jv(v), o.jv(x, v)) <= PROD_RTOL, (kind, k)
        w = probe(N, 1).reshape(x.shape)
        assert rel_err(s.jtv(w), o.jtv(x, w)) <= PROD_RTOL, (kind, k)
    s.close()


@pytest.mark.parametrize("kind", ["bulk", "pb"])
def test_bulk_and_pb_zone_solution(kind):
    """Newton converges (||R||_2 <= 1e-10) with the flagged nodes at the bulk density (BULK_ZONE) or at the
    ideal gas in the field, rho_b exp(-V_ext) (PB_ZONE), to 1e-12 relative."""
    from tramonto_gb300 import native
    z, q = _bulk_pb(kind)
    s = native.Solver(q)
    x, it, rn, _ = s.newton_solve(z["x_newton"], resid_tol=1e-10, lin_tol=1e-12, lin_max_iter=1000, max_iter=40)
    assert rn <= 1e-10, (kind, it, rn)
    rho = x[q.first_rho]
    flagged = (np.asarray(q.zone_flag) < 0) & (np.asarray(q.zero_density)[0] == 0) & (np.asarray(q.vext)[0] < q.vext_max)
    want = q.rho_b[0] * (1.0 if kind == "bulk" else np.exp(-np.asarray(q.vext)[0][flagged]))
    assert np.max(np.abs(rho[flagged] / want - 1.0)) <= 1e-12, kind
    s.close()


def test_phase_interface_with_averaged_rows_matches_the_oracle():
    """Averaged rows next to both IN_BULK ends of a phase interface: lv1d_bulkbc (BULK3 with bulk ends) with
    the first three and the last two nodes flagged -1, read as with Mesh_coarsening on and a wall present
    (the reference reads the flags only then, and its interface decks have no walls).  Beyond the low end
    the averaged rows take the LBB state, beyond the high end the RTF state (constant_boundary -3 / -4,
    src/dft_utils.c:89-130); fill, J v and J^T w against the oracle (1e-12), and a step solved on the other
    nodes satisfies the full system (1e-9)."""
    from tramonto_gb300 import native
    z, p = load("lv1d_bulkbc")
    q = copy.copy(p)
    f = np.zeros(p.nnodes, np.int32)
    f[[0, 1, 2, p.nnodes - 2, p.nnodes - 1]] = -1
    q.zone_flag, q.nzone, q.mesh_coarsening, q.nwall = f, 1, 1, 1
    q.zone_stencils = {}
    s = native.Solver(q)
    o = orc.Oracle(q)
    N = q.nunk * q.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        R = s.fill(x)
        want = o.resid(x)
        assert np.max(np.abs(R - want)) <= 1e-12 * max(1.0, float(np.abs(want).max())), k
        v = probe(N, 0).reshape(x.shape)
        assert rel_err(s.jv(v), o.jv(x, v)) <= PROD_RTOL, k
        w = probe(N, 1).reshape(x.shape)
        assert rel_err(s.jtv(w), o.jtv(x, w)) <= PROD_RTOL, k
    x = z["x0"]
    s.fill(x)
    b = probe(N, 4).reshape(x.shape)
    b[:, f < 0] = 0.0
    dx, it, rr = s.solve(b, tol=1e-12, max_iter=1000)
    assert np.linalg.norm(s.jv(dx) - b) <= 1e-9 * np.linalg.norm(b), (it, rr)
    s.close()
