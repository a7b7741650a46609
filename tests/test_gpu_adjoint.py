"""Adjoint of the Euler-Lagrange system on the GPU.

J^T w (tgpu_jtv) against the transpose of the Jacobian the reference assembles
(fixtures JTw*, products of the reference's own matrix) and against the C
oracle; J^T lambda = g (tgpu_adjoint_solve); and sensitivities of the grand
potential (Omega_s, the reference's calc_free_energy) and the excess
adsorption of the converged LJ fluid at a 9-3 wall with respect to the
per-node external field and to the wall parameters
(eps_w, sigma_w), checked against central finite differences with h = 1e-6
and, through a torch.autograd.Function wrapper, by torch.autograd.gradcheck.

Tolerances: J^T w within 1e-12 relative of the reference (same bar as J v);
the adjoint solve to a relative residual of 1e-9; gradients within 1e-5
relative of the finite differences, measured against the largest gradient
component (a central difference with h = 1e-6 carries an absolute error of
~1e-8 here: F(+h) - F(-h) is only known to ~1e-14 of F).
"""
import numpy as np
import pytest

import orc
from goldens import PROD_RTOL, load, probe, rel_err

pytestmark = pytest.mark.gpu

ADJ_CASES = ["lj1d_mf", "mix1d_fmt3", "fmt1_wca_3d", "mix1d_fmt4", "rough3d_fmt2", "rough3d_fmt4",
             "hs1d_wall", "hs1d_c1", "hs1d_fmt2", "hs1d_fmt4", "hs1d_reflect", "hslj1d_wall", "lj1d_a22",
             "lv1d_interface", "lv1d_bulkbc"]
# hs*1d_*: hard-wall boundary weights (hslj1d_wall also on the mean-field stencil); hs1d_reflect also a
# reflecting boundary; lj1d_a22: the mean field summed into the Euler-Lagrange rows (ATTInA22Block = 1);
# lv1d_*: a liquid-vapour interface (bulk states on either side, a pinned density at the mid-plane)
GRAD_RTOL = 1e-5
FD_H = 1e-6


@pytest.mark.parametrize("name", ADJ_CASES)
def test_jtv_matches_reference_transpose(name):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    o = orc.Oracle(p)
    N = p.nunk * p.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        s.fill(x, mode=0)
        w = probe(N, 1).reshape(x.shape)
        got = s.jtv(w)
        assert rel_err(got, z[f"JTw{k}"]) <= PROD_RTOL, (name, k)
        assert rel_err(got, o.jtv(x, w)) <= PROD_RTOL, (name, k)
    s.close()


@pytest.mark.parametrize("name", ADJ_CASES)
def test_jtv_is_the_adjoint_of_jv(name):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    x = z["x0"]
    s.fill(x, mode=0)
    rng = np.random.default_rng(7)
    for _ in range(3):
        u = rng.standard_normal(x.shape)
        v = rng.standard_normal(x.shape)
        lhs = float(np.sum(u * s.jv(v)))
        rhs = float(np.sum(s.jtv(u) * v))
        scale = float(np.abs(u * s.jv(v)).sum())
        assert abs(lhs - rhs) <= 1e-12 * scale, (name, lhs, rhs)
    s.close()


@pytest.mark.parametrize("name", ADJ_CASES)
def test_adjoint_solve(name):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    x = z[f"x{len(z['states']) - 1}"]
    s.fill(x, mode=0)
    N = p.nunk * p.nnodes
    g = probe(N, 3).reshape(x.shape)
    lam, it, rr = s.adjoint_solve(g, tol=1e-12, max_iter=1000)
    r = s.jtv(lam) - g
    assert np.linalg.norm(r) <= 1e-9 * np.linalg.norm(g), (name, it, rr, np.linalg.norm(r))
    # the same residual through the oracle's transposed Jacobian (pinned to the reference's matrix)
    ro = orc.Oracle(p).jtv(x, lam) - g
    assert np.linalg.norm(ro) <= 1e-9 * np.linalg.norm(g), (name, np.linalg.norm(ro))
    # duality with the forward solve: <lambda, b> = <g, J^-1 b>
    b = probe(N, 4).reshape(x.shape)
    dx, _, _ = s.solve(b, tol=1e-12, max_iter=1000)
    lb, gd = float(np.sum(lam * b)), float(np.sum(g * dx))
    assert abs(lb - gd) <= 1e-8 * np.abs(g * dx).sum(), (name, lb, gd)
    s.close()


def _reflecting_3d_problem():
    """16 x 12 x 12 FMT1 + WCA problem at a rough 12-3 wall, reflecting in y, periodic in z."""
    from tramonto_gb300 import setup
    from tramonto_gb300.problem import BC_IN_BULK, BC_IN_WALL, BC_PERIODIC, BC_REFLECT, FMT1
    nx, es = (16, 12, 12), (0.25, 0.25, 0.25)
    vext, _ = setup.rough_wall_vext(nx, es, kT=1.2, patches=4, device=False)
    return setup.build_problem(3, nx, es, ((BC_IN_WALL, BC_IN_BULK), (BC_REFLECT, BC_REFLECT), (BC_PERIODIC, BC_PERIODIC)),
                               hs_diam=[1.0], rho_b=[0.6], functional=FMT1, attraction=True, sigma=[[1.0]],
                               eps=[[1.0 / 1.2]], rcut=[[2.5]], vext=vext)


def test_jtv_is_the_adjoint_of_jv_with_reflecting_boundaries_in_3d():
    """Reflections fold mirrored contributions back with the vector components' sign: <u, J v> = <J^T u, v>
    on a 3-D problem reflecting in y (no reference fixture: J v itself is pinned by the forward parity)."""
    from tramonto_gb300 import native, setup
    p = _reflecting_3d_problem()
    s = native.Solver(p)
    x = setup.initial_state(s, p, max_enhancement=1.0)
    s.fill(x, mode=0)
    rng = np.random.default_rng(11)
    for _ in range(3):
        u = rng.standard_normal(s.shape)
        v = rng.standard_normal(s.shape)
        lhs = float(np.sum(u * s.jv(v)))
        rhs = float(np.sum(s.jtv(u) * v))
        scale = float(np.abs(u * s.jv(v)).sum())
        assert abs(lhs - rhs) <= 1e-12 * scale, (lhs, rhs)
    s.close()


# ---- sensitivities of the converged LJ fluid at a 9-3 wall -----------------

WALL = dict(eps_w=3.0, sigma_w=1.0, cut_w=3.0, x_wall=0.5)   # the lj1d_mf field (9-3 cut and shifted)


class _Fluid:
    """lj1d_mf (FMT1 + mean-field LJ, one component) with the 9-3 wall field as a function of its parameters.

    The objectives are the library's Omega_s and Gamma_ex (the reference's calc_free_energy and
    calc_adsorption integrals); their V_ext sensitivities come from tgpu_grad_omega_vext / _gamma_vext."""

    def __init__(self):
        from tramonto_gb300 import native, setup
        self.z, self.p = load("lj1d_mf")
        p = self.p
        self.dist = np.arange(p.nnodes) * p.esize[0] - WALL["x_wall"]
        self.zero = np.asarray(p.zero_density, bool).reshape(-1)
        self.s = native.Solver(p)
        self.setup = setup
        self.x = np.array(self.z[f"x{len(self.z['states']) - 1}"], copy=True)
        self.vext0 = self.field(WALL["eps_w"], WALL["sigma_w"])[0]
        self.x = self.solve(self.vext0)

    def field(self, eps_w, sigma_w):
        v, de, ds = self.setup.lj93_wall_1d(self.dist, eps_w, sigma_w, WALL["cut_w"], self.p.vext_max)
        v = np.where(self.zero, self.p.vext_max, v)
        de = np.where(self.zero, 0.0, de)
        ds = np.where(self.zero, 0.0, ds)
        return v, de, ds

    def solve(self, vext):
        self.s.set_vext(vext.reshape(1, -1))
        x, it, rn, _ = self.s.newton_solve(self.x, resid_tol=1e-12, lin_tol=1e-12, lin_max_iter=1000,
                                           allow_noconv=True)
        assert rn <= 1e-11, rn
        return x

    def objectives(self, x, vext):
        """(Omega_s, Gamma_ex) at (x, V)."""
        self.s.set_vext(vext.reshape(1, -1))
        om, gam = self.s.objectives(x)
        return om, float(gam[0])

    def gradients(self, x, vext):
        """dOmega_s/dV and dGamma_ex/dV at the converged state (adjoint)."""
        self.s.set_vext(vext.reshape(1, -1))
        return [self.s.grad_vext(x, kind=k, tol=1e-13, max_iter=1000).reshape(-1) for k in (0, 1)]


@pytest.fixture(scope="module")
def fluid():
    f = _Fluid()
    yield f
    f.s.close()


def test_wall_field_restatement_matches_reference_field(fluid):
    v = fluid.vext0
    ref = np.asarray(fluid.p.vext).reshape(-1)
    assert np.abs(v - ref).max() <= 1e-8


def test_vext_gradient_matches_finite_differences(fluid):
    x0, v0 = fluid.x, fluid.vext0
    grads = fluid.gradients(x0, v0)
    live = ~fluid.zero
    idx = np.nonzero(live)[0]
    u = np.zeros_like(v0)
    u[idx] = np.cos(0.37 * np.arange(idx.size)) * np.exp(-0.01 * np.arange(idx.size))
    nodes = [idx[2], idx[25], idx[120]]
    dirs = [u] + [np.eye(1, v0.size, k).reshape(-1) for k in nodes]
    for d in dirs:
        fp = fluid.objectives(fluid.solve(v0 + FD_H * d), v0 + FD_H * d)
        fm = fluid.objectives(fluid.solve(v0 - FD_H * d), v0 - FD_H * d)
        for j, name in enumerate(("Omega_s", "Gamma_ex")):
            fd = (fp[j] - fm[j]) / (2 * FD_H)
            adj = float(np.sum(grads[j] * d))
            # judged against the gradient's size: a central difference with h = 1e-6 resolves
            # F(+h) - F(-h) only to ~1e-14 of F, i.e. ~1e-8 in a derivative
            ref_scale = max(abs(fd), float(np.abs(grads[j]).max() * np.abs(d).max()))
            assert abs(adj - fd) <= GRAD_RTOL * ref_scale, (name, adj, fd)
    fluid.solve(v0)


def test_wall_parameter_gradcheck(fluid):
    import torch

    class GrandPotential(torch.autograd.Function):
        """Omega_s and Gamma_ex of the converged fluid as functions of (eps_w, sigma_w); backward by the adjoint."""

        @staticmethod
        def forward(ctx, theta):
            e, s = float(theta[0]), float(theta[1])
            v, de, ds = fluid.field(e, s)
            x = fluid.solve(v)
            om, ga = fluid.objectives(x, v)
            dom, dga = fluid.gradients(x, v)
            jac = np.array([[np.sum(dom * de), np.sum(dom * ds)], [np.sum(dga * de), np.sum(dga * ds)]])
            ctx.save_for_backward(torch.tensor(jac, dtype=torch.float64))
            return torch.tensor([om, ga], dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            (jac,) = ctx.saved_tensors
            return grad_out @ jac

    theta = torch.tensor([WALL["eps_w"], WALL["sigma_w"]], dtype=torch.float64, requires_grad=True)
    ok = torch.autograd.gradcheck(GrandPotential.apply, (theta,), eps=FD_H, atol=1e-7, rtol=GRAD_RTOL,
                                  nondet_tol=1e-9)
    assert ok


def test_hard_wall_vext_gradient_matches_finite_differences():
    """Configuration 1 (HS5 at L = 20, hard wall with boundary weights): dOmega_s/dV_ext by the adjoint,
    whose J^T includes the transpose of the hard-wall weight correction, against central differences of
    re-converged states."""
    from tramonto_gb300 import native
    z, p = load("hs1d_c1")
    s = native.Solver(p)
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
    u = np.zeros(vext0.size)
    u[live] = np.cos(0.37 * np.arange(live.size)) * np.exp(-0.01 * np.arange(live.size))
    dirs = [u, np.eye(1, vext0.size, live[3]).reshape(-1), np.eye(1, vext0.size, live[40]).reshape(-1)]
    for d in dirs:
        d = d.reshape(vext0.shape)
        om_p = s.objectives(converge(vext0 + FD_H * d, x0))[0]
        om_m = s.objectives(converge(vext0 - FD_H * d, x0))[0]
        fd = (om_p - om_m) / (2 * FD_H)
        adj = float(np.sum(g * d))
        scale = max(abs(fd), float(np.abs(g).max() * np.abs(d).max()))
        assert abs(adj - fd) <= GRAD_RTOL * scale, (adj, fd)
    s.close()
