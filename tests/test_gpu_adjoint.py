"""Adjoint of the Euler-Lagrange system on the GPU.

J^T w (tgpu_jtv) against the transpose of the Jacobian the reference assembles
(fixtures JTw*, products of the reference's own matrix) and against the C
oracle; J^T lambda = g (tgpu_adjoint_solve); and sensitivities of the grand
potential and the excess adsorption of the converged LJ fluid at a 9-3 wall
with respect to the per-node external field and to the wall parameters
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

ADJ_CASES = ["lj1d_mf", "mix1d_fmt3", "fmt1_wca_3d"]
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


def test_transpose_rejects_reflecting_boundaries():
    from tramonto_gb300 import native
    z, p = load("hs1d_reflect")
    s = native.Solver(p)
    s.fill(z["x0"], mode=0)
    with pytest.raises(native.TgpuError) as e:
        s.jtv(np.zeros(s.shape))
    assert e.value.status == -4
    s.close()


# ---- sensitivities of the converged LJ fluid at a 9-3 wall -----------------

WALL = dict(eps_w=3.0, sigma_w=1.0, cut_w=3.0, x_wall=0.5)   # the lj1d_mf field (9-3 cut and shifted)


def _phi_fmt1(n, ndim):
    """Rosenfeld FMT free-energy density on SV-ordered weighted densities (torch)."""
    import torch
    n3, n2, n1, n0 = n[0], n[1], n[2], n[3]
    V2 = n[4:4 + ndim]
    V1 = n[4 + ndim:4 + 2 * ndim]
    one = 1.0 - n3
    v1v2 = (V1 * V2).sum(0)
    v2v2 = (V2 * V2).sum(0)
    return -n0 * torch.log(one) + (n1 * n2 - v1v2) / one + (n2 ** 3 - 3.0 * n2 * v2v2) / (24.0 * np.pi * one ** 2)


class _Fluid:
    """lj1d_mf (FMT1 + mean-field LJ, one component) with the 9-3 wall field as a function of its parameters."""

    def __init__(self):
        from tramonto_gb300 import native, setup
        self.z, self.p = load("lj1d_mf")
        p = self.p
        self.dist = np.arange(p.nnodes) * p.esize[0] - WALL["x_wall"]
        self.zero = np.asarray(p.zero_density, bool).reshape(-1)
        self.s = native.Solver(p)
        self.setup = setup
        self.dv = float(p.esize[0])
        self.mu = -(np.log(p.rho_b[0]) + p.betamu_hs_ex[0] + p.betamu_att[0])
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
        """(Omega, Gamma) at (x, V) and their partial gradients in x and V (torch autograd, float64)."""
        import torch
        p = self.p
        with torch.enable_grad():   # also inside a torch.autograd.Function forward
            xt = torch.tensor(x, dtype=torch.float64, requires_grad=True)
            vt = torch.tensor(vext, dtype=torch.float64, requires_grad=True)
            live = torch.tensor(~self.zero)
            rho = xt[p.first_rho]
            rl = torch.where(live, rho, torch.ones_like(rho))
            ideal = torch.where(live, rl * (torch.log(rl) - 1.0) + (vt + self.mu) * rl + 0.5 * rl * xt[p.first_mf],
                                torch.zeros_like(rl))
            omega = self.dv * (ideal.sum() + _phi_fmt1(xt[p.first_rb:p.first_rb + p.nrb], p.ndim).sum())
            gamma = self.dv * torch.where(live, rho - p.rho_b[0], torch.zeros_like(rho)).sum()
            out = []
            for f in (omega, gamma):
                gx, gv = torch.autograd.grad(f, (xt, vt), retain_graph=True, allow_unused=True)
                gv = np.zeros(vext.shape) if gv is None else gv.numpy()
                out.append((f.item(), gx.numpy(), gv))
        return out

    def gradients(self, x, vext):
        """dOmega/dV and dGamma/dV at the converged state (adjoint)."""
        p = self.p
        self.s.set_vext(vext.reshape(1, -1))
        self.s.fill(x, mode=0)
        res = []
        for f, gx, gv in self.objectives(x, vext):
            lam, it, rr = self.s.adjoint_solve(gx, tol=1e-13, max_iter=1000)
            dv = gv - np.where(self.zero, 0.0, lam[p.first_rho])
            res.append((f, dv))
        return res


@pytest.fixture(scope="module")
def fluid():
    f = _Fluid()
    yield f
    f.s.close()


def test_phi_gradient_matches_oracle(fluid):
    import torch
    p = fluid.p
    o = orc.Oracle(p)
    n = torch.tensor(fluid.x[p.first_rb:p.first_rb + p.nrb], dtype=torch.float64, requires_grad=True)
    (g,) = torch.autograd.grad(_phi_fmt1(n, p.ndim).sum(), n)
    d = o.dphi(fluid.x)                      # S0 S1 S2 S3 V1 V2
    nd = p.ndim
    ref = np.concatenate([d[3:4], d[2:3], d[1:2], d[0:1], d[4 + nd:4 + 2 * nd], d[4:4 + nd]])
    assert rel_err(g.numpy(), ref) <= 1e-12


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
        for j, name in enumerate(("Omega", "Gamma")):
            fd = (fp[j][0] - fm[j][0]) / (2 * FD_H)
            adj = float(np.sum(grads[j][1] * d))
            # judged against the gradient's size: a central difference with h = 1e-6 resolves
            # F(+h) - F(-h) only to ~1e-14 of F, i.e. ~1e-8 in a derivative
            ref_scale = max(abs(fd), float(np.abs(grads[j][1]).max() * np.abs(d).max()))
            assert abs(adj - fd) <= GRAD_RTOL * ref_scale, (name, adj, fd)
    fluid.solve(v0)


def test_wall_parameter_gradcheck(fluid):
    import torch

    class GrandPotential(torch.autograd.Function):
        """Omega and Gamma of the converged fluid as functions of (eps_w, sigma_w); backward by the adjoint."""

        @staticmethod
        def forward(ctx, theta):
            e, s = float(theta[0]), float(theta[1])
            v, de, ds = fluid.field(e, s)
            x = fluid.solve(v)
            (om, dom), (ga, dga) = fluid.gradients(x, v)
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
