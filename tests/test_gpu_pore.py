"""Adjoint sensitivities on the binary White-Bear pore workload.

Binary FMT3 hard spheres (sigma 1 and 0.5, rho_b 0.3 and 0.6) in a
cylindrical pore along z with a soft 9-3 shell of strength eps_w and a
0.5 kT Gaussian random field (setup.config3).

- On a 32x32x24 sub-box (pore radius 1.5): the residual, J v and J^T w of
  the GPU equal the C oracle's (restated reference fill) at the converged
  state and at a perturbed one (1e-12, as the fixture parity tests); the
  sensitivities of Omega_s and of both species' Gamma_ex to single V_ext
  nodes, to a smooth V_ext direction and to eps_w match central finite
  differences with h = 1e-6.
- At the full 96x96x64 size: the same sensitivities to eps_w and to the
  random field's amplitude (the direction V_ext += h * field).

Tolerance: 1e-5 of the largest gradient component times the perturbation's
size (the central differences carry ~1e-8 absolute error), and 1e-5 relative
for the eps_w and amplitude derivatives.
"""
import numpy as np
import pytest

import orc
from goldens import probe, rel_err

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-5
FD_H = 1e-6


def _solve(s, x0, tol):
    x, it, rn, _ = s.newton_solve(x0, resid_tol=tol, lin_tol=1e-11, lin_max_iter=500, max_iter=60,
                                  allow_noconv=True)
    assert rn <= 10 * tol, rn
    return x


def _objectives(s, x):
    om, gam = s.objectives(x)
    return np.concatenate([[om], gam])


def _setup(nx, radius, tol):
    from tramonto_gb300 import native, setup
    p, meta = setup.config3(nx=nx, pore_radius=radius)
    s = native.Solver(p)
    x = _solve(s, setup.initial_state(s, p, max_enhancement=1.0), tol)
    return p, meta, s, x


def _fd(s, p, x, v0, d, tol):
    """Central difference of (Omega_s, Gamma_ex...) along V_ext += h d."""
    out = []
    for sgn in (1.0, -1.0):
        s.set_vext(v0 + sgn * FD_H * d)
        out.append(_objectives(s, _solve(s, x, tol)))
    s.set_vext(v0)
    return (out[0] - out[1]) / (2 * FD_H)


def _adjoint(s, p, x):
    """Rows: dOmega_s/dV, dGamma_ex[0]/dV, dGamma_ex[1]/dV ([ncomp][N] each)."""
    g = [s.grad_vext(x, kind=0, tol=1e-13, max_iter=1000)]
    for c in range(p.ncomp):
        g.append(s.grad_vext(x, kind=1, icomp=c, tol=1e-13, max_iter=1000))
    return g


def test_subbox_fill_and_products_match_oracle():
    p, meta, s, x = _setup((32, 32, 24), 1.5, 1e-11)
    o = orc.Oracle(p)
    rng = np.random.default_rng(5)
    xp = x * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, x.shape))
    N = p.nunk * p.nnodes
    for xs in (x, xp):
        R = s.fill(xs, mode=0)
        assert np.abs(R - o.resid(xs)).max() <= 1e-12
        v = probe(N, 0).reshape(xs.shape)
        assert rel_err(s.jv(v), o.jv(xs, v)) <= 1e-12
        w = probe(N, 1).reshape(xs.shape)
        assert rel_err(s.jtv(w), o.jtv(xs, w)) <= 1e-12
    s.close()


def test_subbox_sensitivities_match_finite_differences():
    p, meta, s, x = _setup((32, 32, 24), 1.5, 1e-12)
    v0 = np.array(p.vext)
    grads = _adjoint(s, p, x)
    live = np.nonzero(np.asarray(p.zero_density[0]) == 0)[0]
    dirs = []
    for k in (live[len(live) // 3], live[2 * len(live) // 3]):
        d = np.zeros_like(v0)
        d[0, k] = 1.0
        d[1, k] = 1.0 if p.zero_density[1][k] == 0 else 0.0
        dirs.append(d)
    dirs.append(np.where(np.asarray(p.zero_density) == 0, meta["grf"].reshape(1, -1), 0.0))
    dirs.append(meta["dv_deps"])                    # eps_w: V_ext changes by h dV/deps_w
    for d in dirs:
        fd = _fd(s, p, x, v0, d, 1e-12)
        for j, g in enumerate(grads):
            adj = float(np.sum(g * d))
            scale = max(abs(fd[j]), float(np.abs(g).max() * np.abs(d).max()))
            assert abs(adj - fd[j]) <= GRAD_RTOL * scale, (j, adj, fd[j])
    s.close()


def test_full_size_eps_w_and_field_sensitivities():
    p, meta, s, x = _setup((96, 96, 64), 5.0, 1e-10)
    v0 = np.array(p.vext)
    grads = _adjoint(s, p, x)
    d_field = np.where(np.asarray(p.zero_density) == 0, meta["grf"].reshape(1, -1), 0.0)   # d/d(amplitude)
    for d in (meta["dv_deps"], d_field):
        fd = _fd(s, p, x, v0, d, 1e-10)
        for j, g in enumerate(grads):
            adj = float(np.sum(g * d))
            assert abs(adj - fd[j]) <= GRAD_RTOL * max(abs(fd[j]), 1e-6), (j, adj, fd[j])
    s.close()
