"""The bordering algorithms of isotherm.py (turning points and phase transitions) on a CPU stand-in for the solver.

A mean-field lattice gas on n nodes, R_i = ln x_i - ln(1 - x_i) - eps (K x)_i + V_i - beta mu with K_ij = 1/n,
the grand free energy per node Omega = (1/n) sum [x ln x + (1 - x) ln(1 - x) - (eps/2) x (K x) + (V - beta mu) x]
(R_i = n dOmega/dx_i).  With V = 0 its uniform states follow beta mu(rho) = ln(rho / (1 - rho)) - eps rho:
spinodals where rho (1 - rho) = 1 / eps, and by the symmetry rho <-> 1 - rho coexistence at beta mu = -eps / 2.
The stand-in offers the Solver methods the algorithms call (fill, solve, jv, set_chemical_potential,
set_integration, objectives) with dense FP64 linear algebra, so the algorithms' iterations are checked against
these closed forms without a GPU.
"""
import numpy as np
import pytest

from tramonto_gb300 import isotherm, native

EPS, N = 5.0, 20


class _Problem:
    def __init__(self, n):
        self.ncomp, self.first_rho = 1, 0
        self.vext = np.zeros((1, n))
        self.zero_density = np.zeros((1, n), np.int8)
        self.vext_max = 10.0
        self.w_fluid = np.full((1, n), 1.0 / n)
        self.w_bulk = self.w_fluid.copy()
        self.rhobar_b = np.zeros(4)


class _LatticeGas:
    def __init__(self, n=N, eps=EPS):
        self.n, self.eps = n, eps
        self.shape = (1, n)
        self.K = np.full((n, n), 1.0 / n)
        self.mu = 0.0
        self.J = None

    def set_chemical_potential(self, betamu):
        self.mu = float(np.asarray(betamu).reshape(-1)[0])
        self.J = None

    def set_integration(self, w_fluid, w_bulk, rhobar_b, betamu):
        self.mu = float(np.asarray(betamu).reshape(-1)[0])

    def _check(self, x):
        if not (np.all(x > 0.0) and np.all(x < 1.0)):
            raise native.TgpuError(native.TGPU_ERR_DOMAIN, "density outside (0, 1)")

    def fill(self, x, mode=0):
        x = np.asarray(x, np.float64).reshape(self.shape)
        self._check(x)
        r = x[0]
        R = np.log(r) - np.log1p(-r) - self.eps * (self.K @ r) - self.mu
        self.J = np.diag(1.0 / r + 1.0 / (1.0 - r)) - self.eps * self.K
        return R.reshape(self.shape)

    def jv(self, v):
        return (self.J @ np.asarray(v, np.float64).reshape(-1)).reshape(self.shape)

    def solve(self, rhs, tol=1e-12, max_iter=1000):
        return np.linalg.solve(self.J, np.asarray(rhs, np.float64).reshape(-1)).reshape(self.shape), 1, 0.0

    def objectives(self, x):
        x = np.asarray(x, np.float64).reshape(self.shape)
        self._check(x)
        r = x[0]
        om = np.mean(r * np.log(r) + (1.0 - r) * np.log1p(-r) - 0.5 * self.eps * r * (self.K @ r) - self.mu * r)
        return float(om), np.zeros(1)


def _uniform_mu(rho, eps=EPS):
    return np.log(rho / (1.0 - rho)) - eps * rho


@pytest.mark.parametrize("rho0, sign", [(0.24, -1.0), (0.75, 1.0)])
def test_turning_point_of_the_lattice_gas(rho0, sign):
    """From a uniform state near a spinodal, the Moore-Spence iterations reach it: beta mu = beta mu(rho_s) to 1e-10
    and rho (1 - rho) = 1/eps to 1e-6 (beta mu is quadratic in rho - rho_s there, so the fold's density is the
    ill-conditioned coordinate), with ||J y|| / ||y|| <= 1e-6 (the extended Newton's basin is not the nearest fold's
    everywhere: from 0.25 it reaches the dense spinodal)."""
    s, p = _LatticeGas(), _Problem(N)
    rho_s = 0.5 * (1.0 + sign * np.sqrt(1.0 - 4.0 / EPS))
    x0 = np.full((1, N), rho0)
    x, mu, y, it, rn, jy, ok = isotherm._tp_solver(s, p, x0, _uniform_mu(rho0), tol=1e-12)
    assert ok, (it, rn, jy)
    assert np.max(np.abs(x - rho_s)) <= 1e-6
    assert abs(mu - _uniform_mu(rho_s)) <= 1e-10
    assert jy <= 1e-6


def test_phase_transition_of_the_lattice_gas():
    """From uniform dilute and dense states at beta mu0 = -2.3, the phase-transition iterations reach the
    coexistence of the symmetric lattice gas: beta mu = -eps/2, rho2 = 1 - rho1 with beta mu(rho1) = -eps/2,
    equal grand free energies."""
    s, p = _LatticeGas(), _Problem(N)
    rec = isotherm._pt_solver(s, p, np.full((1, N), 0.1), np.full((1, N), 0.9), -2.3, tol=1e-12)
    assert rec["converged"], rec["iters"]
    assert abs(rec["betamu"] + 0.5 * EPS) <= 1e-10
    r1, r2 = float(rec["x1"].mean()), float(rec["x2"].mean())
    assert abs(r1 + r2 - 1.0) <= 1e-10 and abs(_uniform_mu(r1) + 0.5 * EPS) <= 1e-10
    assert abs(rec["g"]) <= 1e-12


@pytest.mark.parametrize("mu0", [-2.7, -2.45])
def test_phase_transition_from_either_side(mu0):
    s, p = _LatticeGas(), _Problem(N)
    rec = isotherm._pt_solver(s, p, np.full((1, N), 0.08), np.full((1, N), 0.93), mu0, tol=1e-12)
    assert rec["converged"] and abs(rec["betamu"] + 0.5 * EPS) <= 1e-10
