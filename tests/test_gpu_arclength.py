"""Pseudo-arclength continuation in the chemical potential (tramonto_gb300/isotherm.py `arclength`).

* beta mu set directly (`set_chemical_potential`) enters only the live Euler-Lagrange rows, with
  dR/d(beta mu) = -1 there: checked against the difference of two fills (1e-12).
* A 6-sigma slit pore at kT* = 1.0 has a capillary-condensation loop: N(beta mu) folds back between
  the evaporation and condensation spinodals.  The continuation from the dilute state follows the branch
  through both turning points (the tangent's beta mu component changes sign twice, the condensation
  turning point at the larger beta mu), every point solves the Euler-Lagrange system at its own beta mu
  (||R||_2 <= 1e-9, re-evaluated by a separate fill), and the stable branches agree with solves
  warm-started by natural continuation at the same beta mu (N to 1e-7 relative).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WIDTH, KT, DX = 6.0, 1.0, 0.01


def _spec(rho_b=0.01):
    return dict(ndim=1, nx=[int(round(WIDTH / DX)) + 1], dx=DX, rho_b=rho_b, kT=KT)


def test_chemical_potential_enters_live_rows_only():
    from tramonto_gb300 import isotherm, native, setup
    p = setup.slit_pore(_spec())
    s = native.Solver(p)
    x = setup.initial_state(s, p, max_enhancement=1.0)
    mu = float(p.betamu[0])
    s.set_chemical_potential([mu])
    r0 = s.fill(x)
    s.set_chemical_potential([mu + 1.0])
    r1 = s.fill(x)
    want = np.zeros_like(r0)
    want[p.first_rho][isotherm._live_rows(p)[0]] = -1.0
    assert np.abs((r1 - r0) - want).max() <= 1e-12
    s.close()


@pytest.fixture(scope="module")
def branch():
    from tramonto_gb300 import isotherm
    recs, x_end = isotherm.arclength(_spec(), 0.01, n_steps=400, ds=0.01, ds_max=0.02, tol=1e-9,
                                     stop=lambda r: r["N"] / WIDTH > 0.5, keep_states=True)
    return recs, x_end


def _turning_points(recs):
    t = np.array([r["t_mu"] for r in recs[1:]])
    return [i + 1 for i in np.nonzero(np.sign(t[1:]) != np.sign(t[:-1]))[0]]


def test_arclength_passes_both_turning_points(branch):
    recs, _ = branch
    tp = _turning_points(recs)
    assert len(tp) == 2, [round(r["betamu"], 4) for r in recs[::10]]
    mu_cond, mu_evap = recs[tp[0]]["betamu"], recs[tp[1]]["betamu"]
    assert mu_cond > mu_evap + 0.05, (mu_cond, mu_evap)
    assert recs[tp[0]]["N"] < recs[tp[1]]["N"]
    assert recs[-1]["N"] / WIDTH > 0.5


def test_arclength_points_solve_their_own_state(branch):
    from tramonto_gb300 import native, setup
    recs, _ = branch
    p = setup.slit_pore(_spec())
    s = native.Solver(p)
    worst = 0.0
    for r in recs[::5]:
        s.set_chemical_potential([r["betamu"]])
        worst = max(worst, float(np.linalg.norm(s.fill(r["x"]))))
    s.close()
    assert worst <= 1e-9, worst


def test_stable_branches_match_natural_continuation(branch):
    from tramonto_gb300 import isotherm, native, setup
    recs, x_end = branch
    tp = _turning_points(recs)
    p = setup.slit_pore(_spec())
    s = native.Solver(p)
    isotherm.set_mode(s, False)
    # gas-like branch: upward in beta mu from the dilute start
    lower = [r for r in recs[1:tp[0]] if r["betamu"] < recs[tp[1]]["betamu"] - 0.05][::4]
    x = recs[0]["x"]
    for r in lower:
        s.set_chemical_potential([r["betamu"]])
        x, _, rn, _, ok = isotherm.solve_state(s, p, x, False, resid_tol=1e-10)
        assert ok, rn
        n_nat = float(isotherm.adsorption(p, x)[0])
        assert abs(n_nat - r["N"]) <= 1e-7 * abs(r["N"]), (r["betamu"], n_nat, r["N"])
    # liquid-like branch: downward in beta mu from the condensed end
    upper = [r for r in recs[tp[1] + 1:] if r["betamu"] > recs[tp[0]]["betamu"] + 0.05][::-4]
    x = x_end
    for r in upper:
        s.set_chemical_potential([r["betamu"]])
        x, _, rn, _, ok = isotherm.solve_state(s, p, x, False, resid_tol=1e-10)
        assert ok, rn
        n_nat = float(isotherm.adsorption(p, x)[0])
        assert abs(n_nat - r["N"]) <= 1e-7 * abs(r["N"]), (r["betamu"], n_nat, r["N"])
    s.close()
