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


def test_turning_point_solver_locks_onto_the_condensation_fold(branch):
    """The Moore-Spence bordering algorithm (isotherm.turning_point, the reference's turning_point_alg) started
    from the arclength point next to the condensation turning point converges to a state with ||R||_2 <= 1e-9
    whose Jacobian has the null vector y (||J y|| / ||y|| <= 1e-6), at a beta mu at or beyond every arclength point
    of that stretch of the branch (the fold is the branch's local maximum of beta mu), and at the maximum of a
    quadratic fit beta mu(N) through the five arclength points around it (5e-4 in beta mu, 1e-2 relative in N: the
    fit's own error over points ~0.02 apart in arclength)."""
    from tramonto_gb300 import isotherm
    recs, _ = branch
    k = _turning_points(recs)[0]
    rec = isotherm.turning_point(_spec(), recs[k]["x"], recs[k]["betamu"], tol=1e-9)
    near = [r["betamu"] for r in recs[max(1, k - 5):k + 6]]
    print("fold:", rec["betamu"], "arclength max:", max(near), "iterations", rec["iters"], "||R||", rec["resid"],
          "||Jy||/||y||", rec["jy_rel"])
    assert rec["converged"]
    assert rec["resid"] <= 1e-9
    assert rec["betamu"] >= max(near) - 1e-9
    pts = recs[k - 2:k + 3]
    c2, c1, c0 = np.polyfit([r["N"] for r in pts], [r["betamu"] for r in pts], 2)
    n_fit, mu_fit = -c1 / (2 * c2), c0 - c1 * c1 / (4 * c2)
    print("quadratic fit: beta mu", mu_fit, "N", n_fit, " turning point: N", rec["N"])
    assert abs(rec["betamu"] - mu_fit) <= 5e-4 and abs(rec["N"] - n_fit) <= 1e-2 * n_fit
    assert rec["jy_rel"] <= 1e-6


def test_turning_point_continuation_in_the_wall_strength(branch):
    """Continuation of the condensation fold in the wall strength eps_w (LOCA's turning-point continuation,
    zero order with con_lib's step control), both ways from eps_w = 1: every requested point converges
    (||R||_2 <= 1e-9, ||J y|| / ||y|| <= 1e-6), the fold stays the same one (N within 0.1 of the eps_w = 1
    fold; the branch's next fold is at N ~ 2), and a weaker wall attraction moves it to a higher beta mu,
    nearly linearly (the second difference of beta mu is below a tenth of the first)."""
    from tramonto_gb300 import isotherm
    recs, _ = branch
    k = _turning_points(recs)[0]
    for eps in ([1.0, 0.99, 0.98, 0.97], [1.0, 1.01, 1.02, 1.03]):
        out = isotherm.turning_point_continuation(_spec(), recs[k]["x"], recs[k]["betamu"], eps)
        print([(r["eps_w"], round(r["betamu"], 6), round(r["N"], 5), r["iters"], r["substeps"]) for r in out])
        assert len(out) == 4 and all(r["converged"] and r["resid"] <= 1e-9 and r["jy_rel"] <= 1e-6 for r in out)
        mus = np.array([r["betamu"] for r in out])
        assert all(abs(r["N"] - out[0]["N"]) <= 0.1 for r in out)
        d1 = np.diff(mus) * np.sign(eps[1] - eps[0])
        assert np.all(d1 < 0)
        assert np.max(np.abs(np.diff(d1))) <= 0.1 * np.min(np.abs(d1))


def test_phase_transition_between_the_spinodals(branch):
    """The reference's phase-transition algorithm (isotherm.phase_transition) started from a point of the dilute
    branch and one of the condensed branch near the middle of the hysteresis loop converges to two states at one
    beta mu (||R||_2 <= 1e-9 each) with equal grand free energy (|g| <= 1e-9 of |Omega|), the condensed one holding
    more particles, at a beta mu strictly between the evaporation and condensation turning points."""
    from tramonto_gb300 import isotherm
    recs, _ = branch
    tp = _turning_points(recs)
    mu_cond, mu_evap = recs[tp[0]]["betamu"], recs[tp[1]]["betamu"]
    mu0 = 0.5 * (mu_cond + mu_evap)
    lo = min(recs[1:tp[0]], key=lambda r: abs(r["betamu"] - mu0))
    hi = min(recs[tp[1] + 1:], key=lambda r: abs(r["betamu"] - mu0))
    rec = isotherm.phase_transition(_spec(), lo["x"], hi["x"], mu0, tol=1e-9)
    print("coexistence: beta mu", rec["betamu"], "N", rec["N1"], rec["N2"], "iters", rec["iters"], "g", rec["g"],
          "spinodals", mu_evap, mu_cond, "starts", lo["betamu"], hi["betamu"])
    assert rec["converged"] and rec["resid"] <= 1e-9
    assert mu_evap < rec["betamu"] < mu_cond
    assert rec["N2"] > rec["N1"] + 0.5
    assert abs(rec["g"]) <= 1e-8
