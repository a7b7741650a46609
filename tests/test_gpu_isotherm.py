"""Configuration 5 pieces on the GPU: moving the bulk state of a live problem, the adsorption's
derivative in the chemical potential by the adjoint, and isotherms by continuation.

- tgpu_set_bulk_state on a finalized problem gives the same residual as a problem built at the
  new bulk density (1e-13; the 3-D case has a bulk boundary, so the padded bulk values move too);
- dN/d(beta mu) from one adjoint solve equals the central difference of N over a change of the bulk
  density (which moves beta mu) to 1e-5 relative, in a 1-D and a 2-D slit pore;
- an isotherm by continuation on the liquid side converges at every point, N rises with beta mu and
  dN/d(beta mu) > 0, and its last point equals a solve from scratch to 1e-7;
- mixed-precision and FP64 solves of configuration-5 problems give the same adsorption to 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_set_bulk_state_equals_a_fresh_problem():
    from tramonto_gb300 import native, setup
    p1, _ = setup.config2(n=40, rho_b=0.6)
    p2, _ = setup.config2(n=40, rho_b=0.65)
    s1, s2 = native.Solver(p1), native.Solver(p2)
    x = setup.initial_state(s2, p2)
    s1.set_bulk([0.65])
    for mode in (0, 1):
        r1, r2 = s1.fill(x, mode=mode), s2.fill(x, mode=mode)
        assert np.abs(r1 - r2).max() <= 1e-13 * max(1.0, np.abs(r2).max())
    o1, g1 = s1.objectives(x)
    o2, g2 = s2.objectives(x)
    assert abs(o1 - o2) <= 1e-12 * max(1.0, abs(o2)) and np.allclose(g1, g2, rtol=1e-12, atol=1e-14)
    s1.close()
    s2.close()


@pytest.mark.parametrize("spec", [dict(ndim=1, nx=(501, 1, 1), dx=0.01, rho_b=0.5),
                                  dict(ndim=2, nx=(72, 72, 1), dx=0.05, rho_b=0.45)])
def test_dN_dbetamu_matches_finite_differences(spec):
    from tramonto_gb300 import isotherm, native, setup
    p = setup.slit_pore(spec)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p, max_enhancement=1.0)
    x, it, rn, li, ok = isotherm.solve_state(s, p, x0, mixed=False, resid_tol=1e-11)
    assert ok, rn
    adj = isotherm.dN_dbetamu(s, p, x)[0]
    rb = spec["rho_b"]
    vals = []
    for sgn in (1.0, -1.0):
        s.set_bulk([rb * (1.0 + sgn * 1e-5)])
        xs, _, rns, _, oks = isotherm.solve_state(s, p, x, mixed=False, resid_tol=1e-11)
        assert oks, rns
        vals.append((float(p.betamu[0]), isotherm.adsorption(p, xs)[0]))
    fd = (vals[0][1] - vals[1][1]) / (vals[0][0] - vals[1][0])
    print(spec["ndim"], "dN/dbetamu adjoint", adj, "central difference", fd)
    assert abs(adj - fd) <= 1e-5 * abs(fd)
    s.close()


def test_isotherm_by_continuation():
    from tramonto_gb300 import isotherm
    # the liquid side of the bulk equation of state, where beta mu rises with the bulk density (at kT* = 1.2
    # the mean-field bulk has a van der Waals loop between rho_b ~ 0.2 and 0.3)
    spec = dict(ndim=1, nx=(801, 1, 1), dx=0.01, rho_b=0.75)
    ladder = [0.55, 0.6, 0.65, 0.7, 0.75]
    recs, x_last = isotherm.isotherm(spec, ladder, mixed=False, resid_tol=1e-10)
    print([(r["rho_b"], r["betamu"], r["N"], r.get("dN_dbetamu")) for r in recs])
    assert all(r["converged"] for r in recs)
    mu = [r["betamu"] for r in recs]
    N = [r["N"] for r in recs]
    assert all(b > a for a, b in zip(mu, mu[1:]))
    assert all(b > a for a, b in zip(N, N[1:])) and all(r["dN_dbetamu"] > 0 for r in recs)
    scratch, x_scratch = isotherm.isotherm(spec, [0.75], mixed=False, resid_tol=1e-10, with_derivative=False)
    assert abs(scratch[0]["N"] - N[-1]) <= 1e-7 * N[-1]
    print("iterations along the ladder", [r["iters"] for r in recs], "from scratch", scratch[0]["iters"])


def test_mixed_and_fp64_sweeps_agree():
    from tramonto_gb300 import isotherm, setup
    specs = setup.config5()
    pick = [specs[1], specs[5], specs[33], specs[40]]
    mixed = isotherm.sweep(pick, mixed=True, with_derivative=False)
    plain = isotherm.sweep(pick, mixed=False, with_derivative=False)
    for m, f in zip(mixed, plain):
        assert m["converged"] and f["converged"], (m, f)
        assert abs(m["N"] - f["N"]) <= 1e-6 * abs(f["N"])
