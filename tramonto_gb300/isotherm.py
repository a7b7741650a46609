"""Slit-pore state points and isotherms (configuration 5) on one GPU.

A state point is a Newton solve of one slit-pore problem (setup.slit_pore) at one
bulk density; its adsorption N_i = sum_nodes w_i rho_i (the integral of
calc_adsorption, src/dft_out_ads.c:33-112) and dN_i/d(beta mu_i) come with it.
The chemical potential enters only the Euler-Lagrange rows, as -beta mu next to
+V_ext (src/dft_fill_EL.c:401-444), so the response to a uniform shift of
beta mu_i is minus the response to a uniform shift of V_ext,i on the rows that
are not zero-density rows:

    dN/d(beta mu_i) = - sum_nodes dN/dV_ext,i    (one adjoint solve per component)

An isotherm is a continuation in the chemical potential (the reference's LOCA
CONT_BETAMU_I steps): the bulk state moves along a ladder of bulk densities and
every solve starts from the previous state point's solution (tgpu_set_bulk_state).
Around turning points (capillary condensation and evaporation in a pore, where
N(beta mu) folds back) natural steps fail; `arclength` follows the branch by
pseudo-arclength continuation (LOCA's arc-length stepper, NOXLOCA_Solver.cpp:51-134,
loca_lib.c:72): the Newton system is bordered by the arclength equation and solved
by the bordering algorithm, two solves with the Jacobian per corrector iteration.
"""
from __future__ import annotations

import time

import numpy as np

from . import native, setup


def adsorption(p, x):
    """N_i = sum_nodes w_fluid,i rho_i."""
    rho = np.asarray(x)[p.first_rho:p.first_rho + p.ncomp]
    return (np.asarray(p.w_fluid) * rho).sum(axis=1)


def dN_dbetamu(s, p, x, tol=1e-12, max_iter=1000):
    """dN_i/d(beta mu_i) at the converged state x (adjoint)."""
    out = np.zeros(p.ncomp)
    for ic in range(p.ncomp):
        g = s.grad_vext(x, kind=1, icomp=ic, tol=tol, max_iter=max_iter)
        out[ic] = -float(g[ic].sum())
    return out


def set_mode(s, mixed):
    if mixed:
        s.set_precision(native.FP32)
        s.set_fill_arithmetic(native.FILL_MIXED, switch_norm=0.1)
    else:
        s.set_precision(native.FP64)
        s.set_fill_arithmetic(native.FILL_FP64)


def solve_state(s, p, x0, mixed=True, resid_tol=1e-8, max_iter=60):
    """Newton solve from x0; returns (x, iterations, ||R||_2, GMRES iterations, converged).  A solve that
    runs into non-finite values (a Newton path through n3 >= 1) returns unconverged with x0."""
    set_mode(s, mixed)
    try:
        x, it, rn, li = s.newton_solve(x0, resid_tol=resid_tol, max_iter=max_iter,
                                       lin_tol=1e-6 if mixed else 1e-10, lin_max_iter=300, allow_noconv=True)
    except native.TgpuError:
        return np.array(x0), max_iter, float("inf"), 0, False
    return x, it, rn, li, bool(rn <= resid_tol)


def isotherm(spec, rho_ladder, mixed=True, resid_tol=1e-8, with_derivative=True):
    """Continuation along the bulk densities rho_ladder of one problem; one record per state point."""
    p = setup.slit_pore(spec, rho_b=rho_ladder[0])
    s = native.Solver(p)
    try:
        x = setup.initial_state(s, p, max_enhancement=1.0)
        out = []
        for k, rb in enumerate(rho_ladder):
            if k > 0:
                s.set_bulk([rb])
            t0 = time.perf_counter()
            x, it, rn, li, ok = solve_state(s, p, x, mixed, resid_tol)
            t_solve = time.perf_counter() - t0
            rec = dict(rho_b=float(rb), betamu=float(p.betamu[0]), N=float(adsorption(p, x)[0]), iters=it, resid=rn,
                       gmres=li, converged=ok, solve_s=t_solve)
            if with_derivative and ok:
                rec["dN_dbetamu"] = float(dN_dbetamu(s, p, x)[0])
            out.append(rec)
        return out, x
    finally:
        s.close()


def ladders_to(rho_b, steps=4):
    """Bulk-density ladders for reaching rho_b by continuation: from the gas side (0.05) and from the liquid
    side (0.55) of the mean-field van der Waals loop (kT* = 1.2: gas below ~0.2, liquid above ~0.3), the
    side rho_b lies on first."""
    gas = list(np.linspace(0.05, rho_b, steps))
    liquid = list(np.linspace(0.55, rho_b, steps))
    return [gas, liquid] if rho_b < 0.25 else [liquid, gas]


def sweep(specs, mixed=True, resid_tol=1e-8, with_derivative=True):
    """Every configuration-5 problem at its own state point, solved from its initial state; a state point
    that does not converge directly is reached by continuation along ladders_to(rho_b)."""
    recs = []
    for spec in specs:
        t0 = time.perf_counter()
        r, _ = isotherm(spec, [spec["rho_b"]], mixed, resid_tol, with_derivative)
        rec = r[0]
        rec["path"] = "direct"
        for ladder in ([] if rec["converged"] else ladders_to(spec["rho_b"])):
            r, _ = isotherm(spec, ladder, mixed, resid_tol, with_derivative)
            rec = r[-1]
            rec["path"] = f"continuation from {ladder[0]:.2f}"
            rec["iters"] = sum(q["iters"] for q in r)
            if rec["converged"]:
                break
        rec["wall_s"] = time.perf_counter() - t0
        rec["ndim"], rec["nodes"] = spec["ndim"], int(np.prod(spec["nx"][:spec["ndim"]]))
        recs.append(rec)
    return recs


def _live_rows(p):
    """Euler-Lagrange rows that carry -beta mu (not zero-density rows)."""
    v = np.asarray(p.vext, np.float64).reshape(p.ncomp, -1)
    z = np.asarray(p.zero_density).reshape(p.ncomp, -1) != 0
    return ~z & (v < p.vext_max)


def arclength(spec, rho_b0, n_steps, ds=0.02, ds_min=1e-5, ds_max=0.2, direction=1, mixed=False, tol=1e-9,
              max_corrector=12, x0=None, stop=None, keep_states=False):
    """Pseudo-arclength continuation in beta mu of one configuration-5 pore problem (one component).

    The branch is parametrised by arclength in (rho, beta mu) with the density part measured as
    (sum_i w_i drho_i^2 / sum_i w_i)^(1/2) (w: integration weights).  Starting from the converged state at
    bulk density rho_b0 (or from x0), each step predicts along the tangent, then corrects with Newton on
        R(x, mu) = 0,   t_x . (x - x_k) + t_mu (mu - mu_k) - ds = 0
    by the bordering algorithm (J a = -R, J b = -dR/dmu, dmu = -(g + t_x.a)/(t_x.b + t_mu), dx = a + dmu b),
    with the density-positivity fraction of update_solution applied to the whole step.  The step halves
    when the corrector fails and grows by 1.5 when it converges in 3 iterations or fewer; the next tangent is
    the secant of the last step.  Returns one record per point: beta mu, N, ||R||_2, corrector iterations,
    the tangent's mu component (its sign changes at turning points) and the step length (and the state,
    with keep_states).  stop(record) ends the continuation early when it returns True."""
    p = setup.slit_pore(spec, rho_b=rho_b0)
    if p.ncomp != 1:
        raise ValueError("one component")
    s = native.Solver(p)
    try:
        set_mode(s, mixed)
        if x0 is None:
            x0 = setup.initial_state(s, p, max_enhancement=1.0)
        x, _, rn, _, ok = solve_state(s, p, x0, mixed, resid_tol=tol)
        if not ok:
            raise RuntimeError(f"no converged start at rho_b = {rho_b0} (||R||_2 = {rn:.2e})")
        r0 = p.first_rho
        wv = np.asarray(p.w_fluid, np.float64).reshape(-1)
        W = wv / wv.sum()
        live = _live_rows(p)[0]
        R_mu = np.zeros(s.shape)
        R_mu[r0][live] = -1.0
        lin_tol = 1e-6 if mixed else 1e-12

        def dot(a, b):
            return float(np.sum(W * a[r0] * b[r0]))

        def lin(rhs):
            return s.solve(rhs, tol=lin_tol, max_iter=1000)[0]

        mu = float(p.betamu[0])
        s.set_chemical_potential([mu])
        s.fill(x, mode=0)
        b = lin(-R_mu)
        nrm = np.sqrt(dot(b, b) + 1.0)
        tx, tm = direction * b / nrm, direction * 1.0 / nrm
        recs = [dict(betamu=mu, N=float(adsorption(p, x)[0]), resid=float(rn), iters=0, t_mu=tm, ds=0.0)]
        if keep_states:
            recs[0]["x"] = x.copy()

        def corrector(xc, mc, xk, mk):
            for it in range(max_corrector + 1):
                s.set_chemical_potential([mc])
                R = s.fill(xc, mode=0)
                g = dot(tx, xc - xk) + tm * (mc - mk) - ds
                rn_c = float(np.linalg.norm(R))
                if not np.isfinite(rn_c):
                    return False, xc, mc, it, rn_c
                if rn_c <= tol and abs(g) <= tol:
                    return True, xc, mc, it, rn_c
                if it == max_corrector:
                    break
                a = lin(-R)
                bb = lin(-R_mu)
                den = dot(tx, bb) + tm
                if den == 0.0 or not np.isfinite(den):
                    return False, xc, mc, it, rn_c
                dm = -(g + dot(tx, a)) / den
                dxv = a + dm * bb
                rho, drho = xc[r0], dxv[r0]
                neg = live & (drho < -0.9 * rho)
                f = min(1.0, float(np.min(-0.9 * rho[neg] / drho[neg]))) if neg.any() else 1.0
                xc = xc + f * dxv
                mc = mc + f * dm
            return False, xc, mc, max_corrector, rn_c

        for _ in range(n_steps):
            while True:
                xp = x + ds * tx
                xp[r0] = np.where(live, np.maximum(xp[r0], 1e-12), xp[r0])
                ok, xn, mn, its, rn_c = corrector(xp, mu + ds * tm, x, mu)
                if ok:
                    break
                ds *= 0.5
                if ds < ds_min:
                    raise RuntimeError(f"arclength step below {ds_min} at beta mu = {mu:.6f}")
            sx, sm = xn - x, mn - mu
            nrm = np.sqrt(dot(sx, sx) + sm * sm)
            tx, tm = sx / nrm, sm / nrm
            x, mu = xn, mn
            recs.append(dict(betamu=mu, N=float(adsorption(p, x)[0]), resid=rn_c, iters=its, t_mu=tm, ds=ds))
            if keep_states:
                recs[-1]["x"] = x.copy()
            if stop is not None and stop(recs[-1]):
                break
            if its <= 3:
                ds = min(1.5 * ds, ds_max)
        return recs, x
    finally:
        s.close()
