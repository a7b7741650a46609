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
