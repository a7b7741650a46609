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


def _tp_solver(s, p, x, mu, y=None, tol=1e-9, max_iter=40, perturb=1e-6, lin_tol=1e-12, log=None):
    """Moore-Spence turning-point iterations on a live solver (see turning_point); returns (x, mu, y,
    iterations, ||R||_2, ||J y|| / ||y||, converged)."""
    r0 = p.first_rho
    live = _live_rows(p)[0]
    R_mu = np.zeros(s.shape)
    R_mu[r0][live] = -1.0
    n_unk = float(s.shape[0] * s.shape[1])

    def lt(v):                     # ltransnorm with phi = ones: the mean of v over all unknowns
        return float(v.sum()) / n_unk

    def lin(rhs):
        return s.solve(rhs, tol=lin_tol, max_iter=2000)[0]

    def djy(v, h, Jy):
        """(J(x + h v) y - J(x) y) / h; where x + h v leaves the functional's domain (a density <= 0 next to
        a wall, where v is large) the backward difference, then steps 16 and 256 times smaller, are taken."""
        for hh in (h, -h, h / 16, -h / 16, h / 256, -h / 256):
            try:
                s.fill(x + hh * v, mode=0)
            except native.TgpuError as err:
                if err.status != native.TGPU_ERR_DOMAIN:
                    raise
                continue
            return (s.jv(y) - Jy) / hh
        raise native.TgpuError(native.TGPU_ERR_DOMAIN, "no finite-difference step inside the domain")

    rn, jy_rel = float("inf"), float("inf")
    R = None
    for it in range(max_iter + 1):
        if R is None:                            # (a later iteration's residual comes from the update below)
            s.set_chemical_potential([mu])
            R = s.fill(x, mode=0)
        rn = float(np.linalg.norm(R))
        a = lin(R)                               # J a = R (a = -dx of a Newton step)
        b = lin(R_mu)                            # J b = dR/dmu
        if y is None:                            # first iteration: the null vector guess is b, normalised
            y = b / lt(b)
        else:
            y = y / lt(y)
        Jy = s.jv(y)
        jy_rel = float(np.linalg.norm(Jy) / max(np.linalg.norm(y), 1e-300))
        if log is not None:
            log(it, mu, rn, jy_rel)
        if it > 0 and rn <= tol and abs(dmu) <= 1e-10 * (1.0 + abs(mu)) and r_upd <= 1.0:
            return x, mu, y, it, rn, jy_rel, True
        if it == max_iter:
            break
        xnorm = float(np.sqrt(np.sum(x * x)))
        ha = perturb * (perturb + xnorm / max(float(np.sqrt(np.sum(a * a))), 1e-300))
        hb = perturb * (perturb + xnorm / max(float(np.sqrt(np.sum(b * b))), 1e-300))
        dJy_a = djy(a, ha, Jy)
        dJy_b = djy(b, hb, Jy)
        s.fill(x, mode=0)                        # back to the Jacobian at x for the last two solves
        # the reference's linear_solver_conwrap solves with the negated right-hand side of
        # calc_rhs_continuation, so these are its c and d
        c = lin(dJy_a)                           # TP_CONT_SOL3 (AGS_option 0): J c = (d/dx J y) a
        d = lin(dJy_b)                           # TP_CONT_SOL4: J d = (d/dx J y) b (J does not depend on beta mu)
        den = lt(d)
        if den == 0.0 or not np.isfinite(den):
            break
        dmu = (1.0 - lt(c)) / den
        y_new = c + dmu * d
        # the null vector's scaled update (reltol 1e-6, abstol 1e-9; converged below 1)
        r_upd = float(np.sqrt(np.mean(((y_new - y) / (np.abs(y_new) * 1e-6 + 1e-9)) ** 2)))
        dx = -a - dmu * b
        rho, drho = x[r0], dx[r0]                # the density-positivity fraction of update_solution
        neg = live & (drho < -0.9 * rho)
        f = min(1.0, float(np.min(-0.9 * rho[neg] / drho[neg]))) if neg.any() else 1.0
        # an update that leaves the functional's domain (a packing fraction n3 >= 1) is halved until the
        # residual can be taken again; eight halvings without success end the solve unconverged
        R = None
        for _ in range(9):
            s.set_chemical_potential([mu + f * dmu])
            try:
                R = s.fill(x + f * dx, mode=0)
                break
            except native.TgpuError as err:
                if err.status != native.TGPU_ERR_DOMAIN:
                    raise
                f *= 0.5
        if R is None:
            break
        x = x + f * dx
        mu = mu + f * dmu
        y = y_new
    return x, mu, y, max_iter, rn, jy_rel, False


def turning_point(spec, x0, mu0, y0=None, mixed=False, tol=1e-9, max_iter=40, perturb=1e-6, log=None):
    """A turning point (spinodal) of the beta mu branch of a one-component pore problem, located by the
    reference's Moore-Spence bordering algorithm (turning_point_alg, src/loca_bord.c:164-420, AGS_option 0).

    Unknowns: the state x, beta mu and the null vector y of the Jacobian J, normalised by <y, phi>/n = 1 with
    phi = ones (calc_scale_vec_conwrap, src/dft_continuation.c:501-528; ltransnorm, src/loca_util.c:209).
    Each iteration solves four systems with J at x,
        J a = R,   J b = dR/dmu,   J c = (J(x + h_a a) y - J(x) y)/h_a,   J d = (J(x + h_b b) y - J(x) y)/h_b
    (h_v = perturb (perturb + |x|/|v|); the right-hand sides of calc_rhs_continuation TP_CONT_SOL2-4,
    src/loca_bord.c:1352-1520, negated as its linear solver takes them; beta mu enters R linearly, dR/dmu = -1
    on the live Euler-Lagrange rows, so J does not depend on it), then
        dmu = (1 - <c, phi>/n) / (<d, phi>/n),   y <- c + dmu d,   x <- x - a - dmu b,   mu <- mu + dmu,
    with the density-positivity fraction of update_solution on the state update.  Starts from a state
    (x0, mu0) near the fold (e.g. an arclength point where the tangent's mu component changes sign); y0, a
    null vector guess (the previous fold's), is optional.  Returns a record: beta mu, N, ||R||_2,
    ||J y|| / ||y||, iterations, converged, and the state and null vector."""
    p = setup.slit_pore(spec)
    if p.ncomp != 1:
        raise ValueError("one component")
    s = native.Solver(p)
    try:
        set_mode(s, mixed)
        x = np.array(x0, np.float64)
        live = _live_rows(p)[0]
        rho = x[p.first_rho]
        rho[~live] = 0.0                         # rows that are zero-density rows at this wall strength
        fresh = live & ~(rho > 0.0)              # rows that are live only at this wall strength: the ideal gas
        rho[fresh] = np.exp(float(mu0) - np.asarray(p.vext, np.float64).reshape(-1)[fresh])
        x, mu, y, it, rn, jy, ok = _tp_solver(s, p, x, float(mu0), y0, tol, max_iter, perturb,
                                              1e-6 if mixed else 1e-12, log)
        return dict(betamu=mu, N=float(adsorption(p, x)[0]), resid=rn, jy_rel=jy, iters=it, converged=ok, x=x, y=y)
    finally:
        s.close()


def _off_fold(x, y, offset):
    """x + s y with |s y| = offset |x|, on the side that keeps every positive entry of x above half its value
    (the other side, or a smaller offset, when one does not)."""
    scale = offset * float(np.linalg.norm(x)) / max(float(np.linalg.norm(y)), 1e-300)
    pos = x > 0
    for s in (scale, -scale, 0.25 * scale, -0.25 * scale):
        xs = x + s * y
        if np.all(xs[pos] >= 0.5 * x[pos]):
            return xs
    return x


def turning_point_continuation(spec, x0, mu0, eps_values, tol=1e-9, max_iter=25, first_step=0.002, max_step=0.01,
                               step_ctrl=0.5, min_step=1e-5, restart_offset=0.01, log=None):
    """Zero-order continuation of a turning point in the wall strength eps_w (LOCA's
    TURNING_POINT_CONTINUATION: each step re-solves the turning-point system from the previous fold's
    state, beta mu and null vector, src/loca_lib.c:582-640) with con_lib's step control
    (src/loca_lib.c:440-512): a converged step of `its` Newton iterations multiplies the step by
    1 + step_ctrl ((max_iter - its) / (max_iter - 1))^2 (simple_step_control, src/loca_lib.c:1007-1033) up to
    max_step, a failed one halves it and retries from the last converged fold, down to min_step.  The
    steps start from eps_values[0] (solved from x0, mu0) and land on every requested value; one record per
    requested eps_w, "substeps" counting the turning-point solves that reached it.  Small steps matter: the
    Moore-Spence iteration converges only near its fold, and a step that is too long may converge on
    another fold of the same branch.  Each step restarts a distance restart_offset ||x|| along the null vector
    from the last fold, where the branch passes (x_f + s y at beta mu_f + O(s^2)): at the fold itself J is
    singular to rounding, a = J^-1 R and b = J^-1 dR/dmu carry null components of order |R| / sigma_min that
    the update -a - dmu b must cancel to that relative precision, which the finite-difference second
    derivatives cannot give, whereas off the fold J is nonsingular by O(s) (as at an arclength point next to
    the fold).  log(eps_w, record), when given, sees every turning-point solve."""
    out = []
    x, mu, y = np.array(x0, np.float64), float(mu0), None
    e_cur, step = None, float(first_step)
    for e in eps_values:
        e = float(e)
        n_sub, rec = 0, None
        while True:
            if e_cur is None:
                target = e
            else:
                target = e if abs(e - e_cur) <= step else e_cur + np.copysign(step, e - e_cur)
            rec = turning_point(dict(spec, eps_w=target), _off_fold(x, y, restart_offset) if e_cur is not None else x,
                                mu, y, tol=tol, max_iter=max_iter)
            n_sub += 1
            if log is not None:
                log(target, rec)
            if rec["converged"]:
                x, mu, y = rec["x"], rec["betamu"], rec["y"]
                if e_cur is not None:
                    f = (max_iter - rec["iters"]) / (max_iter - 1.0)
                    step = min(step * (1.0 + step_ctrl * f * f), max_step)
                e_cur = target
                if target == e:
                    break
                continue
            step *= 0.5
            if e_cur is None or step < min_step:
                break
        rec["eps_w"] = e
        rec["substeps"] = n_sub
        out.append(rec)
        if not rec["converged"]:
            break
    return out


def grand_free_energy(s, p, x, mu):
    """Omega_s of state x at beta mu on a live solver (the objectives' chemical potential set to mu; the bulk
    reference term at rho_b is the same for every state at that mu)."""
    s.set_chemical_potential([mu])
    s.set_integration(p.w_fluid, p.w_bulk, p.rhobar_b, [mu])
    return float(s.objectives(x)[0])


def phase_transition(spec, x1, x2, mu0, tol=1e-9, max_iter=30, perturb=1e-6, log=None):
    """Two states of one slit-pore problem at one beta mu with equal grand free energy (a first-order transition,
    e.g. capillary condensation), by the reference's phase-transition algorithm (phase_transition_alg,
    src/loca_bord.c:1073-1190): Newton on R(x1, mu) = 0, R(x2, mu) = 0, g = Omega(x1, mu) - Omega(x2, mu) = 0,
    bordered per state (J_i a_i = R_i, J_i b_i = dR/dmu, so dx_i = -a_i - dmu b_i) with g's derivatives by finite
    differences as the reference takes them (dg/dmu at fixed states; the directional derivatives along (a1, a2) and
    (b1, b2) with the step perturb sqrt(|x1|^2 / (|v1|^2 + perturb) + |x2|^2 / (|v2|^2 + perturb))):
        dmu = (g - D_a) / (D_b - dg/dmu).
    The density-positivity fraction of update_solution, the smaller of the two, scales the whole update.  Starts
    from two states near the transition (e.g. points of the two stable branches of an arclength continuation) and
    mu0.  Returns beta mu, both states with their adsorption N, ||R||_2 (the larger), g, iterations, converged."""
    p = setup.slit_pore(spec)
    if p.ncomp != 1:
        raise ValueError("one component")
    s = native.Solver(p)
    try:
        set_mode(s, False)
        return _pt_solver(s, p, x1, x2, mu0, tol, max_iter, perturb, log)
    finally:
        s.close()


def _pt_solver(s, p, x1, x2, mu0, tol=1e-9, max_iter=30, perturb=1e-6, log=None):
    """phase_transition's iterations on a live solver (any object with the Solver methods it calls)."""
    r0 = p.first_rho
    live = _live_rows(p)[0]
    R_mu = np.zeros(s.shape)
    R_mu[r0][live] = -1.0
    x1, x2, mu = np.array(x1, np.float64), np.array(x2, np.float64), float(mu0)

    def lin(rhs):
        return s.solve(rhs, tol=1e-12, max_iter=2000)[0]

    def g(y1, y2, m):
        return grand_free_energy(s, p, y1, m) - grand_free_energy(s, p, y2, m)

    def dirder(g0, v1, v2):
        """(g(x1 + h v1, x2 + h v2) - g) / h; the backward difference, then smaller steps, where a step leaves
        the functional's domain."""
        h = perturb * np.sqrt(np.sum(x1 * x1) / (np.sum(v1 * v1) + perturb)
                              + np.sum(x2 * x2) / (np.sum(v2 * v2) + perturb))
        for hh in (h, -h, h / 16, -h / 16):
            try:
                return (g(x1 + hh * v1, x2 + hh * v2, mu) - g0) / hh
            except native.TgpuError as err:
                if err.status != native.TGPU_ERR_DOMAIN:
                    raise
        raise native.TgpuError(native.TGPU_ERR_DOMAIN, "no finite-difference step inside the domain")

    def frac(x, dx):
        rho, drho = x[r0], dx[r0]
        neg = live & (drho < -0.9 * rho)
        return min(1.0, float(np.min(-0.9 * rho[neg] / drho[neg]))) if neg.any() else 1.0

    rn, gv, dmu = float("inf"), float("inf"), float("inf")
    for it in range(max_iter + 1):
        s.set_chemical_potential([mu])
        R1 = s.fill(x1, mode=0)
        a1, b1 = lin(R1), lin(R_mu)
        R2 = s.fill(x2, mode=0)
        a2, b2 = lin(R2), lin(R_mu)
        rn = max(float(np.linalg.norm(R1)), float(np.linalg.norm(R2)))
        gv = g(x1, x2, mu)
        if log is not None:
            log(it, mu, rn, gv)
        if it > 0 and rn <= tol and abs(dmu) <= 1e-10 * (1.0 + abs(mu)):
            return dict(betamu=mu, x1=x1, x2=x2, N1=float(adsorption(p, x1)[0]), N2=float(adsorption(p, x2)[0]),
                        resid=rn, g=gv, iters=it, converged=True)
        if it == max_iter:
            break
        hm = perturb * (abs(mu) + perturb)
        g_mu = (g(x1, x2, mu + hm) - gv) / hm
        Da, Db = dirder(gv, a1, a2), dirder(gv, b1, b2)
        den = Db - g_mu
        if den == 0.0 or not np.isfinite(den):
            break
        dmu = (gv - Da) / den
        dx1, dx2 = -a1 - dmu * b1, -a2 - dmu * b2
        f = min(frac(x1, dx1), frac(x2, dx2))
        x1, x2, mu = x1 + f * dx1, x2 + f * dx2, mu + f * dmu
    return dict(betamu=mu, x1=x1, x2=x2, N1=float(adsorption(p, x1)[0]), N2=float(adsorption(p, x2)[0]),
                resid=rn, g=gv, iters=max_iter, converged=False)
