"""The objectives of a state on the GPU: the surface excess grand free energy
Omega_s (the reference's calc_free_energy) and the excess adsorption Gamma_ex
(calc_adsorption), against the values the reference itself computed for the
fixture states, and their partial derivatives (tgpu_objective_grad_device)
against central differences of the objectives.

Tolerances: Omega_s within 1e-11 of max(1, |Omega_s|) and Gamma_ex within
1e-12 relative (the sums run in a different order than the reference's);
partial derivatives within 1e-6 of the directional derivative's scale.
"""
import numpy as np
import pytest

from goldens import CASES, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", CASES)
def test_objectives_match_reference(name):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    for k in range(len(z["states"])):
        om, gam = s.objectives(z[f"x{k}"])
        ref_om = float(z[f"omega_s{k}"])
        ref_gam = np.asarray(z[f"ads{k}"]) - np.asarray(z[f"ads_b{k}"])
        assert abs(om - ref_om) <= 1e-11 * max(1.0, abs(ref_om)), (name, k, om, ref_om)
        assert np.abs(gam - ref_gam).max() <= 1e-12 * np.abs(np.asarray(z[f"ads{k}"])).max(), (name, k, gam, ref_gam)
    s.close()


@pytest.mark.parametrize("name", ["lj1d_mf", "mix1d_fmt3", "fmt1_wca_3d", "hs1d_wall", "hslj1d_wall", "lj1d_a22"])
def test_objective_partials_match_finite_differences(name):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    x = np.array(z["x0"])
    zero = np.asarray(p.zero_density, bool)
    rng = np.random.default_rng(11)
    dx = rng.standard_normal(x.shape) * 1e-2
    dx[p.first_rho:p.first_rho + p.ncomp][zero] = 0.0            # densities fixed at zero there
    dx[p.first_rho:p.first_rho + p.ncomp] *= x[p.first_rho:p.first_rho + p.ncomp]   # keep rho > 0
    dv = rng.standard_normal((p.ncomp, p.nnodes)) * 1e-2
    v0 = np.array(p.vext)
    h = 1e-4
    for kind, icomp in [(0, 0)] + [(1, c) for c in range(p.ncomp)]:
        gx, gv = s.objective_grad(x, kind, icomp)

        def F(xx, vv):
            s.set_vext(vv)
            om, gam = s.objectives(xx)
            return om if kind == 0 else gam[icomp]

        fd_x = (F(x + h * dx, v0) - F(x - h * dx, v0)) / (2 * h)
        an_x = float(np.sum(gx * dx))
        assert abs(fd_x - an_x) <= 1e-6 * max(abs(an_x), float(np.abs(gx * dx).sum())), (name, kind, fd_x, an_x)
        fd_v = (F(x, v0 + h * dv) - F(x, v0 - h * dv)) / (2 * h)
        an_v = float(np.sum(gv * dv))
        assert abs(fd_v - an_v) <= 1e-6 * max(abs(an_v), float(np.abs(gv * dv).sum()), 1e-12), (name, kind, fd_v, an_v)
        s.set_vext(v0)
    s.close()


def test_objective_partials_with_reflecting_boundaries_match_finite_differences():
    """dOmega_s/dx with attraction and a reflecting boundary (the mean-field term's transposed sums fold the
    mirrored positions back), on a 3-D problem reflecting in y, against central differences."""
    from tramonto_gb300 import native, setup
    from test_gpu_adjoint import _reflecting_3d_problem
    p = _reflecting_3d_problem()
    s = native.Solver(p)
    x = setup.initial_state(s, p, max_enhancement=1.0)
    zero = np.asarray(p.zero_density, bool) | (np.asarray(p.vext) >= p.vext_max)
    rng = np.random.default_rng(12)
    dx = rng.standard_normal(x.shape) * 1e-2
    dx[p.first_rho:p.first_rho + p.ncomp][zero] = 0.0
    dx[p.first_rho:p.first_rho + p.ncomp] *= x[p.first_rho:p.first_rho + p.ncomp]
    h = 1e-4
    gx, _ = s.objective_grad(x, 0, 0)
    fd = (s.objectives(x + h * dx)[0] - s.objectives(x - h * dx)[0]) / (2 * h)
    an = float(np.sum(gx * dx))
    assert abs(fd - an) <= 1e-6 * max(abs(an), float(np.abs(gx * dx).sum())), (fd, an)
    s.close()
