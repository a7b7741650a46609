"""Host set-up against the reference: generated stencil tables and bulk constants."""
import numpy as np
import pytest

from goldens import load
from tramonto_gb300 import setup

CASES = ["hs1d_wall", "hs1d_reflect", "lj1d_mf", "mix1d_fmt3", "fmt1_wca_3d", "hs1d_c1", "mix1d_fmt4", "rough3d_fmt2",
         "lj1d_sigzero", "lj1d_jdc", "yuk1d_mf", "exp1d_mf", "sw1d_mf", "hslj1d_wall"]


@pytest.mark.parametrize("case", CASES)
def test_stencils_match_reference(case):
    z, p = load(case)
    d = z["info_doubles"]
    nc = p.ncomp
    sig, eps, cut = (d[a:a + 36].reshape(6, 6) for a in (147, 111, 183))
    for (t, idx), (off, w, hw) in p.stencils.items():
        if t < 2:
            o2, w2, h2 = setup.make_stencil(t, p.ndim, p.esize, hs_diam=p.hs_diam[idx], with_hw=hw is not None)
        else:
            i, j = idx % nc, idx // nc
            rmin = setup.lj_rmin(sig[i, j], eps[i, j], cut[i, j], p.esize[0])
            ints = z["info_ints"]
            if len(ints) > 43:    # fixtures that carry the pair potential and its core
                pot, core_r, core_c = int(ints[40]), int(ints[42]), int(ints[43])
                kappa, rzero = d[221:257].reshape(6, 6)[i, j], d[293:329].reshape(6, 6)[i, j]
                o2, w2, h2 = setup.make_attraction_stencil(p.ndim, p.esize, pot, core_r, core_c, sigma=sig[i, j],
                                                           eps=eps[i, j], rcut=cut[i, j], rmin=rmin, rzero=rzero,
                                                           kappa=kappa, with_hw=hw is not None)
            else:
                o2, w2, h2 = setup.make_stencil(t, p.ndim, p.esize, sigma=sig[i, j], eps=eps[i, j], rcut=cut[i, j],
                                                rmin=rmin, with_hw=hw is not None)
        assert np.array_equal(o2, off), (case, t, idx)
        assert np.abs(w2 - w).max() <= 1e-14 * np.abs(w).max(), (case, t, idx)
        if hw is not None:
            assert np.abs(h2 - hw).max() <= 1e-14 * np.abs(hw).max(), (case, t, idx)


@pytest.mark.parametrize("case", CASES)
def test_bulk_constants_match_reference(case):
    z, p = load(case)
    d = z["info_doubles"]
    nc = p.ncomp
    uat = {k[1]: v for k, v in p.stencils.items() if k[0] == 2}
    b = setup.bulk_constants(p.functional, d[7:7 + nc], d[13:13 + nc], p.attraction, uat, nc)
    assert np.allclose(b["rhobar_b"], d[55:59], rtol=1e-14, atol=0)
    assert np.allclose(b["dphi_bulk"], d[65:69], rtol=1e-14, atol=1e-15)
    assert np.allclose(b["betamu_hs_ex"], d[19:19 + nc], rtol=1e-13)
    if p.attraction:
        assert np.allclose(b["betamu_att"], d[25:25 + nc], rtol=1e-13)


def test_config_generators_are_seeded():
    v1, m1 = setup.rough_wall_vext((48, 16, 16), (0.1, 0.1, 0.1), seed=5)
    v2, m2 = setup.rough_wall_vext((48, 16, 16), (0.1, 0.1, 0.1), seed=5)
    assert np.array_equal(v1, v2) and m1 == m2
    assert v1.max() == 10.0 and v1.min() < 0.0


def test_lj93_wall_matches_reference_field():
    """The lj1d_mf deck's field is the cut-and-shifted 9-3 wall with eps_wf*rho_w = 3, sigma_wf = 1,
    cut 3, surface at x = 0.5; nodes the reference flags zero-density hold VEXT_MAX."""
    z, p = load("lj1d_mf")
    d = np.arange(p.nnodes) * p.esize[0] - 0.5
    v, de, ds = setup.lj93_wall_1d(d, 3.0, 1.0, 3.0, p.vext_max)
    zero = np.asarray(p.zero_density, bool).reshape(-1)
    ref = np.asarray(p.vext).reshape(-1)
    assert np.abs(np.where(zero, p.vext_max, v) - ref).max() <= 1e-8
    # analytic parameter derivatives against central differences of the formula itself
    live = ~zero & (d < 3.0)
    h = 1e-6
    fd_e = (setup.lj93_wall_1d(d, 3.0 + h, 1.0, 3.0, 1e300)[0] - setup.lj93_wall_1d(d, 3.0 - h, 1.0, 3.0, 1e300)[0]) / (2 * h)
    fd_s = (setup.lj93_wall_1d(d, 3.0, 1.0 + h, 3.0, 1e300)[0] - setup.lj93_wall_1d(d, 3.0, 1.0 - h, 3.0, 1e300)[0]) / (2 * h)
    assert np.abs(de[live] - fd_e[live]).max() <= 1e-6 * np.abs(de[live]).max()
    assert np.abs(ds[live] - fd_s[live]).max() <= 1e-6 * np.abs(ds[live]).max()


def test_config5_problems_are_seeded_and_in_range():
    a, b = setup.config5(), setup.config5()
    assert a == b and len(a) == 64
    for s in a[:32]:
        assert s["ndim"] == 1 and 300 <= s["nx"][0] <= 4001 and 3.0 <= s["width"] <= 40.0
    for s in a[32:]:
        assert s["ndim"] == 2 and 100 <= s["nx"][0] <= 400 and s["nx"][0] == s["nx"][1]
    assert all(0.05 <= s["rho_b"] <= 0.8 for s in a)


def test_slit_pore_field_is_mirror_symmetric():
    v = setup.slit_pore_vext(1, (501, 1, 1), (0.01,))[0]
    assert np.allclose(v, v[::-1], rtol=1e-10, atol=1e-12) and v[0] == 10.0 and v.min() < -1.0
    v2 = setup.slit_pore_vext(2, (120, 80, 1), (0.05, 0.05)).reshape(80, 120)
    assert np.allclose(v2, v2[:, ::-1]) and not np.allclose(v2[0], v2[40])
