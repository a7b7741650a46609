"""The GPU stencil builder (tgpu_make_stencil_device) against the host builder and the reference.

Both builders run the same per-element quadrature in the same IEEE operations (stencils.cu is
compiled without multiply-add contraction), merge corner weights in element order and renormalise
with a sequential sum in table order, so their tables must be bit-identical: offsets, weights
and per-corner weights, in the same order.  Cases: the delta shell, theta ball and WCA
attraction in 1, 2 and 3 dimensions, including the 3-D attraction stencils of the 128^3 (dx 0.1)
and 256^3 (dx 0.08) workloads, and the reference's own tables of the golden cases (1e-14).
"""
import time

import numpy as np
import pytest

from goldens import load

pytestmark = pytest.mark.gpu

D, T, U = 0, 1, 2


def _both(stype, ndim, esize, **kw):
    from tramonto_gb300 import setup
    t0 = time.perf_counter()
    h = setup.make_stencil(stype, ndim, esize, with_hw=True, device=False, **kw)
    t1 = time.perf_counter()
    d = setup.make_stencil(stype, ndim, esize, with_hw=True, device=True, **kw)
    t2 = time.perf_counter()
    return h, d, t1 - t0, t2 - t1


def _uatt(rcut=2.5, h=0.1):
    from tramonto_gb300 import setup
    eps = 1.0 / 1.2
    return dict(sigma=1.0, eps=eps, rcut=rcut, rmin=setup.lj_rmin(1.0, eps, rcut, h))


SPECS = [
    (D, 1, [0.01], dict(hs_diam=1.0)), (T, 1, [0.01], dict(hs_diam=1.0)), (U, 1, [0.05], _uatt(h=0.05)),
    (D, 2, [0.05, 0.05], dict(hs_diam=1.0)), (T, 2, [0.05, 0.05], dict(hs_diam=1.0)),
    (U, 2, [0.05, 0.05], _uatt(h=0.05)),
    (D, 3, [0.1, 0.1, 0.1], dict(hs_diam=1.0)), (T, 3, [0.1, 0.1, 0.1], dict(hs_diam=1.0)),
    (D, 3, [0.25, 0.2, 0.3], dict(hs_diam=0.6)), (T, 3, [0.25, 0.2, 0.3], dict(hs_diam=0.6)),
    (U, 3, [0.1, 0.1, 0.1], _uatt(h=0.1)),
    (D, 3, [0.08, 0.08, 0.08], dict(hs_diam=1.0)), (U, 3, [0.08, 0.08, 0.08], _uatt(h=0.08)),
]


@pytest.mark.parametrize("spec", SPECS, ids=lambda s: f"type{s[0]}-{s[1]}d-h{s[2][0]}")
def test_device_builder_is_bit_identical_to_host(spec):
    stype, ndim, esize, kw = spec
    (oh, wh, hh), (od, wd, hd), th, td = _both(stype, ndim, esize, **kw)
    print(f"type {stype} {ndim}-D h={esize[0]}: L={len(wh)} host {th * 1e3:.1f} ms, device {td * 1e3:.1f} ms")
    assert np.array_equal(oh, od)
    assert np.array_equal(wh.view(np.uint64), wd.view(np.uint64))
    assert np.array_equal(hh.view(np.uint64), hd.view(np.uint64))


@pytest.mark.parametrize("case", ["fmt1_wca_3d", "mix1d_fmt3", "rough3d_fmt4", "hs1d_wall"])
def test_device_builder_matches_reference_tables(case):
    from tramonto_gb300 import setup
    z, p = load(case)
    d = z["info_doubles"]
    nc = p.ncomp
    sig, eps, cut = (d[a:a + 36].reshape(6, 6) for a in (147, 111, 183))
    for (t, idx), (off, w, hw) in p.stencils.items():
        if t < 2:
            o2, w2, h2 = setup.make_stencil(t, p.ndim, p.esize, hs_diam=p.hs_diam[idx], with_hw=hw is not None,
                                            device=True)
        else:
            i, j = idx % nc, idx // nc
            rmin = setup.lj_rmin(sig[i, j], eps[i, j], cut[i, j], p.esize[0])
            o2, w2, h2 = setup.make_stencil(t, p.ndim, p.esize, sigma=sig[i, j], eps=eps[i, j], rcut=cut[i, j],
                                            rmin=rmin, device=True)
        assert np.array_equal(o2, off), (case, t, idx)
        assert np.abs(w2 - w).max() <= 1e-14 * np.abs(w).max(), (case, t, idx)
        if hw is not None:
            assert np.abs(h2 - hw).max() <= 1e-14 * np.abs(hw).max(), (case, t, idx)


POTS = [("lj_sigma_zero", dict(pot=0, core_r=0, core_const=1)), ("lj_jdc", dict(pot=0, core_r=3, core_const=0)),
        ("yukawa", dict(pot=3, core_r=1, core_const=0, kappa=1.8)), ("exp", dict(pot=4, core_r=1, core_const=0, kappa=0.5)),
        ("square_well", dict(pot=5, core_r=1, core_const=0))]


@pytest.mark.parametrize("name,pp", POTS, ids=[n for n, _ in POTS])
@pytest.mark.parametrize("ndim,h", [(1, 0.05), (3, 0.1)])
def test_attraction_stencils_of_other_pair_potentials(name, pp, ndim, h):
    """Host and GPU builders of the other mean-field kernels: bit-identical for the LJ cores and the square
    well (pure arithmetic), within 1e-14 for Yukawa and exponential (exp() of two libraries)."""
    from tramonto_gb300 import setup
    rcut = 1.5 if name == "square_well" else 2.5
    rmin = setup.lj_rmin(1.0, 1.0 / 1.2, rcut, h)
    kw = dict(pp, sigma=1.0, eps=1.0 / 1.2, rcut=rcut, rmin=rmin)
    oh, wh, hh = setup.make_attraction_stencil(ndim, [h] * ndim, with_hw=True, device=False, **kw)
    od, wd, hd = setup.make_attraction_stencil(ndim, [h] * ndim, with_hw=True, device=True, **kw)
    assert np.array_equal(oh, od)
    if pp["pot"] in (3, 4):
        assert np.abs(wh - wd).max() <= 1e-14 * np.abs(wh).max()
        assert np.abs(hh - hd).max() <= 1e-14 * np.abs(hh).max()
    else:
        assert np.array_equal(wh.view(np.uint64), wd.view(np.uint64))
        assert np.array_equal(hh.view(np.uint64), hd.view(np.uint64))


@pytest.mark.parametrize("name", ["sten3d_dx010", "sten3d_dx008"])
def test_device_builder_matches_reference_tables_of_the_3d_workloads(name):
    """The GPU builder's tables of the 128^3 (dx 0.1) and 256^3 (dx 0.08) workloads against the reference's
    calc_stencils at the same element sizes (tests/golden/make_stencil_golden.py)."""
    from test_stencils_3d_cpu import CASES, compare, workload_tables
    compare(name, workload_tables(CASES[name][0], device=True))
