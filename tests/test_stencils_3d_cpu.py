"""The 3-D stencil tables of the 128^3 (dx 0.1) and 256^3 (dx 0.08) workloads against the reference's own
calc_stencils (tests/golden/sten3d_dx0*.npz, made by tests/golden/make_stencil_golden.py).

The host builder is called with exactly the arguments build_problem passes for those workloads (FMT1,
sigma = 1, LJ 12-6 attraction with eps/kT = 1/1.2, cut 2.5, core at r_min): offsets must be identical and
weights within 1e-14 of the largest weight."""
import os

import numpy as np
import pytest

from tramonto_gb300 import setup
from tramonto_gb300.problem import DELTA, THETA, UATT

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
KT, RCUT, SIGMA, HS_DIAM = 1.2, 2.5, 1.0, 1.0
CASES = {"sten3d_dx010": (0.1, (844, 1015, 71831)), "sten3d_dx008": (0.08, (1468, 1911, 137299))}


def workload_tables(esize, device=False):
    es = (esize,) * 3
    eps = 1.0 / KT
    rmin = setup.lj_rmin(SIGMA, eps, RCUT, esize)
    return {DELTA: setup.make_stencil(DELTA, 3, es, hs_diam=HS_DIAM, device=device),
            THETA: setup.make_stencil(THETA, 3, es, hs_diam=HS_DIAM, device=device),
            UATT: setup.make_stencil(UATT, 3, es, sigma=SIGMA, eps=eps, rcut=RCUT, rmin=rmin, device=device)}


def compare(name, tables):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    esize, lens = CASES[name]
    for t, L in zip((DELTA, THETA, UATT), lens):
        off_ref, w_ref = z[f"sten_{t}_0_off"].astype(np.int16), z[f"sten_{t}_0_w"]
        off, w, _ = tables[t]
        assert len(w_ref) == L and len(w) == L, (name, t, len(w), len(w_ref))
        assert np.array_equal(off, off_ref), (name, t)
        assert np.abs(w - w_ref).max() <= 1e-14 * np.abs(w_ref).max(), (name, t, np.abs(w - w_ref).max())


@pytest.mark.parametrize("name", list(CASES))
def test_fixture_records_the_workload_parameters(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    esize, _ = CASES[name]
    assert float(z["esize"]) == esize and float(z["hs_diam"]) == HS_DIAM and float(z["sigma_ff"]) == SIGMA
    assert abs(float(z["eps_ff"]) - 1.0 / KT) <= 1e-15 and float(z["cut_ff"]) == RCUT


@pytest.mark.parametrize("name", list(CASES))
def test_host_builder_matches_reference_tables(name):
    compare(name, workload_tables(CASES[name][0], device=False))


def test_config2_uses_the_pinned_tables():
    """The 128^3 workload's problem is built from these very tables (small grid: the tables do not depend on it)."""
    p, meta = setup.config2(n=56)
    z = np.load(os.path.join(GOLDEN, "sten3d_dx010.npz"))
    for t in (DELTA, THETA, UATT):
        off, w, _ = p.stencils[(t, 0)]
        assert np.array_equal(off, z[f"sten_{t}_0_off"].astype(np.int16))
        assert np.abs(w - z[f"sten_{t}_0_w"]).max() <= 1e-14 * np.abs(z[f"sten_{t}_0_w"]).max()


@pytest.mark.parametrize("name", list(CASES))
def test_bulk_constants_of_the_workload_match_reference(name):
    """Bulk weighted densities, dPhi/dn and excess chemical potentials at rho_b = 0.6 with the pinned tables
    against the reference's own thermo of the same deck."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = z["info_doubles"]
    uat = {0: (None, z[f"sten_{UATT}_0_w"])}
    b = setup.bulk_constants(0, [HS_DIAM], [0.6], True, uat, 1)
    assert np.allclose(b["rhobar_b"], d[55:59], rtol=1e-14, atol=0)
    assert np.allclose(b["dphi_bulk"], d[65:69], rtol=1e-14, atol=1e-15)
    assert np.allclose(b["betamu_hs_ex"], d[19:20], rtol=1e-13)
    assert np.allclose(b["betamu_att"], d[25:26], rtol=1e-13)
