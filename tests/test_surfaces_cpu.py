"""Surfaces and their external fields on the CPU: the oracle's restatement (oracle/surfaces.c) against
the reference's own set-up of its example decks (tests/golden/surf_*.npz, made by
tests/golden/make_surface_golden.py: integrated LJ walls of the GEOM decks, distance-based 9-3 walls in
1-D, 2-D and 3-D), and the deck reader of tramonto_gb300.surfaces.

Bars: wall elements and zero-density flags identical; V_ext/kT within 1e-10 of the reference's
(powers by pow() as the reference, Gauss nodes computed rather than tabulated: differences of a few
1e-12 over sums of thousands of element integrals)."""
import glob
import os
import sys
import time

import numpy as np
import pytest

from tramonto_gb300 import surfaces

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
FIXTURES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "golden", "surf_*.npz")))
# the fixtures the oracle restates in a few seconds (its loops are the reference's, one thread)
ORACLE_FIXTURES = ["surf_cylpore2d", "surf_block2d", "surf_cyl2d", "surf_plane2d_periodic", "surf_sphere3d",
                   "surf_lj93_plane2d_cosx", "surf_lj93_plane2d_cosy", "surf_lj93_1d", "surf_lj93_mix1d",
                   "surf_lj93_cont1d", "surf_lj93_2d_three", "surf_lj93_3d_three", "surf_rough_plane2d",
                   "surf_rough_plane3d", "surf_rough_cylpore2d", "surf_cut_notch2d", "surf_cut_cylpore2d"]
V_TOL = 1e-10


def load(name):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    return z, surfaces.spec_from_arrays(z)


def last_wall(mask):
    """the highest wall owning each element (the reference's Wall_elems keeps the last one), -1 for fluid"""
    m = mask.astype(np.int64)
    out = np.full(m.shape, -1)
    for w in range(16):
        out[(m >> w) & 1 == 1] = w
    return out


def test_fixtures_present():
    assert len(FIXTURES) >= 10, FIXTURES


@pytest.mark.parametrize("name", FIXTURES)
def test_deck_reader_carries_the_reference_parameters(name):
    """the spec read from the deck (stored in the fixture) holds the wall-fluid parameters and wall
    positions the reference used (mixing rules, per-type arrays, positions)"""
    z, spec = load(name)
    nc, nt = spec.ncomp, spec.ntypes
    for key in ("sigma_wf", "eps_wf", "cut_wf"):
        mine = np.array([[getattr(spec.type[t], key)[c] for t in range(nt)] for c in range(nc)])
        assert np.array_equal(mine, z["ref_" + key]), key
    assert np.array_equal(np.array([spec.wall_pos[w][:] for w in range(spec.nwalls)]), z["ref_wall_pos"])


@pytest.mark.parametrize("name", ORACLE_FIXTURES)
def test_oracle_matches_reference(name):
    import orc
    z, spec = load(name)
    t = time.time()
    v, zero, wall_el = orc.surface_field(spec)
    secs = time.time() - t
    assert np.array_equal(last_wall(wall_el), z["ref_wall_elems"])
    assert np.array_equal(zero, z["ref_zero"][:, :v.shape[1]])
    err = np.abs(v - z["ref_vext"]).max()
    print(f"{name}: oracle {secs:.2f} s (reference {float(z['ref_seconds']):.2f} s), max |dV| {err:.2e}")
    assert err <= V_TOL


def test_spec_round_trip():
    spec = surfaces.make_spec(3, (6.0, 5.0, 4.0), (0.25, 0.25, 0.25), [(-1, 0), (1, 1), (2, 2)], 2,
                              [(0, (0.0, 0.5, 0.0)), (1, (1.0, 0.0, -1.0))],
                              [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=0, param=(1.0, 2.0, 0.0),
                                    ipot_wf=5, sigma_wf=[1, 1], eps_wf=[1, 2], cut_wf=[3, 3],
                                    linear=[(0, 0.5, 1.0, 3.0)]),
                               dict(surf_type=surfaces.SURF_COLLOID, param=(0.5, 0, 0), ipot_wf=1,
                                    periodic=[(1, 0.2, 2.0, 0.0)])],
                              vext_max=12.0, apply_offset=(1, 0, 0))
    assert bytes(surfaces.spec_from_arrays(surfaces.spec_arrays(spec))) == bytes(spec)


DECK = """\
@ -1. -1. -1. -1. 12. \tLength_ref Density_ref Temp Dielec_ref VEXT_MAX
@ 2 \tNdim
@ 8.0 6.0 \tSize_x(idim): idim=0,Ndim-1
@ 0.2 0.25 \tEsize_x(idim): idim=0,Ndim-1
@ 2 -1 \tType_bc(x0,: left, right)
@ 1 1 \tType_bc(x1,: down, up)
@ 0 0 \tType_bc(x2,: back, front)
@ 2 3 2 1 0 \tNwall_types Nwall Nlink Lauto_center Lauto_size
@ 0 0 \tXtest_reflect_TF[ilink=0,Nlink-1][idim=0,Ndim-1]
@ 0 2 \tSurf_type[iwall_type] ; iwall_type=0,Nwall_type-1
@ 0 0 \tOrientation[iwall_type]: iwall_type=0,Nwall_type-1
@ 1.5 0.75 \tWallParam[iwall_type]
@ 0. 0. \tWallParam2[iwall_type]
@ 0. 0. \tWallParam3[iwall_type]
@ 1 0 0 \tLapply_offest[3] (applies offsets)
@ 0 0 \tLrough_surf[iwall_type]
@ 0. 0. \trough_param_max[iwall_type]
@ 0. 0. \tRough_length[iwall_type]
@ 1 0 \tNperiodic_overlay_fncs[iwall_type]
@ 1 \tOrientationPeriodicFnc[iwall_type][Nperiodic_overlay_fncs]
@ 0.3 \tAmplitude[iwall_type][Nperiodic_overlay_fncs]
@ 3.0 \tPeriod[iwall_type][Nperiodic_overlay_fncs]
@ 0.5 \tOrigin[iwall_type][Nperiodic_overlay_fncs]
@ 2 0 \tNlinear_overlay_fncs[iwall_type]
@ 1 \tOrientationLinearFnc[iwall_type][Nperiodic_overlay_fncs]
@ 0.1 -0.1 \tSlope[iwall_type][Nperiodic_overlay_fncs]
@ 0. 0. \tOrigin_linear[iwall_type][Nperiodic_overlay_fncs]
@ 2. -2. \tEndpoint_linear[iwall_type][Nperiodic_overlay_fncs]
@ 0 0 \tLangleCutout_surf[iwall_type]
@ 0. 0. \tAngle_start[iwall_type]
@ 0. 0. \tAngle_end[iwall_type]
@ 5 1 \tType of neutral surface-fluid interactions (param. Ipot_wf_n[iwall_type])
@ 0 \tLhard_surf (Logical)
@ 1 0 \tType_vext[iwall_type] (0=VEXT_DEFINED; 1=VEXT_PAIR_POTENTIAL)
@ 0 0 \tVext_PotentialID[iwall_type]: if Type_vext=0 select from list here.
@ 0 \tType of wall-wall interactions::Ipot_ww_n[iwall_type][jwall_type]
@ 0 \tType_uwwPot
@ 2 0 \tNcomp Mix_type (0=L-B Rules, 1=manual input)
@ 1. \tHS_diam[i] i=0,Ncomp-1
@ 1. 1. \tMass[i] i=0,Ncomp-1
@ 0. 0. \tCharge[i] i=0,Ncomp-1
@ 0. 0. \tPol[i] i=0,Ncomp-1
@ 1. 0.8 \tSigma_ff[i][j]
@ 1. 0.5 \tEps_ff[i][j]
@ 3. 2.5 \tCut_ff[i][j]
@ 1. 1. \tBond_ff[i][j]
@ 0. \tEpsYukawa_ff[i][j]
@ 0. \tYukawaK_ff[i][j]
@ 0. \tNpow_ff[i][j]
@ 1. 1. \tRho_w[i]
@ 1.2 0.6 \tSigma_ww[i][j]
@ 4. 2. \tEps_ww[i][j]
@ 3. 2. \tCut_ww[i][j]
"""


def test_read_deck_of_own_text(tmp_path):
    """label-keyed reading, Lorentz-Berthelot wall-fluid parameters, a short overlay line (the missing
    orientation reads as 0), wall positions from dft_surfaces.dat and Lauto_center"""
    (tmp_path / "dft_input.dat").write_text(DECK)
    (tmp_path / "dft_surfaces.dat").write_text(" 0 0 -2.0 1.0 0.\n 1 0 1.0 -1.0 0.\n 1 1 3.0 0.0 0.\n")
    s = surfaces.read_deck(str(tmp_path / "dft_input.dat"))
    assert s.ndim == 2 and s.ncomp == 2 and s.ntypes == 2 and s.nwalls == 3 and s.vext_max == 12.0
    assert list(s.size[:2]) == [8.0, 6.0] and list(s.esize[:2]) == [0.2, 0.25]
    assert [tuple(s.bc[d]) for d in range(2)] == [(2, -1), (1, 1)] and list(s.apply_offset) == [1, 0, 0]
    t0, t1 = s.type[0], s.type[1]
    assert (t0.surf_type, t1.surf_type, t0.ipot_wf, t1.ipot_wf) == (0, 2, 5, 1)
    assert t0.nperiodic == 1 and t0.periodic_orient[0] == 1 and t0.amplitude[0] == 0.3 and t0.wavelength[0] == 3.0
    assert t0.nlinear == 2 and list(t0.linear_orient[:2]) == [1, 0] and list(t0.slope[:2]) == [0.1, -0.1]
    assert t1.nperiodic == 0 and t1.nlinear == 0 and t1.param[0] == 0.75
    assert list(t0.sigma_wf[:2]) == [0.5 * (1.0 + 1.2), 0.5 * (0.8 + 1.2)]
    assert list(t1.eps_wf[:2]) == [np.sqrt(1.0 * 2.0), np.sqrt(0.5 * 2.0)]
    assert list(t1.cut_wf[:2]) == [0.5 * (3.0 + 2.0), 0.5 * (2.5 + 2.0)]
    # Lauto_center: positions shifted by the centre of their bounding box (x: -2..3, y: -1..1)
    assert [list(s.wall_pos[w][:2]) for w in range(3)] == [[-2.5, 1.0], [0.5, -1.0], [2.5, 0.0]]
    assert list(s.wall_type[:3]) == [0, 1, 1]


def test_read_deck_refuses_what_is_not_built(tmp_path):
    (tmp_path / "dft_input.dat").write_text(DECK.replace("@ 0 \tLhard_surf", "@ 1 \tLhard_surf"))
    (tmp_path / "dft_surfaces.dat").write_text(" 0 0 -2.0 1.0 0.\n 1 0 1.0 -1.0 0.\n 1 1 3.0 0.0 0.\n")
    with pytest.raises(NotImplementedError):
        surfaces.read_deck(str(tmp_path / "dft_input.dat"))


def test_rough_table_is_the_c_library_rand():
    """the builder's roughness patch heights equal Rough_precalc as the reference fills it: rand() % (2^31 - 1)
    after srand(135649), every wall type in order (here the C library's own rand(), when it is glibc)"""
    import ctypes
    try:
        libc = ctypes.CDLL("libc.so.6")
        libc.gnu_get_libc_version
    except (OSError, AttributeError):
        pytest.skip("not glibc")
    lj = dict(sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0])
    spec = surfaces.make_spec(2, (10.0, 10.0), (0.25, 0.25), [(-1, -1), (1, 1)], 1, [(0, (0.0, 0.0)), (1, (3.0, 0.0))],
                              [dict(surf_type=surfaces.SURF_PLANAR, param=(1.0, 0, 0), rough=1, rough_max=0.5,
                                    rough_length=0.5, **lj),
                               dict(surf_type=surfaces.SURF_COLLOID, param=(1.0, 0, 0), rough=1, rough_max=0.3,
                                    rough_length=0.4, **lj)])
    tab = surfaces.rough_table(spec)
    libc.srand(135649)
    r = np.array([libc.rand() % 2147483647 for _ in range(20000)], np.float64).reshape(2, 100, 100)
    assert np.array_equal(tab[0], 0.5 * (-0.5 + r[0] / 2147483647.0))
    assert np.array_equal(tab[1], 0.3 * (-0.5 + r[1] / 2147483647.0))
