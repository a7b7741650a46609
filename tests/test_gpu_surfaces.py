"""Surfaces and their external fields built on the GPU (tgpu_surface_field_*) against the reference's own
set-up of its example decks (tests/golden/surf_*.npz: integrated LJ walls of cylindrical pores in 2-D and
3-D, a tapered 3-D pore with linear overlays, blocks, cylinders, spheres, periodic-overlay and wedge planes;
distance-based 9-3 walls in 1-D, 2-D and 3-D; reflecting, last-node, in-wall and in-bulk boundaries) and
against the oracle's restatement on specs with periodic images, several walls, every 1-D wall form and the
distances to surfaces and to centres.

Bars: wall elements and zero-density flags identical; V_ext/kT within 1e-10 of the reference's (the
kernel forms powers as products and sums the Gauss points of an element over the lanes of a warp, in
another order than the reference's loops: differences of a few 1e-12)."""
import glob
import os
import sys
import time

import numpy as np
import pytest

from tramonto_gb300 import surfaces
from test_surfaces_cpu import last_wall, load

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
FIXTURES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(HERE, "golden", "surf_*.npz")))
V_TOL = 1e-10


@pytest.mark.parametrize("name", FIXTURES)
def test_gpu_surface_field_matches_reference(name):
    z, spec = load(name)
    surfaces.surface_field(spec)          # first call: context and module load
    t = time.time()
    v, zero, wall_el = surfaces.surface_field(spec)
    secs = time.time() - t
    assert np.array_equal(last_wall(wall_el), z["ref_wall_elems"])
    assert np.array_equal(zero, z["ref_zero"][:, :v.shape[1]])
    err = np.abs(v - z["ref_vext"]).max()
    print(f"{name}: {v.shape[1]} nodes x {v.shape[0]} components, GPU {1e3 * secs:.1f} ms against the reference's "
          f"{float(z['ref_seconds']):.1f} s set-up, max |dV| {err:.2e}")
    assert err <= V_TOL


def _periodic_specs():
    """specs with periodic and reflected images, walls sharing elements, both overlay kinds and hard walls"""
    lj = dict(sigma_wf=[1.0, 0.8], eps_wf=[1.5, 0.7], cut_wf=[2.5, 2.0])
    s2 = surfaces.make_spec(2, (6.0, 5.0), (0.25, 0.25), [(1, 1), (2, -1)], 2,
                            [(0, (2.6, 0.3)), (0, (-2.7, -1.0)), (1, (0.0, -2.5))],
                            [dict(surf_type=surfaces.SURF_COLLOID, param=(0.9, 0, 0), ipot_wf=5, **lj),
                             dict(surf_type=surfaces.SURF_PLANAR, orientation=1, param=(0.5, 0, 0), ipot_wf=5,
                                  periodic=[(0, 0.25, 3.0, 0.0)], linear=[(0, 0.1, -1.0, 1.0)], **lj)])
    s3 = surfaces.make_spec(3, (4.0, 4.0, 3.0), (0.25, 0.25, 0.25), [(1, 1), (1, 1), (-1, 0)], 2,
                            [(0, (1.8, -1.6, -0.5)), (1, (0.0, 0.0, 1.0))],
                            [dict(surf_type=surfaces.SURF_COLLOID, param=(0.8, 0, 0), ipot_wf=5, **lj),
                             dict(surf_type=surfaces.SURF_BLOCK, param=(0.5, 0.5, 0.5), ipot_wf=1, **lj)])
    s3p = surfaces.make_spec(3, (3.0, 3.0, 5.0), (0.25, 0.25, 0.25), [(2, 2), (1, 1), (1, 1)], 1,
                             [(0, (0.0, 0.0, 0.0))],
                             [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=2, param=(1.0, 1.5, 0.0),
                                   ipot_wf=5, sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0],
                                   linear=[(2, 0.2, 0.0, 1.5)])], apply_offset=(1, 0, 0))
    # distance-based walls: every 1-D form and the pair potential, distances to surfaces and to centres
    lj1 = dict(sigma_wf=[1.0, 0.8], eps_wf=[1.2, 0.6], cut_wf=[2.5, 2.2], rho_w=0.9)
    sd2 = surfaces.make_spec(2, (8.0, 6.0), (0.2, 0.25), [(-1, -1), (1, 1)], 2,
                             [(0, (-3.0, 0.0)), (1, (3.0, 0.0)), (2, (0.5, 1.0)), (3, (-0.5, -1.5))],
                             [dict(surf_type=surfaces.SURF_PLANAR, orientation=0, param=(1.0, 0, 0), ipot_wf=2,
                                   pot_id=surfaces.WALL1D_LJ93_CS, periodic=[(1, 0.3, 3.0, 0.0)], **lj1),
                              dict(surf_type=surfaces.SURF_PLANAR, orientation=0, param=(1.0, 0, 0), ipot_wf=2,
                                   pot_id=surfaces.WALL1D_LJ93_SHIFTX_CS, **lj1),
                              dict(surf_type=surfaces.SURF_COLLOID, param=(0.8, 0, 0), ipot_wf=3, type_vext=1, **lj1),
                              dict(surf_type=surfaces.SURF_BLOCK, param=(0.6, 0.4, 0), ipot_wf=2,
                                   pot_id=surfaces.WALL1D_EXP_ATT, **lj1)], sigma_ff=[1.0, 1.3])
    sd3 = surfaces.make_spec(3, (5.0, 4.0, 4.0), (0.25, 0.25, 0.25), [(0, 0), (1, 1), (2, 2)], 1,
                             [(0, (0.0, 0.0, 0.0)), (1, (1.5, 1.0, 1.0)), (2, (-1.5, 0.0, 0.0))],
                             [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=0, param=(1.5, 1.0, 0), ipot_wf=2,
                                   pot_id=surfaces.WALL1D_LJ93_V2_CS, sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0]),
                              dict(surf_type=surfaces.SURF_FINITE_CYL, orientation=2, param=(0.5, 0.75, 0), ipot_wf=3,
                                   pot_id=surfaces.WALL1D_REPULSIVE9, sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0]),
                              dict(surf_type=surfaces.SURF_PORE, param=(2.4, 0, 0), ipot_wf=2,
                                   pot_id=surfaces.WALL1D_LJ93_NOCS, sigma_wf=[1.0], eps_wf=[0.5], cut_wf=[2.5])])
    # an integrated planar wall in 1-D (the 2 pi rho dz out-of-line integral) with a face copy region
    si1 = surfaces.make_spec(1, (8.0,), (0.1,), [(-1, 0)], 2, [(0, (-3.5,))],
                             [dict(surf_type=surfaces.SURF_PLANAR, orientation=0, param=(0.5, 0, 0), ipot_wf=5, **lj)])
    # rough 3-D cylindrical pore (integrated) next to a rough slit pore wall in 2-D (distance-based)
    sr3 = surfaces.make_spec(3, (4.0, 4.0, 5.0), (0.25, 0.25, 0.25), [(-1, -1), (-1, -1), (1, 1)], 1, [(0, (0.0, 0.0, 0.0))],
                             [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=2, param=(1.5, 1.75, 0.0), ipot_wf=5,
                                   rough=1, rough_max=0.4, rough_length=0.5, sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0])])
    sr2 = surfaces.make_spec(2, (6.0, 8.0), (0.2, 0.2), [(-1, -1), (1, 1)], 2, [(0, (0.0, 0.0))],
                             [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=1, param=(1.5, 3.0, 0.0), ipot_wf=2,
                                   rough=1, rough_max=0.5, rough_length=0.3, pot_id=surfaces.WALL1D_LJ93_CS, **lj1)])
    # angle cutouts of a 3-D sphere (no orientation: the wedge about x) and of a spherical cavity, and a 2-D
    # wedge that wraps past 360 degrees
    sc3 = surfaces.make_spec(3, (4.0, 4.0, 4.0), (0.25, 0.25, 0.25), [(2, 2), (2, 2), (2, 2)], 1,
                             [(0, (0.0, 0.0, 0.0)), (1, (0.0, 0.0, 0.0))],
                             [dict(surf_type=surfaces.SURF_COLLOID, param=(1.0, 0, 0), ipot_wf=5, cutout=1,
                                   angle_start=30.0, angle_end=200.0, sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0]),
                              dict(surf_type=surfaces.SURF_PORE, param=(1.8, 0, 0), ipot_wf=5, cutout=1,
                                   angle_start=300.0, angle_end=60.0, sigma_wf=[1.0], eps_wf=[0.5], cut_wf=[2.0])])
    sc2 = surfaces.make_spec(2, (6.0, 6.0), (0.2, 0.2), [(-1, -1), (1, 1)], 2, [(0, (0.0, 0.0))],
                             [dict(surf_type=surfaces.SURF_COLLOID, param=(1.2, 0, 0), ipot_wf=5, cutout=1,
                                   angle_start=250.0, angle_end=80.0, **lj)])
    return {"periodic2d": s2, "periodic3d": s3, "reflect_periodic_pore3d": s3p, "distance_walls2d": sd2,
            "distance_walls3d": sd3, "integrated1d": si1, "rough_pore3d": sr3, "rough_slit2d": sr2,
            "cutout_sphere3d": sc3, "cutout_wrap2d": sc2}


@pytest.mark.parametrize("case", list(_periodic_specs()))
def test_gpu_surface_field_matches_oracle(case):
    import orc
    spec = _periodic_specs()[case]
    v_o, z_o, w_o = orc.surface_field(spec)
    v, zero, wall_el = surfaces.surface_field(spec)
    assert np.array_equal(wall_el, w_o)
    assert np.array_equal(zero, z_o)
    err = np.abs(v - v_o).max()
    print(f"{case}: {int((z_o == 0).sum())} fluid nodes, max |V| below the cap {np.abs(v_o[v_o < spec.vext_max]).max():.3f}, "
          f"max |dV| {err:.2e}")
    assert err <= V_TOL


def test_device_entry_matches_host_entry():
    import ctypes as C

    import torch
    from tramonto_gb300 import native
    z, spec = load("surf_cylpore2d")
    nodes, els = spec.mesh()
    n, ne = int(np.prod(nodes)), int(np.prod(els))
    v_h, z_h, w_h = surfaces.surface_field(spec)
    dv = torch.zeros((spec.ncomp, n), dtype=torch.float64, device="cuda")
    dz = torch.zeros((spec.ncomp, n), dtype=torch.int8, device="cuda")
    dw = torch.zeros(ne, dtype=torch.int16, device="cuda")
    lib = native.load()
    torch.cuda.synchronize()
    native._check(lib.tgpu_surface_field_device(C.byref(spec), dv.data_ptr(), dz.data_ptr(), dw.data_ptr()), lib)
    assert np.array_equal(dv.cpu().numpy(), v_h)
    assert np.array_equal(dz.cpu().numpy(), z_h)
    assert np.array_equal(dw.cpu().numpy().view(np.uint16), w_h)


def test_fields_drive_a_solve():
    """the 2-D cylindrical pore's field and flags from the GPU builder set up a solvable problem: FMT3 hard
    spheres in the pore of GEOM25 at rho_b 0.2 converge, and the density is zero where the builder says"""
    from tramonto_gb300 import native, setup
    z, spec = load("surf_cylpore2d")
    vext, zero = surfaces.problem_fields(spec)
    nodes, _ = spec.mesh()
    p = setup.build_problem(2, nodes[:2], (spec.esize[0], spec.esize[1]), ((-1, -1), (-1, -1)),
                            hs_diam=[1.0], rho_b=[0.2], functional=setup.FMT3, vext=vext[:1], zero_density=zero[:1],
                            vext_max=spec.vext_max)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    x, iters, rn, _ = s.newton_solve(x0, resid_tol=1e-9, lin_tol=1e-10)
    s.close()
    rho = x[p.first_rho]
    assert rn <= 1e-9 and np.all(rho[zero[0] != 0] == 0.0) and rho[zero[0] == 0].min() > 0.0
