"""Make the surface fixtures tests/golden/surf_*.npz from the reference's own GEOM example decks.

For each deck the reference library (oracle/_ref, built from the reference tree by
oracle/refbuild/Makefile) runs its set-up (tref.extract: surfaces, mesh, external field) and the
fixture keeps, next to the surface spec that tramonto_gb300.surfaces.read_deck makes of the same
deck (spec_arrays), the reference's results:
  ref_vext [ncomp][nodes]      V_ext/kT (Vext)
  ref_zero [ncomp][nodes]      Zero_density_TF
  ref_wall_elems [elements]    Wall_elems of the last list (last wall owning the element, -1 fluid)
  ref_sigma_wf/eps_wf/cut_wf   the wall-fluid parameters the reference used [ncomp][Nwall_type]
  ref_wall_pos [Nwall][3]      WallPos
  ref_seconds                  the reference's set-up time here (single thread)
The generator checks that the spec read from the deck carries the reference's parameters and wall
positions.  Run from the repository root:  python tests/golden/make_surface_golden.py [deck ...]
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import tref  # noqa: E402
from tramonto_gb300 import surfaces  # noqa: E402

# deck -> fixture name: the example decks whose surfaces the GPU builder covers (no roughness, angle cutouts
# or Lhard_surf), small enough for the reference to set up in about two minutes: every such GEOM deck with
# integrated LJ 12-6 walls, decks of the distance-based 9-3 walls in 1-D, 2-D and 3-D, rough surfaces and
# angle cutouts
DECKS = {
    "GEOM25_CYL_PORE_2D": "surf_cylpore2d",
    "GEOM31_TAPERED_CYLPORE_3D": "surf_taperedpore3d",
    "GEOM8_BLOCK_2D": "surf_block2d",
    "GEOM9_BLOCK_3D": "surf_block3d",
    "GEOM10_SPHERE_3D": "surf_sphere3d",
    "GEOM11_CYL_2D": "surf_cyl2d",
    "GEOM12_CYL_2D": "surf_cyl2d_six",
    "GEOM20_CYL_3D": "surf_cyl3d",
    "GEOM23_CYL_PERIODIC_3D": "surf_cyl3d_periodic",
    "GEOM34_PLANE_PERIODIC3_2D": "surf_plane2d_periodic",
    "GEOM35_PLANE_PERIODIC_3D": "surf_plane3d_periodic",
    "GEOM37_WEDGE_LINEAR_2D": "surf_wedge2d",
    "GEOM38_WEDGE_3D": "surf_wedge3d",
    # distance-based walls (Ipot_wf_n 2: the 9-3 cut-and-shifted form of the distance to the surface)
    "GEOM32_PLANE_PERIODIC_2D": "surf_lj93_plane2d_cosx",
    "GEOM33_PLANE_PERIODIC2_2D": "surf_lj93_plane2d_cosy",
    "LJ1_FMT1_WCA_1D": "surf_lj93_1d",
    "MIX2_FMT1_WCA_1D": "surf_lj93_mix1d",
    "CONT1_FMT1_WCA_1D": "surf_lj93_cont1d",
    "BC1_FMT1_WCA_ELEC_2D": "surf_lj93_2d_three",
    "BC7_FMT1_WCA_ELEC_3D": "surf_lj93_3d_three",
    # roughness patches (Rough_precalc from the C library's rand() after srand(135649))
    "GEOM1_PLANE_ROUGH_2D": "surf_rough_plane2d",
    "GEOM3_PLANE_ROUGH_3D": "surf_rough_plane3d",
    "GEOM6_PLANE_ROUGH_VEXTINT_2D": "surf_rough_vextint2d",
    "GEOM7_PLANE_ROUGH_VEXTINT_3D": "surf_rough_vextint3d",
    "GEOM13_CYL_ROUGH_2D": "surf_rough_cyl2d",
    "GEOM21_CYL_ROUGH_3D": "surf_rough_cyl3d",
    "GEOM26_CYL_PORE_ROUGH_2D": "surf_rough_cylpore2d",
    # angle cutouts (wedges of cylinders, pores and slits; two and twelve wall types)
    "GEOM14_CYL_WEDGECUTOUT_2D": "surf_cut_cyl2d",
    "GEOM15_CYL_WEDGE2TYPES_2D": "surf_cut_cyl2d_twelve",
    "GEOM16_CYL_WEDGE2TYPES_REFLECT_2D": "surf_cut_cyl2d_reflect",
    "GEOM22_CYL_WEDGE2TYPES_3D": "surf_cut_cyl3d",
    "GEOM27_CYL_PORE_WEDGE2TYPES_2D": "surf_cut_cylpore2d",
    "GEOM28_CYLPORE_WEDGE2TYPES_3D": "surf_cut_cylpore3d",
    "GEOM29_SLITPORE_2D": "surf_cut_slitpore2d",
    "GEOM30_TAPERED_SLITPORE_2D": "surf_cut_taperedslit2d",
    "GEOM36_PLANE_NOTCH_2D": "surf_cut_notch2d",
}


def make(deck, name):
    d = tref.example_dir(deck)
    spec = surfaces.read_deck(os.path.join(d, "dft_input.dat"))
    t0 = time.time()
    ref = tref.extract(tref.read_deck(os.path.join(d, "dft_input.dat")), surfaces_from=d)
    secs = time.time() - t0
    if "error" in ref:
        raise RuntimeError(ref["error"])
    nt, nc, nw = spec.ntypes, spec.ncomp, spec.nwalls
    for key in ("sigma_wf", "eps_wf", "cut_wf"):
        mine = np.array([[getattr(spec.type[t], key)[c] for t in range(nt)] for c in range(nc)])
        assert np.array_equal(mine, ref[key]), (deck, key, mine, ref[key])
    mine_pos = np.array([spec.wall_pos[w][:] for w in range(nw)])
    assert np.array_equal(mine_pos, ref["wall_pos"]), (deck, mine_pos, ref["wall_pos"])
    out = surfaces.spec_arrays(spec)
    out.update(ref_vext=ref["vext"], ref_zero=ref["zero_density"].astype(np.int8), ref_wall_elems=ref["wall_elems"],
               ref_sigma_wf=ref["sigma_wf"], ref_eps_wf=ref["eps_wf"], ref_cut_wf=ref["cut_wf"],
               ref_wall_pos=ref["wall_pos"], ref_seconds=np.float64(secs))
    path = os.path.join(ROOT, "tests", "golden", name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{deck}: {ref['vext'].shape} nodes, reference set-up {secs:.1f} s -> {os.path.relpath(path, ROOT)}")


if __name__ == "__main__":
    tref.build_ref()
    for deck in (sys.argv[1:] or list(DECKS)):
        make(deck, DECKS[deck])
