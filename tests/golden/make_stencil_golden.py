"""Generate the 3-D stencil fixtures of the 128^3 and 256^3 workloads from the reference.

The 128^3 workload (dx = 0.1 sigma) and the 256^3 workload (dx = 0.08 sigma) use
a 3-D FMT1 fluid (sigma = 1) with the WCA mean-field attraction of a
cut-and-shifted LJ 12-6 pair potential (Type_attr 0: core at r_min,
eps/kT = 1/1.2, cut 2.5 sigma).  Their stencil tables (delta shell, theta ball,
attraction ball) depend only on the element size, the hard-sphere diameter and
the pair potential once the box is wider than the stencils, so the
reference's own calc_stencils (src/dft_stencil.c:40-287, built into oracle/_ref
by oracle/refbuild) is run on a small box, periodic in y and z, at each element
size and its zone-0 tables are kept:

    sten3d_dx010.npz   delta (844 points), theta (1015) and attraction (71 831) at dx = 0.1
    sten3d_dx008.npz   the same at dx = 0.08 (attraction: 137 299 points)

Offsets are stored as int8 (every reach is below 32 nodes), weights as float64; the
reference's set-up scalars of the deck (bulk state rho_b = 0.6: weighted densities,
dPhi/dn, excess chemical potentials) are kept with them (info_ints, info_doubles).
Run from the repository root with the reference tree present (read in place):

    python tests/golden/make_stencil_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import tref  # noqa: E402

KT = 1.2
# element size, box edge (a multiple of it); where a stencil is wider than a periodic box the reference folds its
# points onto their periodic images (ijk_to_isten_index, src/dft_stencil.c:654-675; a 3-sigma box at dx = 0.1
# gives 40 610 attraction points), so the box here is wider than the stencils
CASES = {"sten3d_dx010": (0.1, 6.0), "sten3d_dx008": (0.08, 6.4)}


def deck(esize, edge, surfaces_dir):
    with open(os.path.join(surfaces_dir, "dft_surfaces.dat"), "w") as f:
        f.write(" 0 0 -1.5 0.0 0.0  0.0\n")     # one planar wall surface outside the box (stencils ignore it)
    lines = tref.read_deck(os.path.join(tref.example_dir("GEOM3_PLANE_ROUGH_3D"), "dft_input.dat"))
    return tref.edit_deck(lines, {
        "Size_x(idim)": f"{edge} {edge} {edge}", "Esize_x(idim)": f"{esize} {esize} {esize}",
        "Type_bc(x0": "-1 0", "Type_bc(x1": "1 1", "Type_bc(x2": "1 1",
        "Nwall_types Nwall Nlink": "1 1 1 0 0", "Xtest_reflect_TF": "0 0 0",
        "Lrough_surf": "0", "Lapply_offest": "0 0 0", "Eps_ff[i][j]": repr(1.0 / KT), "Cut_ff[i][j]": "2.5",
        "Rho_b_0[icomp]": "0.6", "ATTInA22Block": "0 20 0 0 0", "L_Schur": "1 0 100"})


def make(name, esize, edge):
    with tempfile.TemporaryDirectory() as surf:
        t0 = time.time()
        r = tref.extract(deck(esize, edge, surf), surf, newton=False, fill_states=())
    d = r["info_doubles"]
    # the reference's set-up scalars of the same deck (rho_b = 0.6): bulk weighted densities, dPhi/dn and the
    # excess chemical potentials (its own thermo, src/dft_thermo_hs.c:226-334, src/dft_thermo_att.c:44-63)
    out = {"esize": np.float64(esize), "kT": np.float64(KT), "hs_diam": np.float64(d[7]),
           "sigma_ff": np.float64(d[147]), "eps_ff": np.float64(d[111]), "cut_ff": np.float64(d[183]),
           "info_ints": r["info_ints"], "info_doubles": d}
    for (isten, idx), (off, w, _hw) in r["stencils"].items():
        assert np.abs(off).max() < 128
        out[f"sten_{isten}_{idx}_off"] = off.astype(np.int8)
        out[f"sten_{isten}_{idx}_w"] = w
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    lens = {k: len(v) for k, v in out.items() if k.endswith("_w")}
    print(f"{name}: {lens} ({time.time() - t0:.0f} s)")


def main(argv):
    if not os.path.exists(tref.REF_LIB):
        tref.build_ref()
    for name in argv or list(CASES):
        make(name, *CASES[name])


if __name__ == "__main__":
    main(sys.argv[1:])
