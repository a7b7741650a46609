"""Generate the golden fixtures of the nonlocal-density path from the reference.

Each case is one of the reference's own example decks (Examples/*/dft_input.dat),
optionally edited line by line.  For every case the reference's own C code
(built into oracle/_ref by oracle/refbuild) is run in a child process:

* set-up (stencils, bulk thermodynamics, mesh, external field, hard-wall lists),
* its built-in Newton solver to convergence,
* fill_resid_and_matrix_control at the converged state and at a seeded
  perturbation of it, recording the residual and the assembled Jacobian.

The fixture keeps the problem description (the reference's stencil tables,
constants, V_ext, zero-density flags, hard-wall masks), the two states, their
residuals, and Jacobian products J v, J^T w and the Schur-complement product
S v2 (S = A22 - A21 A11^-1 A12, block split of src/dft_linsolver_setup.c:182-241)
for seeded random vectors.  Run from the repository root:

    python tests/golden/make_golden.py [case ...]

The reference tree must be present (it is read in place, never copied).
"""
from __future__ import annotations

import atexit
import os
import shutil
import sys
import tempfile

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import tref  # noqa: E402

# reference physics ids (src/dft_globals_const.h)
DENSITY, HSRHOBAR, MF_EQ = 0, 1, 8


def deck(example, edits=None, surfaces=None):
    lines = tref.read_deck(os.path.join(tref.example_dir(example), "dft_input.dat"))
    if edits:
        lines = tref.edit_deck(lines, edits)
    return lines, surfaces or tref.example_dir(example)


def write_surfaces(path, text):
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "dft_surfaces.dat"), "w") as f:
        f.write(text)
    return path


SCHUR_LINSOLVE = "1 0 50"       # L_Schur Solver Az_kspace
MF_UNKNOWNS = "0 50 0 0 0"      # NL_Solver Max_NL_iter Physics_scaling ATTInA22Block Analyt_WJDC_Jac


def cases():
    tmp = tempfile.mkdtemp(prefix="golden_surfaces_")     # surface files of the edited decks, removed at exit
    atexit.register(shutil.rmtree, tmp, True)
    c = {}
    # 1-D FMT1 hard sphere against a hard wall (the reference's HS5 example as is)
    c["hs1d_wall"] = deck("HS5_FMT1_1D")
    # configuration 1: HS5 at L = 20 sigma, dx = 0.01 sigma (2000 elements), rho_b = 0.7, Newton to 1e-10
    c["hs1d_c1"] = deck("HS5_FMT1_1D", {"Size_x(idim)": "20.0", "Esize_x(idim)": "0.01",
                                        "Rho_b_0[icomp]": "0.7", "NL_rel_tol NL_abs_tol": "1.0e-6 1.0e-10 0.1"})
    # 1-D FMT1, hard wall on the left, reflecting boundary on the right (HS3 as is)
    c["hs1d_reflect"] = deck("HS3_FMT1_1D")
    # 1-D FMT1 + WCA attraction near a LJ 9-3 wall, mean field as its own unknown
    c["lj1d_mf"] = deck("LJ1_FMT1_WCA_1D", {
        "ATTInA22Block": MF_UNKNOWNS, "L_Schur": SCHUR_LINSOLVE})
    # 1-D binary White-Bear (FMT3) mixture with sizes 1 and 0.6 and WCA attraction
    c["mix1d_fmt3"] = deck("MIX2_FMT1_WCA_1D", {
        "Type_func (": "2 0", "Ncomp Mix_type": "2 1", "HS_diam[i]": "1. 0.6",
        "Sigma_ff[i][j]": "1. 0.8 0.8 0.6", "Eps_ff[i][j]": "1. 0.9 0.9 0.8",
        "Cut_ff[i][j]": "2.5 2.5 2.5 2.5", "Rho_b_0[icomp]": "0.25 0.35",
        "Esize_x(idim)": "0.05", "ATTInA22Block": MF_UNKNOWNS, "L_Schur": SCHUR_LINSOLVE})
    # 3-D FMT1 + WCA, LJ 9-3 planar wall at x=0, bulk at the far x end, periodic y and z
    surf3d = write_surfaces(os.path.join(tmp, "fmt1_wca_3d"), " 0 0 -1.5 0.0 0.0  0.0\n")
    wca3d = {"Size_x(idim)": "3.0 5.5 5.5", "Esize_x(idim)": "0.25 0.25 0.25",
             "Type_bc(x0": "-1 0", "Type_bc(x1": "1 1", "Type_bc(x2": "1 1",
             "Nwall_types Nwall Nlink": "1 1 1 0 0", "Xtest_reflect_TF": "0 0 0",
             "Lrough_surf": "0", "Lapply_offest": "0 0 0", "Cut_ff[i][j]": "2.5", "Rho_b_0[icomp]": "0.6",
             "ATTInA22Block": "0 20 0 0 0", "L_Schur": "1 0 100"}
    c["fmt1_wca_3d"] = deck("GEOM3_PLANE_ROUGH_3D", wca3d, surfaces=surf3d)
    # the same with L1D_bc: every node within 1 sigma of either x end holds the values of the node with the same x
    # on the line y = z = 0 (the one row of such nodes that is filled)
    c["fmt1_wca_3d_1dbc"] = deck("GEOM3_PLANE_ROUGH_3D", dict(wca3d, **{"L1D_bc": "1 1.0"}), surfaces=surf3d)
    # 1-D HS5 with the zero-dimensional-crossover Rosenfeld functional (FMT2) and the
    # White-Bear functional with the same vector correction (FMT4)
    c["hs1d_fmt2"] = deck("HS5_FMT1_1D", {"Type_func (": "1 0"})
    c["hs1d_fmt4"] = deck("HS5_FMT1_1D", {"Type_func (": "3 0"})
    # a binary hard-sphere FMT4 mixture (sizes 1 and 0.6) against a hard wall
    c["mix1d_fmt4"] = deck("MIX2_FMT1_WCA_1D", {
        "Type_func (": "3 0", "Ncomp Mix_type": "2 1", "HS_diam[i]": "1. 0.6",
        "Sigma_ff[i][j]": "1. 0.8 0.8 0.6", "Eps_ff[i][j]": "1. 0.9 0.9 0.8",
        "Cut_ff[i][j]": "2.5 2.5 2.5 2.5", "Rho_b_0[icomp]": "0.25 0.35", "Esize_x(idim)": "0.05",
        "Type_attr Type_pairPot": "-1 0", "Type of neutral surface-fluid": "1"})
    # 3-D hard spheres against a rough hard wall (patches of 0.5 sigma, heights up to 0.5 sigma),
    # periodic y and z: vector weighted densities with all three components nonzero
    rough3d = {"Size_x(idim)": "3.0 3.0 3.0", "Esize_x(idim)": "0.25 0.25 0.25",
               "Type_bc(x0": "-1 0", "Type_bc(x1": "1 1", "Type_bc(x2": "1 1",
               "Nwall_types Nwall Nlink": "1 1 1 0 0", "Xtest_reflect_TF": "0 0 0",
               "Lrough_surf": "1", "Lapply_offest": "1 0 0", "Type_attr Type_pairPot": "-1 0",
               "Type of neutral surface-fluid": "1",
               "Rho_b_0[icomp]": "0.6", "ATTInA22Block": "0 30 0 0 0", "L_Schur": "1 0 100"}
    for name, func in (("rough3d_fmt2", "1 0"), ("rough3d_fmt4", "3 0")):
        c[name] = deck("GEOM3_PLANE_ROUGH_3D", dict(rough3d, **{"Type_func (": func}), surfaces=surf3d)
    # the LJ1 fluid with the other mean-field kernels: LJ 12-6 cores (Type_attr 1: zero inside sigma; 3: zero
    # inside sigma, u(r_min) from sigma to r_min), Yukawa (K sigma = 1.8), exponential (decay length 0.5) and
    # square-well (range 1.5 sigma) attractions
    mf = {"ATTInA22Block": MF_UNKNOWNS, "L_Schur": SCHUR_LINSOLVE}
    c["lj1d_sigzero"] = deck("LJ1_FMT1_WCA_1D", dict(mf, **{"Type_attr Type_pairPot": "1 0"}))
    c["lj1d_jdc"] = deck("LJ1_FMT1_WCA_1D", dict(mf, **{"Type_attr Type_pairPot": "3 0"}))
    c["yuk1d_mf"] = deck("LJ1_FMT1_WCA_1D", dict(mf, **{"Type_attr Type_pairPot": "0 3", "YukawaK_ff[i][j]": "1.8"}))
    c["exp1d_mf"] = deck("LJ1_FMT1_WCA_1D", dict(mf, **{"Type_attr Type_pairPot": "0 4", "YukawaK_ff[i][j]": "0.5"}))
    c["sw1d_mf"] = deck("LJ1_FMT1_WCA_1D", dict(mf, **{"Type_attr Type_pairPot": "0 5", "Cut_ff[i][j]": "1.5"}))
    # HS5's hard wall (boundary weights) with a WCA fluid (eps 1/1.2 kT, cut 2.5) at HS5's rho_b = 0.75: the
    # mean-field stencil takes the hard-wall weights too
    c["hslj1d_wall"] = deck("HS5_FMT1_1D", dict(mf, **{"Type_attr Type_pairPot": "0 0", "Eps_ff[i][j]": "0.8333333333333334",
                                                   "Cut_ff[i][j]": "2.5", "Rho_b_0[icomp]": "0.75"}))
    # liquid-vapor interface (BULK3: PHASE_INTERFACE between the binodal densities, the mid density pinned by
    # Lconstrain_interface), with reflecting ends as in the example and with bulk ends (LBB / RTF sentinels)
    c["lv1d_interface"] = deck("BULK3_FMT1_WCA_1D", {"L_Schur": SCHUR_LINSOLVE})
    c["lv1d_bulkbc"] = deck("BULK3_FMT1_WCA_1D", {"L_Schur": SCHUR_LINSOLVE, "Type_bc(x0": "0 0"})
    # ATTInA22Block = 1: the mean field summed into the Euler-Lagrange rows (no mean-field unknowns)
    c["lj1d_a22"] = deck("LJ1_FMT1_WCA_1D", {"ATTInA22Block": "0 50 0 1 0", "L_Schur": SCHUR_LINSOLVE})
    # mesh coarsening: HS6 (four quadrature zones at 2, 4, 5 sigma from the wall, residuals of the nodes off
    # each zone's coarse lattice averaged from their neighbours) and HS7 (the same with a Jacobian one
    # zone coarser than the residual near the wall)
    c["hs1d_zones"] = deck("HS6_FMT1_1D")
    c["hs1d_jaczones"] = deck("HS7_FMT1_1D")
    # the LJ1 fluid (FMT1 + WCA at a 9-3 wall) with HS6's four zones at 2, 4, 5 sigma from the wall, the mean field
    # as its own unknown and summed into the Euler-Lagrange rows (ATTInA22Block = 1)
    zones = {"Nzone (Coarsens": "4", "Rmax_zone": "2. 4. 5.", "Mesh_coarsening": "1"}
    c["lj1d_zones"] = deck("LJ1_FMT1_WCA_1D", dict(zones, **mf))
    c["lj1d_zones_a22"] = deck("LJ1_FMT1_WCA_1D", dict(zones, **{"ATTInA22Block": "0 50 0 1 0",
                                                                 "L_Schur": SCHUR_LINSOLVE}))
    # MIX1's hard wall (boundary weights, one surface list per component size) with three and four hard-sphere
    # components of different diameters (FMT1, and FMT3 for the four)
    mix = {"Mass[i]": "1. 1. 1. 1.", "Charge[i]": "0. 0. 0. 0.", "Pol[i]": "0. 0. 0. 0.",
           "Eps_ff[i][j]": "0. 0. 0. 0.", "Cut_ff[i][j]": "0. 0. 0. 0.", "Bond_ff[i][j]": "1. 1. 1. 1."}
    c["mix3_hw1d"] = deck("MIX1_FMT1_1D", dict(mix, **{"Ncomp Mix_type": "3 0", "Sigma_ff[i][j]": "1. 0.8 0.6",
                                                      "Rho_b_0[icomp]": "0.25 0.2 0.3"}))
    c["mix4_hw1d_fmt3"] = deck("MIX1_FMT1_1D", dict(mix, **{"Type_func (": "2 0", "Ncomp Mix_type": "4 0",
                                                           "Sigma_ff[i][j]": "1. 0.85 0.7 0.55",
                                                           "Rho_b_0[icomp]": "0.15 0.15 0.2 0.2"}))
    return c


def block_lists(ints, nunk):
    """ind / dep / density unknown lists as linsolver_setup_HSTYPE makes them."""
    ndim, nrb, lhard, nlists = int(ints[0]), int(ints[9]), int(ints[13]), int(ints[14])
    first_rho, first_rb = int(ints[22]), int(ints[23])
    ncomp = int(ints[8])
    one = (lhard and nlists == 2) or (not lhard and nlists == 1)
    ind, dep, dens = [], [], []
    nrb_tot = nrb + 2 * ndim
    for u in range(nunk):
        if first_rho <= u < first_rho + ncomp:
            dens.append(u)
        elif first_rb <= u < first_rb + nrb_tot:
            k = u - first_rb
            if one and ((1 < k < nrb) or k >= nrb + ndim):
                dep.append(u)
            else:
                ind.append(u)
        else:
            ind.append(u)
    return ind, dep, dens


def probe(n, k):
    """Deterministic probe vector k of length n (no RNG, so any machine rebuilds it)."""
    i = np.arange(n, dtype=np.float64)
    return np.sin(1.3 + 0.7071 * k + 0.61803 * (k + 1) * i)


def make_case(name, lines, surfaces, states=("x_newton", ("x_newton", 7, 0.02))):
    r = tref.extract(lines, surfaces, newton=True, fill_states=list(states))
    ints = r["info_ints"]
    nunk, nbox = int(ints[7]), int(ints[5])
    assert int(ints[6]) == nbox and np.array_equal(r["l2b"], np.arange(nbox)) and np.array_equal(r["b2g"], np.arange(nbox)), \
        "single-process box must equal the global mesh"
    out = {"info_ints": ints, "info_doubles": r["info_doubles"], "vext": r["vext"],
           "zero_density": r["zero_density"].astype(np.int8), "newton_iters": np.int32(r["newton_iters"])}
    if "boundary_nodes" in r:
        out["boundary_nodes"] = r["boundary_nodes"]
        out["fluid_masks"] = r["fluid_masks"].astype(np.int16)
    for (isten, idx), (off, w, hw) in r["stencils"].items():
        out[f"sten_{isten}_{idx}_off"] = off.astype(np.int16)
        out[f"sten_{isten}_{idx}_w"] = w
        if hw is not None:
            out[f"sten_{isten}_{idx}_hw"] = hw
    for (zone, isten, idx), (off, w, hw) in r["zone_stencils"].items():
        out[f"zsten_{zone}_{isten}_{idx}_off"] = off.astype(np.int16)
        out[f"zsten_{zone}_{isten}_{idx}_w"] = w
        if hw is not None:
            out[f"zsten_{zone}_{isten}_{idx}_hw"] = hw
    if "coarsen_flag" in r:
        out["coarsen_flag"] = r["coarsen_flag"]
    out["nel_hit"], out["nel_hit2"] = r["nel_hit"].astype(np.int8), r["nel_hit2"].astype(np.int8)
    out["integ"] = r["integ"]
    ind, dep, dens = block_lists(ints, nunk)
    out["blk_ind"], out["blk_dep"], out["blk_dens"] = (np.array(v, np.int32) for v in (ind, dep, dens))
    N = nunk * nbox
    out["x_newton"] = r["x_newton"]
    out["states"] = np.array([0 if isinstance(st, str) else 1 for st in states], np.int8)
    for k, f in enumerate(r["fills"]):
        ng = f["nglobal"]
        assert ng == nbox
        J = sp.csr_matrix((f["vals"], (f["rows"], f["cols"])), shape=(N, N))
        out[f"x{k}"] = f["x"]
        out[f"resid_sum{k}"] = np.float64(f["resid_sum"])
        out[f"R{k}"] = -f["rhs"]  # rhs = -residual
        v = probe(N, 0)
        out[f"Jv{k}"] = (J @ v).reshape(nunk, nbox)
        w = probe(N, 1)
        out[f"JTw{k}"] = (J.T @ w).reshape(nunk, nbox)
        # Schur product on the density block, block operators built from J
        idx1 = np.concatenate([np.arange(u * nbox, (u + 1) * nbox) for u in ind + dep])
        idx2 = np.concatenate([np.arange(u * nbox, (u + 1) * nbox) for u in dens])
        depmask = np.concatenate([np.full(nbox, u in dep) for u in ind + dep])
        A11 = J[idx1][:, idx1].tocsr()
        B = A11.multiply(sp.csr_matrix(depmask[:, None].astype(float))).tocsr()
        B.setdiag(0.0)
        B.eliminate_zeros()
        A12, A21, A22 = J[idx1][:, idx2], J[idx2][:, idx1], J[idx2][:, idx2]
        v2 = probe(len(idx2), 2)
        u1 = A12 @ v2
        y1 = np.where(depmask, -u1 - B @ u1, -u1)
        Sv = A22 @ v2 - A21 @ y1
        out[f"schur_Sv{k}"] = Sv.reshape(len(dens), nbox)
        out[f"nnz{k}"] = np.int64(J.nnz)
        out[f"omega_s{k}"] = np.float64(f["omega_s"])
        out[f"ads{k}"], out[f"ads_b{k}"] = f["ads"], f["ads_b"]
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    return out


def main(argv):
    if not os.path.exists(tref.REF_LIB):
        tref.build_ref()
    allc = cases()
    names = argv or list(allc)
    for n in names:
        lines, surf = allc[n]
        # the 3-D cases keep only the perturbed state to stay small
        states = (("x_newton", 7, 0.02),) if "3d" in n else ("x_newton", ("x_newton", 7, 0.02))
        o = make_case(n, lines, surf, states)
        k = len(states) - 1
        print(f"{n}: nodes={o['info_ints'][5]} unknowns={o['info_ints'][7]} newton_iters={o['newton_iters']} "
              f"|R|={np.abs(o[f'R{k}']).max():.3e} nnz={o[f'nnz{k}']}")


if __name__ == "__main__":
    main(sys.argv[1:])
