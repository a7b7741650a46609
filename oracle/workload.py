"""The 128^3 FMT1 + WCA workload for the oracle alone (test infrastructure and the CPU reference arm).

Builds the problem the GPU arm of bench.py solves, without the product package: the delta, theta and
attraction stencil tables and the bulk constants at rho_b = 0.6 come from the reference's own set-up
(calc_stencils src/dft_stencil.c:40-287 and the thermo of src/dft_thermo_hs.c:226-334 /
src/dft_thermo_att.c:44-63, recorded in tests/golden/sten3d_dx010.npz by tests/golden/make_stencil_golden.py);
the external field is the synthetic rough 12-3 LJ wall of the workload (seeded numpy PCG64 patch heights),
restated here in numpy.  `initial_state` gives the state the GPU arm's timed solves start from
(rho_b exp(-V) with its own weighted densities and mean field), formed with the oracle's own sums on the nodes
a sample of z-planes reads.
"""
from __future__ import annotations

import os
from types import SimpleNamespace

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(os.path.dirname(HERE), "tests", "golden", "sten3d_dx010.npz")

BC_IN_WALL, BC_IN_BULK, BC_PERIODIC = -1, 0, 1
KT, EPS_W, SIGMA_W, WALL_X, PATCHES, AMPLITUDE, SEED = 1.2, 1.0, 1.0, 1.0, 16, 0.5, 1234
LJ123_PREF = 1.0 / (0.75 * 4.0 ** (-1.0 / 3.0))     # min of C ((s/d)^12 - (s/d)^3) is -1
FMT_REACH = 5                                      # theta and delta reach at dx = 0.1 (nodes)


def rough_wall_vext(nx, esize, vext_max):
    """V_ext/kT of the workload's rough 12-3 wall: eps_w C ((sigma/d)^12 - (sigma/d)^3) / kT with d = x - (1 + h(y, z)),
    h i.i.d. U(-0.5, 0.5) on 16 x 16 patches of the periodic y-z plane (PCG64 seed 1234); d <= 0 or V >= vext_max
    clipped to vext_max.  [1][N], node = ix + nx (iy + ny iz)."""
    rng = np.random.default_rng(SEED)
    hpatch = rng.uniform(-AMPLITUDE, AMPLITUDE, size=(PATCHES, PATCHES))
    ny, nz = nx[1], nx[2]
    h = hpatch[(np.arange(ny) * PATCHES) // ny][:, (np.arange(nz) * PATCHES) // nz]
    x = np.arange(nx[0]) * esize[0]
    d = x[None, None, :] - (WALL_X + h.T[:, :, None])
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        s = np.where(d > 0, SIGMA_W / np.maximum(d, 1e-300), np.inf)
        v = (EPS_W / KT) * LJ123_PREF * (s ** 12 - s ** 3)
    v = np.where((d <= 0) | (v >= vext_max) | ~np.isfinite(v), vext_max, v)
    return v.reshape(1, -1)


def config2_problem(n=128):
    """The workload on an n^3 grid (dx = 0.1) as an attribute bag that oracle/orc.py's Oracle accepts."""
    z = np.load(FIXTURE)
    d = np.asarray(z["info_doubles"])
    esize = (float(z["esize"]),) * 3
    nx = (n, n, n)
    pc = lambda k: np.array(d[7 + 6 * k: 8 + 6 * k])  # noqa: E731  per-component blocks of the reference's scalars
    vext_max = float(d[6])
    vext = rough_wall_vext(nx, esize, vext_max)
    st = {}
    for t in (0, 1, 2):
        st[(t, 0)] = (np.asarray(z[f"sten_{t}_0_off"], np.int16), np.asarray(z[f"sten_{t}_0_w"]), None)
    return SimpleNamespace(
        ndim=3, nx=nx, esize=esize,
        bc=((BC_IN_WALL, BC_IN_BULK), (BC_PERIODIC, BC_PERIODIC), (BC_PERIODIC, BC_PERIODIC)),
        ncomp=1, functional=0, attraction=1, att_in_a22=0, single_size=1, hard_surf=0, nlists_hw=1,
        first_rho=0, first_rb=1, first_mf=11, nunk=12, nnodes=n ** 3,
        hs_diam=pc(0), rho_b=pc(1), betamu_hs_ex=pc(2), betamu_att=pc(3), inv_rad=pc(4), inv_4pir=pc(5),
        inv_4pirsq=pc(6), fac_overlap=pc(7), dphi_bulk=np.array(d[65:69]), vext_max=vext_max, vext=vext,
        zero_density=(vext >= vext_max).astype(np.int8), stencils=st)


def _rows_parallel(oracle, x, ranges, threads):
    """The oracle's residual on node ranges [(begin, end)], one range per thread (ctypes releases the GIL)."""
    from concurrent.futures import ThreadPoolExecutor
    out = np.zeros_like(x)

    def one(r):
        R = oracle.resid_rows(x, r[0], r[1])
        out[:, r[0]:r[1]] = R[:, r[0]:r[1]]
    with ThreadPoolExecutor(max(1, threads)) as ex:
        list(ex.map(one, ranges))
    return out


def plane_ranges(p, planes, threads):
    """Node ranges covering the z-planes `planes` (taken periodic in z), at least `threads` of them when the planes
    are fewer than the threads (planes split into row blocks)."""
    nxy = p.nx[0] * p.nx[1]
    zs = sorted({z % p.nx[2] for z in planes})
    parts = max(1, threads // len(zs))
    step = -(-nxy // parts)
    return [(z * nxy + b, z * nxy + min(nxy, b + step)) for z in zs for b in range(0, nxy, step)]


def initial_state(p, oracle, sample_planes, threads=1):
    """The state the GPU arm's solves start from, on the nodes a residual of z-planes [0, sample_planes) reads:
    rho_b exp(-V) (0 on zero-density rows) everywhere; the weighted densities and the mean field as their own
    oracle sums (R = -x + sums, twice: independent rows, then their local copies) on the sampled planes and the
    FMT reach around them."""
    N = p.nnodes
    x = np.zeros((p.nunk, N))
    v = p.vext[0]
    rho = p.rho_b[0] * np.exp(-np.minimum(v, 50.0))
    rho[(p.zero_density[0] != 0) | (v >= p.vext_max)] = 0.0
    x[0] = rho
    planes = range(-FMT_REACH, sample_planes + FMT_REACH)
    ranges = plane_ranges(p, planes, threads)
    for _ in range(2):
        R = _rows_parallel(oracle, x, ranges, threads)
        for b, e in ranges:
            x[p.first_rb:, b:e] += R[p.first_rb:, b:e]
    return x
