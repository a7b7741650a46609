"""Problem description of the nonlocal-density path.

A :class:`Problem` carries everything the reference's fill reads for one
hard-sphere (+ WCA mean-field) problem on a regular lattice: geometry and
boundary conditions, the unknown layout, the bulk constants, the external
field and zero-density flags, the hard-wall boundary masks and the stencil
tables ``stencils[(type, index)] = (offsets[L][ndim], weights[L], hw[L][2^ndim] | None)``
with type 0 = delta (DELTA_FN_R), 1 = theta (THETA_FN_R), 2 = attraction
(THETA_PAIRPOT_RCUT) and index = icomp (+ ncomp*jcomp for the pair stencil),
exactly as the reference stores them (src/dft_globals_const.h:635-646).

Field layouts are SoA ``[component or unknown][node]`` with
``node = ix + nx*(iy + ny*iz)``, which is the layout of the reference's
``x[iunk][inode_box]`` arrays for one process (src/rf_allo.c:171).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# reference codes (src/dft_globals_const.h)
BC_IN_WALL, BC_IN_BULK, BC_PERIODIC, BC_REFLECT = -1, 0, 1, 2
FMT1, FMT2, FMT3, FMT4 = 0, 1, 2, 3
DELTA, THETA, UATT = 0, 1, 2


@dataclass
class Problem:
    ndim: int
    nx: tuple
    esize: tuple
    bc: tuple                      # ((left, right) per dimension)
    ncomp: int
    functional: int = FMT1
    attraction: int = 0
    att_in_a22: int = 0
    single_size: int = 1
    hard_surf: int = 0
    nlists_hw: int = 1
    rho_b: np.ndarray = None
    hs_diam: np.ndarray = None
    betamu_hs_ex: np.ndarray = None
    betamu_att: np.ndarray = None
    inv_rad: np.ndarray = None
    inv_4pir: np.ndarray = None
    inv_4pirsq: np.ndarray = None
    fac_overlap: np.ndarray = None
    dphi_bulk: np.ndarray = None   # bulk dPhi/dn0..dn3 (Dphi_Drhobar_b)
    vext_max: float = 1e300
    # phase interface (Type_interface 2): low/high-side bulk states, the EL chemical potential, a pinned density
    interface: int = 0
    rho_b_lbb: np.ndarray = None
    rho_b_rtf: np.ndarray = None
    dphi_lbb: np.ndarray = None
    dphi_rtf: np.ndarray = None
    betamu_if: np.ndarray = None
    pin_node: int = -1
    pin_value: float = 0.0
    # quadrature zones / mesh coarsening (Nzone, Mesh_coarsening, Coarser_jac): per-node flag (residual
    # zone >= 0, or -1/-2/-3: the node's rows average its neighbours along x/y/z), stencils of zones >= 1
    nzone: int = 1
    mesh_coarsening: int = 0
    coarser_jac: int = 0
    nwall: int = 0
    zone_flag: np.ndarray = None
    l1d_bc: int = 0                  # L1D_bc: nodes flagged -999 copy the line through the origin along dim_1dbc
    dim_1dbc: int = 0
    zone_stencils: dict = None
    rhobar_bc: np.ndarray = None
    vext: np.ndarray = None        # [ncomp][N]
    zero_density: np.ndarray = None  # [ncomp][N] int8
    boundary_nodes: np.ndarray = None  # [nlists][N] int32, -1 = not a boundary node
    fluid_masks: np.ndarray = None     # [nlists][2^ndim][N] int16
    stencils: dict = field(default_factory=dict)
    # integration (objectives Omega_s and Gamma_ex): per-node weights [ncomp][N] of integrateInSpace with
    # Nel_hit2 (w_fluid) and Nel_hit (w_bulk), the bulk weighted densities n3 n2 n1 n0 and betamu
    w_fluid: np.ndarray = None
    w_bulk: np.ndarray = None
    rhobar_b: np.ndarray = None
    betamu: np.ndarray = None

    # ---- unknown layout (setup_nunk_per_node, src/dft_defs_unknowns.c:37-176)
    @property
    def nnodes(self) -> int:
        return int(np.prod(self.nx[: self.ndim]))

    @property
    def nrb(self) -> int:
        return 4 + 2 * self.ndim

    @property
    def first_rho(self) -> int:
        return 0

    @property
    def first_rb(self) -> int:
        return self.ncomp

    @property
    def first_mf(self) -> int:
        return self.ncomp + self.nrb if (self.attraction and not self.att_in_a22) else -1

    @property
    def nunk(self) -> int:
        return self.ncomp + self.nrb + (self.ncomp if (self.attraction and not self.att_in_a22) else 0)

    def dependent_rb(self) -> list:
        """Weighted densities that are local copies (n1, n0, V1) for one particle size."""
        if not self.single_size:
            return []
        nd = self.ndim
        return [k for k in range(self.nrb) if (1 < k < 4) or k >= 4 + nd]


def from_golden(z) -> Problem:
    """Build a Problem from a fixture written by tests/golden/make_golden.py."""
    ints = np.asarray(z["info_ints"])
    d = np.asarray(z["info_doubles"])
    ndim = int(ints[0])
    nx = tuple(int(v) for v in ints[1:4])
    ncomp = int(ints[8])
    lhard, nlists, nwall = int(ints[13]), int(ints[14]), int(ints[15])
    bc = tuple((int(ints[16 + 2 * i]), int(ints[17 + 2 * i])) for i in range(3))
    pc = lambda k: np.array(d[7 + 6 * k: 7 + 6 * k + ncomp])  # noqa: E731  per-component block k
    single = (lhard and nlists == 2) or ((not lhard) and nwall > 0 and nlists == 1)
    st = {}
    for key in z.files:
        if key.startswith("sten_") and key.endswith("_w"):
            _, t, idx, _ = key.split("_")
            t, idx = int(t), int(idx)
            hwk = f"sten_{t}_{idx}_hw"
            st[(t, idx)] = (np.asarray(z[f"sten_{t}_{idx}_off"], np.int16), np.asarray(z[key]),
                            np.asarray(z[hwk]) if hwk in z.files else None)
    p = Problem(
        ndim=ndim, nx=nx, esize=tuple(float(v) for v in d[0:3]), bc=bc, ncomp=ncomp,
        functional=int(ints[10]), attraction=int(int(ints[11]) >= 0), att_in_a22=int(ints[12]),
        single_size=int(bool(single)), hard_surf=lhard, nlists_hw=nlists,
        hs_diam=pc(0), rho_b=pc(1), betamu_hs_ex=pc(2), betamu_att=pc(3), inv_rad=pc(4), inv_4pir=pc(5),
        inv_4pirsq=pc(6), fac_overlap=pc(7), dphi_bulk=np.array(d[65:69]), vext_max=float(d[6]),
        vext=np.asarray(z["vext"], np.float64), zero_density=np.asarray(z["zero_density"], np.int8),
        boundary_nodes=np.asarray(z["boundary_nodes"], np.int32) if "boundary_nodes" in z.files else None,
        fluid_masks=np.asarray(z["fluid_masks"], np.int16) if "fluid_masks" in z.files else None,
        stencils=st)
    assert p.nunk == int(ints[7]), (p.nunk, int(ints[7]))
    p.nwall = nwall
    p.rhobar_bc = np.array(d[55:65])
    if len(ints) > 38:
        p.nzone, p.mesh_coarsening, p.coarser_jac = int(ints[25]), int(ints[37]), int(ints[38])
    if "coarsen_flag" in z.files:
        p.zone_flag = np.asarray(z["coarsen_flag"], np.int32)
    if len(ints) > 47:
        p.l1d_bc, p.dim_1dbc = int(ints[46]), int(ints[47])
    zst = {}
    for key in z.files:
        if key.startswith("zsten_") and key.endswith("_w"):
            _, zone, t, idx, _ = key.split("_")
            base = f"zsten_{zone}_{t}_{idx}"
            zst.setdefault(int(zone), {})[(int(t), int(idx))] = (
                np.asarray(z[base + "_off"], np.int16), np.asarray(z[key]),
                np.asarray(z[base + "_hw"]) if base + "_hw" in z.files else None)
    p.zone_stencils = zst
    if len(ints) > 45 and int(ints[36]) == 2:     # Type_interface = PHASE_INTERFACE
        p.interface = 2
        if nwall == 0:                            # LBB / RTF sentinels beyond bulk boundaries
            p.rho_b_lbb, p.rho_b_rtf = np.array(d[329:329 + ncomp]), np.array(d[335:335 + ncomp])
            p.dphi_lbb, p.dphi_rtf = np.array(d[341:345]), np.array(d[351:355])
        else:
            p.rho_b_lbb, p.rho_b_rtf = p.rho_b.copy(), p.rho_b.copy()
            p.dphi_lbb, p.dphi_rtf = p.dphi_bulk.copy(), p.dphi_bulk.copy()
        p.betamu_if = np.array(d[361:361 + ncomp])
        if int(ints[44]):                         # Lconstrain_interface
            gd = int(ints[45])
            p.pin_node = int(0.5 * d[3 + gd] / d[gd])
            p.pin_value = 0.5 * (float(d[329]) + float(d[335]))
    if "integ" in z.files:
        integ = np.asarray(z["integ"])
        vol_el, nel_v, area, fac_vol, fac_area, per_area = integ[:6]
        scale = fac_vol / (fac_area * area) if (per_area and area > 0) else fac_vol
        unit = vol_el / nel_v * scale
        p.w_fluid = np.asarray(z["nel_hit2"], np.float64) * unit
        p.w_bulk = np.asarray(z["nel_hit"], np.float64) * unit
        p.rhobar_b = np.array(d[55:59])
        if p.interface:
            # the bulk free-energy density of an interface is that of the high-side state
            # (Rhobar_b_RTF, integrand_hs_freen_bulk, src/dft_energy_hs.c:45-60; rhobar_icomp,
            # src/dft_thermo_hs.c:292-311); n3 n2 n1 n0 as Rhobar_b
            rtf, hs = np.array(d[335:335 + ncomp]), p.hs_diam
            fo = p.fac_overlap
            area = np.pi * hs * hs * rtf * fo
            p.rhobar_b = np.array([np.sum(np.pi * hs ** 3 / 6.0 * rtf * fo), np.sum(area),
                                   np.sum(area * p.inv_4pir), np.sum(area * p.inv_4pirsq)])
        p.betamu = np.array(integ[6:6 + ncomp])
    return p
