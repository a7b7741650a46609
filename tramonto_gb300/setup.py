"""Host set-up of a problem: stencil tables, bulk constants, synthetic inputs.

Restates the set-up the reference does once per run before its Newton loop:

* stencils (calc_stencils, src/dft_stencil.c:40-287) through the library's
  ``tgpu_make_stencil`` / ``tgpu_make_stencil_device`` (tramonto_gb300/csrc/stencils.cu);
* bulk FMT constants: rhobar_icomp / dphi_drb_bulk / chempot_FMT_hs
  (src/dft_thermo_hs.c:58-70, 138-153, 292-334) and the 1/R factors
  calc_InvR_params (:58-70);
* the mean-field constants calc_Avdw_att / chempot_att
  (src/dft_thermo_att.c:44-63, 86-99) with int_stencil_bulk
  (src/dft_energy_CLSintsten.c:43-69).

The synthetic geometries of the benchmark workloads (rough Lennard-Jones
12-3 wall, cylindrical pore with a Gaussian random field) are generated here
from seeds; the reference has no 12-3 wall, so its prefactor is fixed below.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import native
from .problem import BC_IN_BULK, BC_IN_WALL, BC_PERIODIC, DELTA, FMT1, FMT3, FMT4, THETA, UATT, Problem

PI = math.pi


def _lib():
    lib = native.load()
    for fn in (lib.tgpu_make_stencil, lib.tgpu_make_stencil_device):
        fn.restype = C.c_int
        fn.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                       C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.tgpu_wall_field_host.restype = C.c_int
    lib.tgpu_wall_field_host.argtypes = [C.c_void_p, C.c_void_p]
    lib.tgpu_lj_rmin.restype = C.c_double
    lib.tgpu_lj_rmin.argtypes = [C.c_double] * 4
    return lib


def _gpu_visible():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


def make_stencil(stype, ndim, esize, hs_diam=0.0, sigma=1.0, eps=1.0, rcut=0.0, rmin=0.0, with_hw=False,
                 device=None):
    """Stencil table (offsets [L][ndim], weights [L], per-corner weights [L][2^ndim] or None), built on the
    GPU (tgpu_make_stencil_device) or on the host (tgpu_make_stencil); the two builders give bit-identical
    tables.  device=None picks the GPU, when one is visible, for the 3-D tables whose quadrature outweighs
    the GPU's fixed cost: the attraction stencil and shells/balls wider than 5.5 nodes."""
    lib = _lib()
    if device is None:
        reach = (rcut if stype == UATT else 0.5 * hs_diam) / min(esize[:ndim])
        device = ndim == 3 and (stype == UATT or reach > 5.5) and _gpu_visible()
    fn = lib.tgpu_make_stencil_device if device else lib.tgpu_make_stencil
    es = (C.c_double * 3)(*(list(esize) + [0.0] * (3 - len(esize))))
    # the size query builds the table once; the second call builds it again into the arrays
    L = fn(stype, ndim, es, hs_diam, sigma, eps, rcut, rmin, 0, None, None, None, None)
    if L < 0:
        raise RuntimeError(f"tgpu_make_stencil{'_device' if device else ''} failed ({L})")
    off = np.zeros((L, ndim), np.int16)
    w = np.zeros(L)
    hw = np.zeros((L, 1 << ndim)) if with_hw else None
    L2 = fn(stype, ndim, es, hs_diam, sigma, eps, rcut, rmin, L, off.ctypes.data, w.ctypes.data,
            hw.ctypes.data if with_hw else None, None)
    assert L2 == L
    return off, w, hw


PAIR_LJ12_6_CS, PAIR_YUKAWA_CS, PAIR_EXP_CS, PAIR_SW = 0, 3, 4, 5
CORE_SIGMA, CORE_UMIN, CORE_UCSZERO, CORE_SIGTOUMIN = 0, 1, 2, 3
CORECONST_UCONST, CORECONST_ZERO = 0, 1
# Type_attr (MFPAIR_*) -> (Type_CoreATT_R, Type_CoreATT_CONST), as src/dft_defs_stencil.c:85-103 sets them
MFPAIR_CORES = {0: (CORE_UMIN, CORECONST_UCONST), 1: (CORE_SIGMA, CORECONST_ZERO), 2: (CORE_SIGMA, CORECONST_UCONST),
                3: (CORE_SIGTOUMIN, CORECONST_UCONST), 4: (CORE_UCSZERO, CORECONST_ZERO)}


class _PairPot(C.Structure):
    _fields_ = [("pot", C.c_int), ("core_r", C.c_int), ("core_const", C.c_int), ("sigma", C.c_double),
                ("eps_over_kT", C.c_double), ("rcut", C.c_double), ("rmin", C.c_double), ("rzero", C.c_double),
                ("kappa", C.c_double)]


def make_attraction_stencil(ndim, esize, pot=PAIR_LJ12_6_CS, core_r=CORE_UMIN, core_const=CORECONST_UCONST,
                            sigma=1.0, eps=1.0, rcut=2.5, rmin=0.0, rzero=0.0, kappa=0.0, with_hw=False, device=None):
    """Mean-field attraction stencil of any of the reference's attraction pair potentials and cores
    (tgpu_make_attraction_stencil); device as in make_stencil."""
    lib = _lib()
    lib.tgpu_make_attraction_stencil.restype = C.c_int
    lib.tgpu_make_attraction_stencil.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                                 C.c_void_p, C.c_void_p, C.c_void_p]
    if device is None:
        device = ndim == 3 and _gpu_visible()
    pp = _PairPot(int(pot), int(core_r), int(core_const), float(sigma), float(eps), float(rcut), float(rmin),
                  float(rzero), float(kappa))
    es = (C.c_double * 3)(*(list(esize) + [0.0] * (3 - len(esize))))
    L = lib.tgpu_make_attraction_stencil(C.byref(pp), ndim, es, int(bool(device)), 0, None, None, None, None)
    if L < 0:
        raise RuntimeError(f"tgpu_make_attraction_stencil failed ({L})")
    off = np.zeros((L, ndim), np.int16)
    w = np.zeros(L)
    hw = np.zeros((L, 1 << ndim)) if with_hw else None
    L2 = lib.tgpu_make_attraction_stencil(C.byref(pp), ndim, es, int(bool(device)), L, off.ctypes.data,
                                          w.ctypes.data, hw.ctypes.data if with_hw else None, None)
    assert L2 == L
    return off, w, hw


def lj_rmin(sigma, eps, rcut, esize0):
    return _lib().tgpu_lj_rmin(sigma, eps, rcut, esize0)


def fmt_dphi_bulk(functional, n):
    """dPhi/dn0..dn3 at a bulk state (vector terms vanish): FMT2 equals FMT1 there and FMT4 equals
    FMT3 (FMT1stDerivBulk_switch, src/dft_switch_FMT.c:98-120)."""
    n0, n1, n2, n3 = n
    a = 1.0 / (1.0 - n3)
    d0 = math.log(a)
    d1 = n2 * a
    if functional in (FMT3, FMT4):
        if n3 > 1e-10:
            lg = math.log(1.0 - n3)
            F = n3 + (1 - n3) ** 2 * lg
            F1 = n3 - 2 * (1 - n3) * lg
            G1 = 2.0 * (-a * a / n3 ** 3 + a ** 3 / n3 ** 2)
            f = F * a * a / (36 * PI * n3 * n3)
            f1 = (F1 * a * a / (n3 * n3) + F * G1) / (36 * PI)
            d2 = n1 * a + 3 * n2 * n2 * f
            d3 = n0 * a + n1 * n2 * a * a + n2 ** 3 * f1
        else:
            d2 = d3 = 0.0
    else:
        d2 = n1 * a + n2 * n2 * a * a / (8 * PI)
        d3 = n0 * a + n1 * n2 * a * a + n2 ** 3 * a ** 3 / (12 * PI)
    return np.array([d0, d1, d2, d3])


def bulk_constants(functional, hs_diam, rho_b, attraction=False, uatt_stencils=None, ncomp=None):
    """Bulk weighted densities, dPhi/dn, excess chemical potentials (reference set-up)."""
    hs_diam = np.asarray(hs_diam, float)
    rho_b = np.asarray(rho_b, float)
    nc = len(rho_b) if ncomp is None else ncomp
    inv_rad = 2.0 / hs_diam
    inv_4pir = inv_rad / (4 * PI)
    inv_4pirsq = inv_4pir * inv_rad
    rhobar = np.zeros(4)   # solution-vector order n3, n2, n1, n0
    for i in range(nc):
        vol = PI * hs_diam[i] ** 3 / 6.0
        area = PI * hs_diam[i] ** 2
        rhobar += np.array([vol * rho_b[i], area * rho_b[i], area * rho_b[i] * inv_4pir[i],
                            area * rho_b[i] * inv_4pirsq[i]])
    n = (rhobar[3], rhobar[2], rhobar[1], rhobar[0])
    dphi = fmt_dphi_bulk(functional, n)
    betamu_hs = np.zeros(nc)
    for i in range(nc):
        r = hs_diam[i] / 2.0
        sums = np.array([1.0, r, 4 * PI * r * r, 4 * PI / 3 * r ** 3])
        betamu_hs[i] = float(np.dot(dphi, sums))
    betamu_att = np.zeros(nc)
    avdw = np.zeros((nc, nc))
    if attraction:
        for i in range(nc):
            for j in range(nc):
                avdw[i, j] = float(np.sum(uatt_stencils[i + nc * j][1]))
        betamu_att = avdw @ rho_b
    return dict(inv_rad=inv_rad, inv_4pir=inv_4pir, inv_4pirsq=inv_4pirsq, rhobar_b=rhobar, dphi_bulk=dphi,
                betamu_hs_ex=betamu_hs, betamu_att=betamu_att, avdw=avdw)


def build_problem(ndim, nx, esize, bc, hs_diam, rho_b, functional=FMT1, attraction=False, sigma=None, eps=None,
                  rcut=None, vext=None, zero_density=None, vext_max=10.0, pair=None):
    """Assemble a Problem with generated stencils and bulk constants.  pair (optional) selects the attraction's
    pair potential and core: dict(pot=PAIR_*, core_r=CORE_*, core_const=CORECONST_*, kappa=...); the default is
    the cut-and-shifted LJ 12-6 with its core held at u(r_min) (Type_attr 0)."""
    nc = len(rho_b)
    st = {}
    for i in range(nc):
        st[(DELTA, i)] = make_stencil(DELTA, ndim, esize, hs_diam=hs_diam[i])
        st[(THETA, i)] = make_stencil(THETA, ndim, esize, hs_diam=hs_diam[i])
    uat = {}
    if attraction:
        for i in range(nc):
            for j in range(nc):
                rmin = lj_rmin(sigma[i][j], eps[i][j], rcut[i][j], esize[0])
                if pair is None:
                    uat[i + nc * j] = make_stencil(UATT, ndim, esize, sigma=sigma[i][j], eps=eps[i][j],
                                                   rcut=rcut[i][j], rmin=rmin)
                else:
                    uat[i + nc * j] = make_attraction_stencil(ndim, esize, sigma=sigma[i][j], eps=eps[i][j],
                                                              rcut=rcut[i][j], rmin=rmin, **pair)
                st[(UATT, i + nc * j)] = uat[i + nc * j]
    b = bulk_constants(functional, hs_diam, rho_b, attraction, uat, nc)
    N = int(np.prod(nx[:ndim]))
    if vext is None:
        vext = np.zeros((nc, N))
    if zero_density is None:
        zero_density = (vext >= vext_max).astype(np.int8)
    w = integration_weights(ndim, nx, esize, bc)
    betamu = np.log(np.asarray(rho_b, float)) + b["betamu_hs_ex"] + b["betamu_att"]
    return Problem(ndim=ndim, nx=tuple(nx), esize=tuple(esize), bc=tuple(bc), ncomp=nc, functional=functional,
                   attraction=int(attraction), att_in_a22=0, single_size=int(nc == 1), hard_surf=0, nlists_hw=1,
                   rho_b=np.asarray(rho_b, float), hs_diam=np.asarray(hs_diam, float), betamu_hs_ex=b["betamu_hs_ex"],
                   betamu_att=b["betamu_att"], inv_rad=b["inv_rad"], inv_4pir=b["inv_4pir"],
                   inv_4pirsq=b["inv_4pirsq"], fac_overlap=np.ones(nc), dphi_bulk=b["dphi_bulk"],
                   vext_max=vext_max, vext=np.ascontiguousarray(vext, float),
                   zero_density=np.ascontiguousarray(zero_density, np.int8), stencils=st,
                   w_fluid=np.tile(w, (nc, 1)), w_bulk=np.tile(w, (nc, 1)), rhobar_b=b["rhobar_b"], betamu=betamu)


def integration_weights(ndim, nx, esize, bc):
    """Per-node integration weights of a box without wall elements: Vol_el times the fraction of the
    node's 2^ndim elements that lie in the box (setup_integrals, src/dft_out_utils.c:179-270, with no
    surfaces), i.e. the trapezoid rule with half weights on non-periodic faces.  [N]"""
    w = np.ones(1)
    for d in range(ndim):
        f = np.ones(nx[d])
        if bc[d][0] != BC_PERIODIC:
            f[0] *= 0.5
        if bc[d][1] != BC_PERIODIC:
            f[-1] *= 0.5
        w = np.multiply.outer(f, w)          # slowest index last: [.., d] -> node = x + nx*(y + ny*z)
    return (w * float(np.prod(esize[:ndim]))).reshape(-1)


# ---- synthetic workloads ----------------------------------------------------

# 12-3 Lennard-Jones wall V(d) = eps_w * C * ((sigma/d)^12 - (sigma/d)^3), C chosen so that min V = -eps_w
LJ123_PREF = 1.0 / (0.75 * 4.0 ** (-1.0 / 3.0))


WALL_LJ93_CS, WALL_LJ123 = 0, 1


class _Wall(C.Structure):
    _fields_ = [("form", C.c_int), ("side", C.c_int), ("position", C.c_double), ("eps", C.c_double),
                ("sigma", C.c_double), ("cut", C.c_double), ("pattern", C.c_double), ("patches", C.c_int * 2),
                ("heights", C.c_void_p)]


class _WallField(C.Structure):
    _fields_ = [("ndim", C.c_int), ("nx", C.c_int * 3), ("esize", C.c_double * 3), ("nwalls", C.c_int),
                ("wall", _Wall * 2), ("vext_max", C.c_double)]


def wall_field_device(ndim, nx, esize, walls, vext_max):
    """The field of one or two planar walls computed on the GPU (tgpu_wall_field_host); walls are dicts
    with form, side, position, eps, sigma, cut, pattern and optional heights [py][pz]."""
    lib = _lib()
    f = _WallField()
    f.ndim = ndim
    for d in range(3):
        f.nx[d] = int(nx[d]) if d < ndim else 1
        f.esize[d] = float(esize[d]) if d < ndim else 0.0
    f.nwalls = len(walls)
    f.vext_max = float(vext_max)
    keep = []
    for k, w in enumerate(walls):
        o = f.wall[k]
        o.form, o.side = int(w["form"]), int(w.get("side", 0))
        o.position, o.eps, o.sigma = float(w["position"]), float(w["eps"]), float(w["sigma"])
        o.cut, o.pattern = float(w.get("cut", 0.0)), float(w.get("pattern", 0.0))
        h = w.get("heights")
        if h is not None:
            h = np.ascontiguousarray(h, np.float64)
            keep.append(h)
            o.patches[0], o.patches[1] = h.shape
            o.heights = h.ctypes.data
    out = np.empty(int(np.prod([nx[d] for d in range(ndim)])))
    st = lib.tgpu_wall_field_host(C.byref(f), out.ctypes.data_as(C.c_void_p))
    if st != 0:
        raise RuntimeError(f"tgpu_wall_field_host failed ({st})")
    return out


def rough_wall_vext(nx, esize, eps_w=1.0, kT=1.2, sigma_w=1.0, wall_x=1.0, patches=16, amplitude=0.5, seed=1234,
                    vext_max=10.0, device=None):
    """V_ext/kT of a rough 12-3 LJ wall normal to x.

    The surface sits at x = wall_x + h(y, z); h is i.i.d. uniform in
    [-amplitude, amplitude] sigma on a patches x patches grid over the periodic
    y-z plane (numpy PCG64 seeded with `seed`).  Nodes with d <= 0 or
    V >= vext_max are clipped to vext_max (zero-density rows).  The field is computed on the GPU
    (tgpu_wall_field_host) when one is visible or device=True, else with numpy.
    """
    rng = np.random.default_rng(seed)
    hpatch = rng.uniform(-amplitude, amplitude, size=(patches, patches))
    meta = dict(patches=patches, amplitude=amplitude, seed=seed, wall_x=wall_x, eps_w=eps_w,
                prefactor=LJ123_PREF, form="eps_w*C*((s/d)^12-(s/d)^3)/kT")
    if _gpu_visible() if device is None else device:
        wall = dict(form=WALL_LJ123, side=0, position=wall_x, eps=(eps_w / kT) * LJ123_PREF, sigma=sigma_w,
                    heights=hpatch)
        return wall_field_device(3, nx, esize, [wall], vext_max).reshape(1, -1), meta
    ny, nz = nx[1], nx[2]
    iy = (np.arange(ny) * patches) // ny
    iz = (np.arange(nz) * patches) // nz
    h = hpatch[iy][:, iz]                                  # [ny][nz]
    x = np.arange(nx[0]) * esize[0]
    d = x[None, None, :] - (wall_x + h.T[:, :, None])      # [nz][ny][nx]
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        s = np.where(d > 0, sigma_w / np.maximum(d, 1e-300), np.inf)
        v = (eps_w / kT) * LJ123_PREF * (s ** 12 - s ** 3)
    v = np.where((d <= 0) | (v >= vext_max) | ~np.isfinite(v), vext_max, v)
    return v.reshape(1, -1), meta


def lj93_wall_1d(dist, eps_w, sigma_w, cut_w, vext_max=10.0):
    """V_ext/kT of a planar cut-and-shifted LJ 9-3 wall and its derivatives in (eps_w, sigma_w).

    Vext_LJ9_3_CS (src/dft_vext_1D.c:42-56): with prefactor eps_w (the reference's
    Eps_wf*Rho_w, already over kT) and d the distance from the wall surface,
    V = eps_w (2 pi/3) sigma^3 [(2/15)((sigma/d)^9 - (sigma/cut)^9) - ((sigma/d)^3 - (sigma/cut)^3)]
    for d <= cut and 0 beyond.  Nodes with d <= 0 or V >= vext_max hold vext_max
    (zero-density rows, derivatives 0).  Returns (V, dV/deps_w, dV/dsigma_w).
    """
    d = np.asarray(dist, np.float64)
    inside = (d > 0) & (d <= cut_w)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        dd = np.where(inside, d, 1.0)
        a9 = 1.0 / dd ** 9 - 1.0 / cut_w ** 9
        a3 = 1.0 / dd ** 3 - 1.0 / cut_w ** 3
        pref = 2.0 * np.pi / 3.0
        shape = pref * ((2.0 / 15.0) * sigma_w ** 12 * a9 - sigma_w ** 6 * a3)
        dshape = pref * ((2.0 / 15.0) * 12.0 * sigma_w ** 11 * a9 - 6.0 * sigma_w ** 5 * a3)
    v = np.where(inside, eps_w * shape, 0.0)
    clamp = (d <= 0) | (v >= vext_max)
    v = np.where(clamp, vext_max, v)
    dv_de = np.where(inside & ~clamp, shape, 0.0)
    dv_ds = np.where(inside & ~clamp, eps_w * dshape, 0.0)
    return v, dv_de, dv_ds


def config2(n=128, esize=0.1, seed=1234, rho_b=0.6):
    """3-D FMT1 + WCA (eps=1, r_c=2.5, kT*=1.2) fluid at rho_b=0.6 next to a rough 12-3 LJ wall.

    Periodic in y and z; the wall side of x is IN_WALL, the far side IN_BULK."""
    nx = (n, n, n)
    es = (esize, esize, esize)
    kT = 1.2
    vext, meta = rough_wall_vext(nx, es, kT=kT, seed=seed)
    p = build_problem(3, nx, es, ((BC_IN_WALL, BC_IN_BULK), (BC_PERIODIC, BC_PERIODIC), (BC_PERIODIC, BC_PERIODIC)),
                      hs_diam=[1.0], rho_b=[rho_b], functional=FMT1, attraction=True, sigma=[[1.0]],
                      eps=[[1.0 / kT]], rcut=[[2.5]], vext=vext)
    meta.update(grid=list(nx), dx=esize, rho_b=rho_b, kT=kT, rcut=2.5, functional="FMT1", attraction="WCA LJ12-6")
    return p, meta


def config4(n=256, esize=0.08, seed=1234):
    """The configuration-2 fluid and wall at scale: 256^3 nodes, dx = 0.08 (attraction reach 31 nodes,
    1.4e5 stencil points).  The problem is built at rho_b = 0.6 and brought to rho_b = 0.70 by continuation
    (meta["ladder"]): at this resolution the contact density grows without bound as rho_b approaches ~0.71
    (max rho 2.0, 3.6, 8.3, 10.3 at rho_b 0.60, 0.65, 0.70, 0.705; n3 up to 0.67), and Newton (mixed or FP64,
    direct or by continuation in steps of 0.005) finds no solution at 0.71-0.75."""
    p, meta = config2(n=n, esize=esize, seed=seed, rho_b=0.6)
    meta["initial_cap"] = 1.0   # initial densities at most rho_b: rho_b exp(-V) in the wall's well overlaps (n3 > 1)
    meta["ladder"] = [0.6, 0.65, 0.7]
    return p, meta


def gaussian_random_field(nx, esize, corr_len=1.0, seed=4321):
    """Zero-mean, unit-variance Gaussian random field on the periodic box (numpy PCG64 `seed`): white noise filtered in
    Fourier space by exp(-k^2 corr_len^2 / 2), so the covariance falls as exp(-r^2 / (4 corr_len^2)). [nz][ny][nx]"""
    rng = np.random.default_rng(seed)
    white = rng.standard_normal(tuple(nx[::-1]))
    k = [np.fft.fftfreq(m, d=esize[0]) * 2 * PI for m in nx[::-1]]
    kk = k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2 + k[2][None, None, :] ** 2
    g = np.real(np.fft.ifftn(np.fft.fftn(white) * np.exp(-0.5 * kk * corr_len ** 2)))
    g -= g.mean()
    return g / g.std()


def pore_vext(nx, esize, hs_diam, eps_w, field, pore_radius=5.0, grf_amplitude=0.5, vext_max=10.0):
    """V_ext/kT of a cylindrical pore along z (axis at the box centre in x, y) and its eps_w derivative.

    The pore is the reference's own surface: a cylindrical pore (Surf_type 8, orientation z, radius
    pore_radius, unbounded length; surface_cylindricalPore3D_inSurfaceTest,
    src/dft_surfaces_cylindricalPore3D.c:38-96) whose wall acts through the cut-and-shifted 9-3 form of
    the distance to its surface (Ipot_wf_n 2, Vext_LJ9_3_CS, src/dft_vext_1D.c:42-56) with prefactor
    eps_w, sigma_wf = (sigma_i + 1)/2 and cut 2.5 sigma_wf — built on the GPU by the surface builder
    (tramonto_gb300.surfaces), zero-density nodes by the reference's element rule.  Species i also sees
    grf_amplitude * field.  Nodes whose field reaches vext_max hold vext_max (zero-density rows).  Returns
    (V [ncomp][N], dV/deps_w [ncomp][N], zero-density flags [ncomp][N])."""
    from . import surfaces
    nx = tuple(int(v) for v in nx)
    size = ((nx[0] - 1) * esize[0], (nx[1] - 1) * esize[1], nx[2] * esize[2])
    swf = [0.5 * (sig + 1.0) for sig in hs_diam]
    spec = surfaces.make_spec(
        3, size, esize, [(BC_IN_WALL, BC_IN_WALL), (BC_IN_WALL, BC_IN_WALL), (BC_PERIODIC, BC_PERIODIC)], len(hs_diam),
        [(0, (0.0, 0.0, 0.0))],
        [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=2, param=(pore_radius, 1.0e6, 0.0),
              ipot_wf=surfaces.VEXT_DIST_TO_SURF, type_vext=0, pot_id=surfaces.WALL1D_LJ93_CS, rho_w=1.0,
              sigma_wf=swf, eps_wf=[eps_w] * len(hs_diam), cut_wf=[2.5 * v for v in swf])],
        vext_max=vext_max, sigma_ff=list(hs_diam))
    nodes, _ = spec.mesh()
    if tuple(nodes) != nx:
        raise ValueError(f"pore mesh {nodes} differs from {nx}")
    shell, zero, _ = surfaces.surface_field(spec)
    g = grf_amplitude * np.asarray(field).reshape(-1)
    vs, ds, zs = [], [], []
    for i in range(len(hs_diam)):
        live = zero[i] == 0
        v = np.where(live, shell[i] + g, vext_max)
        z = ~live | (v >= vext_max)
        vs.append(np.where(z, vext_max, v))
        ds.append(np.where(z, 0.0, shell[i] / eps_w))
        zs.append(z)
    return np.array(vs), np.array(ds), np.array(zs, np.int8)


def config3(nx=(96, 96, 64), esize=0.1, seed=4321, pore_radius=5.0, eps_w=0.5):
    """3-D binary White-Bear (FMT3) hard spheres (sigma 1 and 0.5, rho_b 0.3 and 0.6) in a cylindrical pore
    of radius 5 along z (the reference's cylindrical pore surface, built on the GPU) with a soft 9-3 wall of
    strength eps_w; V_ext += 0.5 kT * Gaussian random field (correlation length 1).  Walls outside the box
    in x and y, periodic in z."""
    es = (esize,) * 3
    field = gaussian_random_field(nx, es, 1.0, seed)
    vext, dv_deps, zd = pore_vext(nx, es, [1.0, 0.5], eps_w, field, pore_radius)
    p = build_problem(3, nx, es, ((BC_IN_WALL, BC_IN_WALL), (BC_IN_WALL, BC_IN_WALL), (BC_PERIODIC, BC_PERIODIC)),
                      hs_diam=[1.0, 0.5], rho_b=[0.3, 0.6], functional=FMT3, vext=vext, zero_density=zd)
    return p, dict(grid=list(nx), dx=esize, seed=seed, pore_radius=pore_radius, rho_b=[0.3, 0.6], eps_w=eps_w,
                   functional="FMT3", field="0.5 kT Gaussian random field, correlation length 1",
                   shell="eps_w * 9-3 cut-and-shifted of the distance to the cylindrical pore surface (Ipot_wf_n 2), "
                         "sigma_wf=(sigma_i+1)/2, cut 2.5 sigma_wf, built on the GPU",
                   grf=field, dv_deps=dv_deps)


def slit_pore_vext(ndim, nx, esize, eps_w=1.0, sigma_w=1.0, cut_w=3.0, pattern=0.5, vext_max=10.0, device=None):
    """V_ext/kT of a slit pore: two planar cut-and-shifted 9-3 walls (the form of Vext_LJ9_3_CS,
    src/dft_vext_1D.c:42-56) with surfaces at the two x ends of the box; in 2-D the wall strength varies
    along the periodic y direction as eps_w (1 + pattern cos(2 pi y / L_y)) (a chemically patterned slit).
    Nodes with V >= vext_max or on a surface hold vext_max.  Returns [1][N] (node = ix + nx*iy).  Computed on
    the GPU (tgpu_wall_field_host) when one is visible or device=True, else with numpy."""
    L = (nx[0] - 1) * esize[0]
    if _gpu_visible() if device is None else device:
        pat = pattern if ndim >= 2 else 0.0
        walls = [dict(form=WALL_LJ93_CS, side=side, position=pos, eps=eps_w, sigma=sigma_w, cut=cut_w, pattern=pat)
                 for side, pos in ((0, 0.0), (1, L))]
        return wall_field_device(ndim, nx, esize, walls, vext_max).reshape(1, -1)
    x = np.arange(nx[0]) * esize[0]
    s1 = lj93_wall_1d(x, 1.0, sigma_w, cut_w, vext_max=np.inf)[0]
    s2 = lj93_wall_1d(L - x, 1.0, sigma_w, cut_w, vext_max=np.inf)[0]
    shape = s1 + s2
    surface = (x <= 0) | (x >= L)
    if ndim == 1:
        eps = np.array([eps_w])
    else:
        y = np.arange(nx[1]) * esize[1]
        eps = eps_w * (1.0 + pattern * np.cos(2 * PI * y / (nx[1] * esize[1])))
    v = eps[:, None] * shape[None, :]
    v = np.where(surface[None, :] | (v >= vext_max), vext_max, v)
    return v.reshape(1, -1)


def slit_pore(spec, rho_b=None):
    """One configuration-5 problem: FMT1 + WCA (eps = 1, r_c = 2.5, kT* = spec.get("kT", 1.2)) in a slit pore
    (spec from config5); walls beyond both x ends, periodic y in 2-D, of strength spec.get("eps_w", 1.0) (the
    zero-density rows follow from the field at that strength)."""
    ndim, nx, dx = spec["ndim"], tuple(spec["nx"]), spec["dx"]
    es = (dx,) * ndim
    kT = float(spec.get("kT", 1.2))
    bc = [(BC_IN_WALL, BC_IN_WALL)] + [(BC_PERIODIC, BC_PERIODIC)] * (ndim - 1)
    vext = slit_pore_vext(ndim, nx, es, eps_w=float(spec.get("eps_w", 1.0)))
    return build_problem(ndim, nx, es, tuple(bc), hs_diam=[1.0], rho_b=[spec["rho_b"] if rho_b is None else rho_b],
                         functional=FMT1, attraction=True, sigma=[[1.0]], eps=[[1.0 / kT]], rcut=[[2.5]], vext=vext)


def config5(seed=2024, n_problems=64):
    """Configuration 5: 64 independent slit-pore problems (numpy PCG64 `seed`): the first half 1-D with
    widths U(3, 40) sigma at dx = 0.01 (300-4000 nodes), the second half 2-D cross-sections of n x n nodes,
    n uniform in [100, 400], at dx = 0.05; each with its own bulk density U(0.05, 0.8)."""
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n_problems):
        if k < n_problems // 2:
            width = rng.uniform(3.0, 40.0)
            n = int(round(width / 0.01)) + 1
            spec = dict(ndim=1, nx=(n, 1, 1), dx=0.01, width=(n - 1) * 0.01)
        else:
            n = int(rng.integers(100, 401))
            spec = dict(ndim=2, nx=(n, n, 1), dx=0.05, width=(n - 1) * 0.05)
        spec["rho_b"] = float(rng.uniform(0.05, 0.8))
        specs.append(spec)
    return specs


def initial_state(solver, p: Problem, max_enhancement=None):
    """Density rho_b*exp(-V) (0 in walls; at most max_enhancement*rho_b when given); weighted densities
    and mean field from their own sums."""
    N = p.nnodes
    x = np.zeros((p.nunk, N))
    for c in range(p.ncomp):
        v = p.vext[c]
        rho = p.rho_b[c] * np.exp(-np.minimum(v, 50.0))
        if max_enhancement is not None:
            rho = np.minimum(rho, max_enhancement * p.rho_b[c])
        rho[p.zero_density[c] != 0] = 0.0
        rho[v >= p.vext_max] = 0.0
        x[p.first_rho + c] = np.maximum(rho, 0.0)
    # R = -x + sums on the weighted-density and mean-field rows: two passes set
    # the independent unknowns to their sums, then the dependent local copies
    for _ in range(2):
        R = solver.fill(x, mode=1)
        x[p.first_rb:] += R[p.first_rb:]
    return x
