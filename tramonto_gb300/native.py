"""ctypes binding of libtramonto_gpu.so and the host-side solver object.

:class:`Solver` mirrors, for one problem, the operations the reference's
Newton driver performs through its linear-problem manager:

=====================  ==========================================================
``fill(x, mode)``      fill_resid_and_matrix_control (src/dft_fill_control.c:39)
``jv(v)``              dft_linprobmgr_applymatrix (src/dft_BasicLinProbMgr.cpp)
``schur(v2)``          dft_Schur_Epetra_Operator::Apply (src/dft_Schur_Epetra_Operator.cpp:86)
``solve(b)``           dft_linprobmgr_setupsolver + dft_linprobmgr_solve
                       (src/dft_HardSphereLinProbMgr.cpp:345-428)
``newton(x)``          newton_solver (src/dft_newton.c:131-198)
=====================  ==========================================================

Arrays are numpy ``[unknown][node]`` float64 (host) or torch CUDA tensors
(``*_device`` methods).  Every call goes through the C ABI of
include/tramonto_gpu.h; there is no CPU fallback: if the library or a GPU is
missing the constructor raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .problem import Problem

TGPU_OK = 0
TGPU_ERR_DOMAIN = -7
FP64, FP32, BF16X3, FP16TC, FP64_FFT = 0, 1, 2, 3, 4
FILL_FP64, FILL_FP32, FILL_REFINED, FILL_MIXED, FILL_FF, FILL_MIXED_FF, FILL_FFT, FILL_MIXED_FFT = 0, 1, 2, 3, 4, 5, 6, 7
TIME_FFT32 = 16   # time_stencil_sum: the FP32 FFT convolution
JAC_REFERENCE, JAC_EXACT = 0, 1
STATUS = {0: "ok", -1: "bad argument", -2: "CUDA error", -3: "call out of order", -4: "unsupported",
          -5: "no convergence", -6: "non-finite values", -7: "domain error"}


class TgpuError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Geometry(C.Structure):
    _fields_ = [
        ("ndim", C.c_int), ("nx", C.c_int * 3), ("esize", C.c_double * 3), ("bc", (C.c_int * 2) * 3),
        ("ncomp", C.c_int), ("functional", C.c_int), ("attraction", C.c_int), ("att_in_a22", C.c_int),
        ("single_size", C.c_int), ("hard_surf", C.c_int), ("nlists_hw", C.c_int),
        ("rho_b", C.c_double * 4), ("betamu_hs_ex", C.c_double * 4), ("betamu_att", C.c_double * 4),
        ("inv_rad", C.c_double * 4), ("inv_4pir", C.c_double * 4), ("inv_4pirsq", C.c_double * 4),
        ("fac_overlap", C.c_double * 4), ("dphi_bulk", C.c_double * 4), ("vext_max", C.c_double),
        ("interface", C.c_int), ("rho_b_lbb", C.c_double * 4), ("rho_b_rtf", C.c_double * 4),
        ("dphi_lbb", C.c_double * 4), ("dphi_rtf", C.c_double * 4), ("betamu", C.c_double * 4),
        ("pin", C.c_int), ("pin_node", C.c_long), ("pin_value", C.c_double),
    ]


class Stats(C.Structure):
    _fields_ = [("fill_ms", C.c_double), ("schur_ms", C.c_double), ("conv_ms", C.c_double), ("gmres_ms", C.c_double),
                ("schur_applies", C.c_long), ("conv_launches", C.c_long), ("kernel_launches", C.c_long),
                ("fp64_refreshes", C.c_long)]


_LIB = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the CUDA library; raises when it is missing (no silent fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run tramonto_gb300.build.build() (nvcc, sm_103a) first")
        _build.build()
    lib = C.CDLL(path)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.tgpu_last_error.restype = C.c_char_p
    sigs = {
        "tgpu_create": [C.POINTER(Geometry), C.c_int, C.POINTER(vp)],
        "tgpu_destroy": [vp],
        "tgpu_set_stencil": [vp, C.c_int, C.c_int, C.c_int, vp, vp, vp],
        "tgpu_set_zones": [vp, C.c_int, vp, vp], "tgpu_set_1d_boundary": [vp, C.c_int],
        "tgpu_set_fft_threshold": [vp, C.c_int],
        "tgpu_set_fft32_policy": [vp, C.c_int],
        "tgpu_fft32_choice": [vp, C.c_int, C.c_int, ip, dp],
        "tgpu_set_tc_wait_limit": [vp, C.c_long],
        "tgpu_time_fft_pass": [vp, C.c_int, C.c_int, C.c_int, dp, C.POINTER(C.c_long), C.POINTER(C.c_long)],
        "tgpu_pass_timer_begin": [vp],
        "tgpu_pass_timer_end": [vp, C.POINTER(C.c_long), dp, dp, C.POINTER(C.c_long)],
        "tgpu_set_zone_stencil": [vp, C.c_int, C.c_int, C.c_int, C.c_int, vp, vp, vp],
        "tgpu_set_vext": [vp, vp], "tgpu_set_zero_density": [vp, vp], "tgpu_set_hard_wall": [vp, vp, vp],
        "tgpu_finalize": [vp], "tgpu_set_precision": [vp, C.c_int], "tgpu_set_stream": [vp, vp],
        "tgpu_set_jacobian_form": [vp, C.c_int],
        "tgpu_set_fill_arithmetic": [vp, C.c_int, C.c_double, C.c_double],
        "tgpu_sizes": [vp, C.POINTER(C.c_long), ip, ip],
        "tgpu_fill": [vp, vp, vp, C.c_int], "tgpu_fill_device": [vp, vp, vp, C.c_int],
        "tgpu_jv": [vp, vp, vp], "tgpu_jv_device": [vp, vp, vp],
        "tgpu_jtv": [vp, vp, vp], "tgpu_jtv_device": [vp, vp, vp],
        "tgpu_adjoint_solve": [vp, vp, vp, C.c_double, C.c_int, ip, dp],
        "tgpu_adjoint_solve_device": [vp, vp, vp, C.c_double, C.c_int, ip, dp],
        "tgpu_schur_apply": [vp, vp, vp], "tgpu_schur_apply_device": [vp, vp, vp],
        "tgpu_schur_rhs_device": [vp, vp, vp], "tgpu_schur_x1_device": [vp, vp, vp, vp],
        "tgpu_solve": [vp, vp, vp, C.c_double, C.c_int, ip, dp],
        "tgpu_solve_device": [vp, vp, vp, C.c_double, C.c_int, ip, dp],
        "tgpu_newton": [vp, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, ip, dp],
        "tgpu_newton_device": [vp, vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_int, ip, dp],
        "tgpu_newton_solve": [vp, vp, C.c_double, C.c_int, C.c_double, C.c_int, C.c_double, ip, dp, ip],
        "tgpu_newton_solve_device": [vp, vp, C.c_double, C.c_int, C.c_double, C.c_int, C.c_double, ip, dp, ip],
        "tgpu_time_stencil_sum": [vp, C.c_int, C.c_int, C.c_int, C.c_int, dp],
        "tgpu_get_stats": [vp, C.POINTER(Stats)], "tgpu_reset_stats": [vp],
        "tgpu_set_integration": [vp, vp, vp, vp, vp],
        "tgpu_set_bulk_state": [vp, vp, vp, vp, vp],
        "tgpu_objectives": [vp, vp, dp, dp], "tgpu_objectives_device": [vp, vp, dp, dp],
        "tgpu_objective_grad_device": [vp, vp, C.c_int, C.c_int, vp, vp],
        "tgpu_grad_vext_device": [vp, vp, C.c_int, C.c_int, C.c_double, C.c_int, vp, ip],
        "tgpu_grad_omega_vext": [vp, vp, C.c_double, C.c_int, vp, ip],
        "tgpu_grad_gamma_vext": [vp, vp, C.c_int, C.c_double, C.c_int, vp, ip],
        "tgpu_grad_epsw": [vp, vp, C.c_int, C.c_int, vp, C.c_double, C.c_int, dp, ip],
        "tgpu_surface_mesh": [vp, ip, ip],
        "tgpu_surface_field_host": [vp, vp, vp, vp], "tgpu_surface_field_device": [vp, vp, vp, vp],
        "tgpu_surface_rough_table": [vp, vp],
    }
    for name, args in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _LIB = lib
    return lib


def _check(st, lib, ok=(TGPU_OK,)):
    if st not in ok:
        raise TgpuError(st, lib.tgpu_last_error().decode())
    return st


def geometry(p: Problem) -> Geometry:
    g = Geometry()
    g.ndim = p.ndim
    for d in range(3):
        g.nx[d] = int(p.nx[d]) if d < p.ndim else 1
        g.esize[d] = float(p.esize[d]) if d < p.ndim else 0.0
        for k in range(2):
            g.bc[d][k] = int(p.bc[d][k]) if d < p.ndim else 0
    g.ncomp, g.functional, g.attraction = p.ncomp, p.functional, p.attraction
    g.att_in_a22, g.single_size, g.hard_surf, g.nlists_hw = p.att_in_a22, p.single_size, p.hard_surf, p.nlists_hw
    for name in ("rho_b", "betamu_hs_ex", "betamu_att", "inv_rad", "inv_4pir", "inv_4pirsq", "fac_overlap"):
        arr = getattr(g, name)
        for i, v in enumerate(np.asarray(getattr(p, name), np.float64)[:4]):
            arr[i] = float(v)
    for i in range(4):
        g.dphi_bulk[i] = float(p.dphi_bulk[i])
    g.vext_max = float(p.vext_max)
    g.interface = int(p.interface)
    if p.interface:
        for name, src in (("rho_b_lbb", p.rho_b_lbb), ("rho_b_rtf", p.rho_b_rtf), ("dphi_lbb", p.dphi_lbb),
                          ("dphi_rtf", p.dphi_rtf), ("betamu", p.betamu_if)):
            arr = getattr(g, name)
            for i, v in enumerate(np.asarray(src, np.float64)[:4]):
                arr[i] = float(v)
    g.pin = int(p.pin_node >= 0)
    g.pin_node = int(max(p.pin_node, 0))
    g.pin_value = float(p.pin_value)
    return g


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def mesh_coarsened(p: Problem) -> bool:
    """Flags that change the residual, read as the fill reads them: with Mesh_coarsening on and walls present, or
    with L1D_bc (src/dft_fill_main.c:120)."""
    if p.zone_flag is None:
        return False
    return bool((p.mesh_coarsening and p.nwall > 0) or p.l1d_bc)


def _rhobar_bulk(p: Problem):
    """Rhobar_b beyond IN_BULK boundaries in solution order; [LBB, RTF] with a phase interface (rhobar_icomp,
    src/dft_thermo_hs.c:292-311)."""
    nrb = p.nrb
    if p.interface != 2:
        return np.ascontiguousarray(np.asarray(p.rhobar_bc, np.float64)[:nrb])
    out = np.zeros((2, nrb))
    for side, rho in enumerate((p.rho_b_lbb, p.rho_b_rtf)):
        for ic in range(p.ncomp):
            d = float(p.hs_diam[ic])
            vol, area = np.pi * d * d * d / 6.0, np.pi * d * d
            f = float(p.fac_overlap[ic]) * float(rho[ic])
            out[side, :4] += [f * vol, f * area, f * area * p.inv_4pir[ic], f * area * p.inv_4pirsq[ic]]
    return np.ascontiguousarray(out.reshape(-1))


class Solver:
    """One problem resident on one GPU (see module doc)."""

    def __init__(self, p: Problem, device: int = 0, precision: int = FP64):
        self.lib = lib = load()
        self.p = p
        self.h = C.c_void_p()
        _check(lib.tgpu_create(C.byref(geometry(p)), device, C.byref(self.h)), lib)
        try:
            for (t, idx), (off, w, hw) in sorted(p.stencils.items()):
                off = np.ascontiguousarray(off, np.int16)
                w = np.ascontiguousarray(w, np.float64)
                hwp = None
                if hw is not None and p.hard_surf:
                    hw = np.ascontiguousarray(hw, np.float64)
                    hwp = _ptr(hw)
                _check(lib.tgpu_set_stencil(self.h, t, idx, len(w), _ptr(off), _ptr(w), hwp), lib)
            vext = np.ascontiguousarray(p.vext, np.float64)
            _check(lib.tgpu_set_vext(self.h, _ptr(vext)), lib)
            zd = np.ascontiguousarray(p.zero_density, np.int8)
            _check(lib.tgpu_set_zero_density(self.h, _ptr(zd)), lib)
            if p.hard_surf:
                bn = np.ascontiguousarray(p.boundary_nodes, np.int32)
                fm = np.ascontiguousarray(p.fluid_masks, np.int16)
                _check(lib.tgpu_set_hard_wall(self.h, _ptr(bn), _ptr(fm)), lib)
            if mesh_coarsened(p):
                # the fill reads the zones only with Mesh_coarsening on and walls present
                # (src/dft_fill_main.c:120); the Jacobian is the residual's own derivative
                flag = np.ascontiguousarray(p.zone_flag, np.int32)
                rbb = _rhobar_bulk(p)
                if p.l1d_bc:
                    _check(lib.tgpu_set_1d_boundary(self.h, int(p.dim_1dbc)), lib)
                _check(lib.tgpu_set_zones(self.h, int(max(p.nzone, 1)), _ptr(flag), _ptr(rbb)), lib)
                for zone, tabs in sorted(p.zone_stencils.items()):
                    for (t, idx), (off, w, hw) in sorted(tabs.items()):
                        off = np.ascontiguousarray(off, np.int16)
                        w = np.ascontiguousarray(w, np.float64)
                        hwp = None
                        if hw is not None and p.hard_surf:
                            hw = np.ascontiguousarray(hw, np.float64)
                            hwp = _ptr(hw)
                        _check(lib.tgpu_set_zone_stencil(self.h, zone, t, idx, len(w), _ptr(off), _ptr(w), hwp), lib)
            _check(lib.tgpu_finalize(self.h), lib)
            self.set_precision(precision)
            if p.w_fluid is not None:
                self.set_integration(p.w_fluid, p.w_bulk, p.rhobar_b, p.betamu)
        except Exception:
            self.close()
            raise
        self.N = p.nnodes
        self.shape = (p.nunk, self.N)

    # ---- lifecycle
    def close(self):
        if self.h:
            self.lib.tgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_vext(self, vext):
        """Replace V_ext/kT ([ncomp][N]); nodes equal to vext_max stay zero-density rows."""
        v = self._host(vext, (self.p.ncomp, self.N))
        _check(self.lib.tgpu_set_vext(self.h, _ptr(v)), self.lib)

    def set_bulk(self, rho_b):
        """Move the bulk state (chemical potential) to the bulk densities rho_b: the bulk constants are
        recomputed as at set-up (tgpu_set_bulk_state) and the objectives' constants follow."""
        from . import setup
        from .problem import UATT
        p = self.p
        rho_b = np.asarray(rho_b, np.float64).reshape(p.ncomp)
        uat = {k[1]: v for k, v in p.stencils.items() if k[0] == UATT} if p.attraction else None
        b = setup.bulk_constants(p.functional, p.hs_diam, rho_b, bool(p.attraction), uat, p.ncomp)
        hs, att = np.ascontiguousarray(b["betamu_hs_ex"], np.float64), np.ascontiguousarray(b["betamu_att"], np.float64)
        dphi = np.ascontiguousarray(b["dphi_bulk"], np.float64)
        _check(self.lib.tgpu_set_bulk_state(self.h, _ptr(rho_b), _ptr(hs), _ptr(att), _ptr(dphi)), self.lib)
        p.rho_b, p.betamu_hs_ex, p.betamu_att, p.dphi_bulk = rho_b.copy(), hs, att, dphi
        if p.w_fluid is not None:
            p.rhobar_b = b["rhobar_b"]
            p.betamu = np.log(rho_b) + hs + att
            self.set_integration(p.w_fluid, p.w_bulk, p.rhobar_b, p.betamu)

    def set_chemical_potential(self, betamu):
        """Set beta mu_i directly, for problems without bulk boundaries (pores): the Euler-Lagrange rows
        hold -(ln rho_b + betamu_hs_ex + betamu_att) = -beta mu (src/dft_fill_EL.c:401-410), and rho_b
        itself is read only at bulk boundaries and by the objectives' bulk terms.  rho_b is kept and
        betamu_att takes up the change (tgpu_set_bulk_state); Omega_s and Gamma_ex, which compare with
        the bulk at rho_b, are then not those of the new state, the absolute adsorption is."""
        from .problem import BC_IN_BULK
        p = self.p
        if any(BC_IN_BULK in tuple(p.bc[d]) for d in range(p.ndim)):
            raise ValueError("beta mu can be set directly only without bulk boundaries")
        bm = np.asarray(betamu, np.float64).reshape(p.ncomp)
        rho_b = np.ascontiguousarray(p.rho_b, np.float64)
        hs = np.ascontiguousarray(p.betamu_hs_ex, np.float64)
        att = np.ascontiguousarray(bm - np.log(rho_b) - hs, np.float64)
        dphi = np.ascontiguousarray(p.dphi_bulk, np.float64)
        _check(self.lib.tgpu_set_bulk_state(self.h, _ptr(rho_b), _ptr(hs), _ptr(att), _ptr(dphi)), self.lib)
        p.betamu_att = att

    def set_integration(self, w_fluid, w_bulk, rhobar_b, betamu):
        """Integration weights ([ncomp][N] each), bulk n3 n2 n1 n0 and betamu of the objectives."""
        nc = self.p.ncomp
        wf = np.ascontiguousarray(w_fluid, np.float64).reshape(nc, -1)
        wb = np.ascontiguousarray(w_bulk, np.float64).reshape(nc, -1)
        rb = np.ascontiguousarray(rhobar_b, np.float64).reshape(4)
        bm = np.ascontiguousarray(betamu, np.float64).reshape(nc)
        _check(self.lib.tgpu_set_integration(self.h, _ptr(wf), _ptr(wb), _ptr(rb), _ptr(bm)), self.lib)

    def objectives(self, x):
        """(Omega_s, Gamma_ex[ncomp]) of the state x (host array)."""
        x = self._host(x, self.shape)
        om = C.c_double(0.0)
        gam = np.zeros(self.p.ncomp)
        _check(self.lib.tgpu_objectives(self.h, _ptr(x), C.byref(om), gam.ctypes.data_as(C.POINTER(C.c_double))), self.lib)
        return om.value, gam

    def objective_grad(self, x, kind=0, icomp=0):
        """(dF/dx, dF/dV_ext at fixed x) of Omega_s (kind 0) or Gamma_ex[icomp] (kind 1); host arrays."""
        import torch
        xt = torch.tensor(self._host(x, self.shape), dtype=torch.float64, device="cuda")
        gx = torch.empty_like(xt)
        gv = torch.empty((self.p.ncomp, self.N), dtype=torch.float64, device="cuda")
        _check(self.lib.tgpu_objective_grad_device(self.h, self._dptr(xt), kind, icomp, self._dptr(gx),
                                                   self._dptr(gv)), self.lib)
        torch.cuda.synchronize()
        return gx.cpu().numpy(), gv.cpu().numpy()

    def grad_vext(self, x, kind=0, icomp=0, tol=1e-12, max_iter=500):
        """dF/dV_ext ([ncomp][N]) of Omega_s (kind 0) or Gamma_ex[icomp] (kind 1) at the converged state x."""
        x = self._host(x, self.shape)
        out = np.empty((self.p.ncomp, self.N))
        it = C.c_int(0)
        if kind == 0:
            st = self.lib.tgpu_grad_omega_vext(self.h, _ptr(x), tol, max_iter, _ptr(out), C.byref(it))
        else:
            st = self.lib.tgpu_grad_gamma_vext(self.h, _ptr(x), icomp, tol, max_iter, _ptr(out), C.byref(it))
        _check(st, self.lib)
        return out

    def grad_param(self, x, dvext_dp, kind=0, icomp=0, tol=1e-12, max_iter=500):
        """dF/dp for a wall parameter p entering through V_ext (dvext_dp = dV_ext/dp, [ncomp][N])."""
        x = self._host(x, self.shape)
        dv = self._host(dvext_dp, (self.p.ncomp, self.N))
        val = C.c_double(0.0)
        it = C.c_int(0)
        _check(self.lib.tgpu_grad_epsw(self.h, _ptr(x), kind, icomp, _ptr(dv), tol, max_iter, C.byref(val),
                                       C.byref(it)), self.lib)
        return val.value

    def set_precision(self, precision: int):
        _check(self.lib.tgpu_set_precision(self.h, int(precision)), self.lib)

    def set_jacobian_form(self, form: int):
        """FMT second derivatives in J, J^T and Schur products: JAC_REFERENCE (the reference's tables,
        default) or JAC_EXACT (the Hessian of the energy density); they differ for FMT2 and FMT4 only."""
        _check(self.lib.tgpu_set_jacobian_form(self.h, int(form)), self.lib)

    def set_fill_arithmetic(self, arith: int, tau: float = 0.0, switch_norm: float = 0.0):
        """Residual arithmetic: FILL_FP64, FILL_FP32, FILL_REFINED, FILL_MIXED, FILL_FF, FILL_MIXED_FF,
        FILL_FFT or FILL_MIXED_FFT (see include/tramonto_gpu.h)."""
        _check(self.lib.tgpu_set_fill_arithmetic(self.h, int(arith), float(tau), float(switch_norm)), self.lib)

    def set_fft_threshold(self, min_points: int):
        """Stencils of at least min_points points take the FFT in FILL_FFT; < 0: the cost model decides."""
        _check(self.lib.tgpu_set_fft_threshold(self.h, int(min_points)), self.lib)

    def set_fft32_policy(self, policy: int):
        """FP32 sums as FP32 FFT convolutions: -1 timed choice (default), 0 never, 1 always."""
        _check(self.lib.tgpu_set_fft32_policy(self.h, int(policy)), self.lib)

    def fft32_choice(self, stype: int, index: int = 0) -> dict:
        """The FP32 sums' timed choice for a stencil: forward / transposed (1 FFT, -1 direct, 0 undecided) and the
        timed milliseconds per sum behind them."""
        ch = (C.c_int * 2)()
        ms = (C.c_double * 4)()
        _check(self.lib.tgpu_fft32_choice(self.h, stype, index, ch, ms), self.lib)
        return {"forward": ch[0], "transposed": ch[1], "ms_direct_fwd": ms[0], "ms_fft_fwd": ms[1],
                "ms_direct_tr": ms[2], "ms_fft_tr": ms[3]}

    def set_stream(self, stream_handle: int):
        _check(self.lib.tgpu_set_stream(self.h, C.c_void_p(stream_handle)), self.lib)

    # ---- host-array entry points
    def _host(self, a, shape):
        a = np.ascontiguousarray(a, np.float64)
        if a.size != int(np.prod(shape)):
            raise ValueError(f"expected {shape}, got {a.shape}")
        return a

    def fill(self, x, mode: int = 0):
        x = self._host(x, self.shape)
        R = np.empty(self.shape)
        _check(self.lib.tgpu_fill(self.h, _ptr(x), _ptr(R), mode), self.lib)
        return R

    def jv(self, v):
        v = self._host(v, self.shape)
        out = np.empty(self.shape)
        _check(self.lib.tgpu_jv(self.h, _ptr(v), _ptr(out)), self.lib)
        return out

    def jtv(self, w):
        w = self._host(w, self.shape)
        out = np.empty(self.shape)
        _check(self.lib.tgpu_jtv(self.h, _ptr(w), _ptr(out)), self.lib)
        return out

    def adjoint_solve(self, g, tol=1e-12, max_iter=500):
        """Solve J^T lambda = g (host arrays [nunk][N]); returns (lambda, GMRES iterations, relative residual)."""
        g = self._host(g, self.shape)
        lam = np.empty(self.shape)
        it, rr = C.c_int(0), C.c_double(0.0)
        st = self.lib.tgpu_adjoint_solve(self.h, _ptr(g), _ptr(lam), tol, max_iter, C.byref(it), C.byref(rr))
        _check(st, self.lib, ok=(0, -5))
        return lam, it.value, rr.value

    def schur(self, v2):
        shape2 = (self.p.ncomp, self.N)
        v2 = self._host(v2, shape2)
        out = np.empty(shape2)
        _check(self.lib.tgpu_schur_apply(self.h, _ptr(v2), _ptr(out)), self.lib)
        return out

    def solve(self, b, tol=1e-10, max_iter=500):
        b = self._host(b, self.shape)
        dx = np.empty(self.shape)
        it, rr = C.c_int(0), C.c_double(0.0)
        st = self.lib.tgpu_solve(self.h, _ptr(b), _ptr(dx), tol, max_iter, C.byref(it), C.byref(rr))
        _check(st, self.lib, ok=(0, -5))
        return dx, it.value, rr.value

    def newton(self, x0, rel_tol=1e-3, abs_tol=1e-8, update_floor=0.1, max_iter=50, lin_tol=1e-10, lin_max_iter=500,
               allow_noconv=False):
        x = np.array(x0, np.float64, copy=True, order="C")
        it, rn = C.c_int(0), C.c_double(0.0)
        st = self.lib.tgpu_newton(self.h, _ptr(x), rel_tol, abs_tol, update_floor, max_iter, lin_tol, lin_max_iter,
                                  C.byref(it), C.byref(rn))
        _check(st, self.lib, ok=(0, -5) if allow_noconv else (0,))
        return x, it.value, rn.value

    # ---- device entry points (torch CUDA tensors, float64, contiguous)
    @staticmethod
    def _dptr(t):
        assert t.is_cuda and t.is_contiguous() and str(t.dtype) == "torch.float64"
        return C.c_void_p(t.data_ptr())

    def fill_device(self, x, R, mode: int = 0):
        _check(self.lib.tgpu_fill_device(self.h, self._dptr(x), self._dptr(R), mode), self.lib)

    def jv_device(self, v, out):
        _check(self.lib.tgpu_jv_device(self.h, self._dptr(v), self._dptr(out)), self.lib)

    def jtv_device(self, w, out):
        _check(self.lib.tgpu_jtv_device(self.h, self._dptr(w), self._dptr(out)), self.lib)

    def adjoint_solve_device(self, g, lam, tol=1e-12, max_iter=500):
        it, rr = C.c_int(0), C.c_double(0.0)
        st = self.lib.tgpu_adjoint_solve_device(self.h, self._dptr(g), self._dptr(lam), tol, max_iter, C.byref(it),
                                                C.byref(rr))
        _check(st, self.lib, ok=(0, -5))
        return it.value, rr.value

    def schur_device(self, v2, y2):
        _check(self.lib.tgpu_schur_apply_device(self.h, self._dptr(v2), self._dptr(y2)), self.lib)

    def solve_device(self, b, dx, tol=1e-10, max_iter=500):
        it, rr = C.c_int(0), C.c_double(0.0)
        st = self.lib.tgpu_solve_device(self.h, self._dptr(b), self._dptr(dx), tol, max_iter, C.byref(it), C.byref(rr))
        _check(st, self.lib, ok=(0, -5))
        return it.value, rr.value

    def newton_device(self, x, rel_tol=1e-3, abs_tol=1e-8, update_floor=0.1, max_iter=50, lin_tol=1e-10,
                      lin_max_iter=500, allow_noconv=False):
        it, rn = C.c_int(0), C.c_double(0.0)
        st = self.lib.tgpu_newton_device(self.h, self._dptr(x), rel_tol, abs_tol, update_floor, max_iter, lin_tol,
                                         lin_max_iter, C.byref(it), C.byref(rn))
        _check(st, self.lib, ok=(0, -5) if allow_noconv else (0,))
        return it.value, rn.value

    def newton_solve(self, x0, resid_tol=1e-8, max_iter=50, lin_tol=1e-8, lin_max_iter=300, update_floor=0.1,
                     allow_noconv=False, inplace=False):
        """Newton to ||R||_2 <= resid_tol (host arrays); returns (x, iterations, ||R||_2, GMRES iterations).
        inplace=True solves in x0 itself (a C-contiguous float64 array, e.g. a view of pinned host memory)."""
        if inplace:
            if not (isinstance(x0, np.ndarray) and x0.dtype == np.float64 and x0.flags.c_contiguous
                    and x0.flags.writeable and x0.size == self.p.nunk * self.p.nnodes):
                raise ValueError("inplace needs a writable C-contiguous float64 array of the state's size")
            x = x0
        else:
            x = np.array(x0, np.float64, copy=True, order="C")
        it, rn, li = C.c_int(0), C.c_double(0.0), C.c_int(0)
        st = self.lib.tgpu_newton_solve(self.h, _ptr(x), resid_tol, max_iter, lin_tol, lin_max_iter, update_floor,
                                        C.byref(it), C.byref(rn), C.byref(li))
        _check(st, self.lib, ok=(0, -5) if allow_noconv else (0,))
        return x, it.value, rn.value, li.value

    def newton_solve_device(self, x, resid_tol=1e-8, max_iter=50, lin_tol=1e-8, lin_max_iter=300,
                            update_floor=0.1, allow_noconv=False):
        it, rn, li = C.c_int(0), C.c_double(0.0), C.c_int(0)
        st = self.lib.tgpu_newton_solve_device(self.h, self._dptr(x), resid_tol, max_iter, lin_tol, lin_max_iter,
                                               update_floor, C.byref(it), C.byref(rn), C.byref(li))
        _check(st, self.lib, ok=(0, -5) if allow_noconv else (0,))
        return it.value, rn.value, li.value

    def pass_timer_begin(self):
        """Start timing every FP32 y/z FFT pass launch (CUDA events on its stream)."""
        _check(self.lib.tgpu_pass_timer_begin(self.h), self.lib)

    def pass_timer_end(self):
        """Stop the pass timer: (launches, summed ms, algorithmic bytes, transforms)."""
        nl, nt = C.c_long(), C.c_long()
        ms, by = C.c_double(), C.c_double()
        _check(self.lib.tgpu_pass_timer_end(self.h, C.byref(nl), C.byref(ms), C.byref(by), C.byref(nt)), self.lib)
        return int(nl.value), float(ms.value), float(by.value), int(nt.value)

    def time_fft_pass(self, precision, axis=1, reps=20):
        """Device milliseconds of one y (axis 1) or z (axis 2) pass of the FFT sums, the half spectrum's size and the
        real box's size."""
        ms, pts, real = C.c_double(0.0), C.c_long(0), C.c_long(0)
        _check(self.lib.tgpu_time_fft_pass(self.h, precision, axis, reps, C.byref(ms), C.byref(pts), C.byref(real)),
               self.lib)
        return ms.value, pts.value, real.value

    def time_stencil_sum(self, stype, index, precision, reps=5) -> float:
        """Device milliseconds of one forward stencil sum (benchmark hook)."""
        ms = C.c_double(0.0)
        _check(self.lib.tgpu_time_stencil_sum(self.h, stype, index, precision, reps, C.byref(ms)), self.lib)
        return ms.value

    def stats(self) -> dict:
        s = Stats()
        _check(self.lib.tgpu_get_stats(self.h, C.byref(s)), self.lib)
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def reset_stats(self):
        _check(self.lib.tgpu_reset_stats(self.h), self.lib)
