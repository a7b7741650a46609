"""ctypes view of the reference's linear-problem-manager ABI as the library serves it
(include/tramonto_legacy.h), used by the legacy-ABI tests."""
import ctypes as C

import numpy as np

from tramonto_gb300 import native

vp, ip, dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)
dpp = C.POINTER(dp)

SIGS = {
    "dft_basic_lin_prob_mgr_create": (vp, [C.c_int, vp, vp]),
    "dft_hardsphere_lin_prob_mgr_create": (vp, [C.c_int, vp, vp]),
    "dft_hardsphere_lin_prob_mgr_destruct": (None, [vp]),
    "dft_linprobmgr_destruct": (None, [vp]),
    "dft_hardsphere_lin_prob_mgr_setindnonlocalequationids": (C.c_int, [vp, C.c_int, ip]),
    "dft_hardsphere_lin_prob_mgr_setdepnonlocalequationids": (C.c_int, [vp, C.c_int, ip]),
    "dft_hardsphere_lin_prob_mgr_setdensityequationids": (C.c_int, [vp, C.c_int, ip]),
    "dft_hardsphere_lin_prob_mgr_seta22blockisdiagonal": (C.c_int, [vp, C.c_int]),
    "dft_linprobmgr_setnodalrowmap": (C.c_int, [vp, C.c_int, ip]),
    "dft_linprobmgr_setnodalcolmap": (C.c_int, [vp, C.c_int, ip]),
    "dft_linprobmgr_finalizeblockstructure": (C.c_int, [vp]),
    "dft_linprobmgr_initializeproblemvalues": (C.c_int, [vp]),
    "dft_linprobmgr_insertrhsvalue": (C.c_int, [vp, C.c_int, C.c_int, C.c_double]),
    "dft_linprobmgr_insertonematrixvalue": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double]),
    "dft_linprobmgr_insertmultinodematrixvalues": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, ip, dp, C.c_int]),
    "dft_linprobmgr_insertmultiphysicsmatrixvalues": (C.c_int, [vp, C.c_int, C.c_int, ip, C.c_int, dp, C.c_int]),
    "dft_linprobmgr_finalizeproblemvalues": (C.c_int, [vp]),
    "dft_linprobmgr_getmatrixvalue": (C.c_double, [vp, C.c_int, C.c_int, C.c_int, C.c_int]),
    "dft_linprobmgr_setrhs": (C.c_int, [vp, dpp]),
    "dft_linprobmgr_getrhs": (C.c_int, [vp, dpp]),
    "dft_linprobmgr_getlhs": (C.c_int, [vp, dpp]),
    "dft_linprobmgr_writeMatrix": (C.c_int, [vp, C.c_char_p, C.c_char_p, C.c_char_p]),
    "dft_linprobmgr_setupsolver": (C.c_int, [vp]),
    "dft_linprobmgr_solve": (C.c_int, [vp]),
    "dft_linprobmgr_applymatrix": (C.c_int, [vp, dpp, dpp]),
    "dft_linprobmgr_importr2c": (C.c_int, [vp, dpp, dpp]),
    "tgpu_legacy_set_solver": (C.c_int, [vp, C.c_double, C.c_int]),
    "tgpu_legacy_last_solve": (C.c_int, [vp, ip, dp]),
    "tgpu_legacy_last_error": (C.c_char_p, []),
}


def lib():
    L = native.load()
    for name, (res, args) in SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def ints(a):
    a = np.ascontiguousarray(a, np.int32)
    return a, a.ctypes.data_as(ip)


class Rows:
    """A [nunk][N] array and the double** the reference's managers take for it."""

    def __init__(self, arr):
        self.a = np.ascontiguousarray(arr, np.float64)
        self.ptrs = (dp * self.a.shape[0])(*[self.a[u].ctypes.data_as(dp) for u in range(self.a.shape[0])])


def dense_jacobian(oracle, x):
    """J column by column from the oracle's J v (small problems only)."""
    n = x.size
    J = np.zeros((n, n))
    e = np.zeros(n)
    for k in range(n):
        e[k] = 1.0
        J[:, k] = oracle.jv(x, e.reshape(x.shape)).reshape(-1)
        e[k] = 0.0
    return J


def make_manager(L, p, z, hardsphere=True, a22_diagonal=True):
    N, nunk = p.nnodes, p.nunk
    h = (L.dft_hardsphere_lin_prob_mgr_create if hardsphere else L.dft_basic_lin_prob_mgr_create)(nunk, None, None)
    assert h
    if hardsphere:
        for fn, key in (("setindnonlocalequationids", "blk_ind"), ("setdepnonlocalequationids", "blk_dep"),
                        ("setdensityequationids", "blk_dens")):
            a, ptr = ints(z[key])
            assert getattr(L, "dft_hardsphere_lin_prob_mgr_" + fn)(h, len(a), ptr) == 0
        assert L.dft_hardsphere_lin_prob_mgr_seta22blockisdiagonal(h, 1 if a22_diagonal else 0) == 0
    assert L.dft_linprobmgr_finalizeblockstructure(h) == -1      # maps not set yet
    g, gp = ints(np.arange(N))
    assert L.dft_linprobmgr_setnodalrowmap(h, N, gp) == 0
    assert L.dft_linprobmgr_setnodalcolmap(h, N, gp) == 0
    assert L.dft_linprobmgr_finalizeblockstructure(h) == 0
    assert L.dft_linprobmgr_finalizeblockstructure(h) == 1       # already done
    return h, g


def insert_matrix(L, h, J, nunk, N, b=None):
    """Insert J (dense, SoA index u*N + node) row by row as the reference's fill does: runs of box nodes per
    (row, column unknown), single values, and a multi-physics call per row's own node."""
    assert L.dft_linprobmgr_initializeproblemvalues(h) == 0
    for r in range(nunk * N):
        u, i = divmod(r, N)
        cols = np.nonzero(J[r])[0]
        if cols.size == 0:
            continue
        ju_all, j_all = np.divmod(cols, N)
        own = j_all == i                         # entries at the row's own node: one multi-physics call
        if own.any():
            ju, pj = ints(ju_all[own])
            v = np.ascontiguousarray(J[r, cols[own]])
            assert L.dft_linprobmgr_insertmultiphysicsmatrixvalues(h, u, i, pj, i, v.ctypes.data_as(dp), len(v)) == 0
        for ju in np.unique(ju_all[~own]):
            sel = (~own) & (ju_all == ju)
            nodes, pn = ints(j_all[sel])
            vals = np.ascontiguousarray(J[r, cols[sel]])
            if len(vals) == 1:
                assert L.dft_linprobmgr_insertonematrixvalue(h, u, i, int(ju), int(nodes[0]), float(vals[0])) == 0
            else:
                # split the run in two inserts so that the manager sums repeated calls correctly
                half = len(vals) // 2
                assert L.dft_linprobmgr_insertmultinodematrixvalues(h, u, i, int(ju), pn, vals.ctypes.data_as(dp),
                                                                    half) == 0
                rest, pr = ints(nodes[half:])
                rv = np.ascontiguousarray(vals[half:])
                assert L.dft_linprobmgr_insertmultinodematrixvalues(h, u, i, int(ju), pr, rv.ctypes.data_as(dp),
                                                                    len(rv)) == 0
        if b is not None:
            assert L.dft_linprobmgr_insertrhsvalue(h, u, i, float(b[r])) == 0
    assert L.dft_linprobmgr_finalizeproblemvalues(h) == 0
