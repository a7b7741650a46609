"""The reference's linear-problem-manager ABI (include/tramonto_legacy.h) solving on the GPU.

The Jacobian of a fixture state (from the C oracle, pinned to the reference's assembled matrix)
is inserted through dft_linprobmgr_insert* as the reference's fill would; setupsolver/solve run
the hard-sphere Schur-complement GMRES (and the basic manager's whole-matrix GMRES) on the GPU;
getlhs must equal a dense solve of the same system to 1e-8 relative, and the hard-sphere result
must equal the matrix-free tgpu_solve of the same state."""
import numpy as np
import pytest

import legacy_mgr as lm
import orc
from goldens import load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["hs1d_wall", "mix1d_fmt3"])
@pytest.mark.parametrize("hardsphere", [True, False])
def test_legacy_manager_solve(name, hardsphere):
    from tramonto_gb300 import native
    z, p = load(name)
    x = np.array(z["x0"])
    J = lm.dense_jacobian(orc.Oracle(p), x)
    b = np.sin(0.37 * np.arange(J.shape[0]))
    L = lm.lib()
    h, _ = lm.make_manager(L, p, z, hardsphere=hardsphere)
    assert L.tgpu_legacy_set_solver(h, 1e-12, 1000) == 0
    lm.insert_matrix(L, h, J, p.nunk, p.nnodes, b=b)
    assert L.dft_linprobmgr_setupsolver(h) == 0, L.tgpu_legacy_last_error()
    assert L.dft_linprobmgr_solve(h) == 0, L.tgpu_legacy_last_error()
    out = lm.Rows(np.zeros((p.nunk, p.nnodes)))
    assert L.dft_linprobmgr_getlhs(h, out.ptrs) == 0
    ref = np.linalg.solve(J, b)
    err = np.abs(out.a.reshape(-1) - ref).max() / np.abs(ref).max()
    it = lm.C.c_int(0)
    rr = lm.C.c_double(0.0)
    L.tgpu_legacy_last_solve(h, lm.C.byref(it), lm.C.byref(rr))
    print(name, "hard-sphere" if hardsphere else "basic", "GMRES", it.value, "relres", rr.value, "error", err)
    assert err <= 1e-8
    if hardsphere:
        s = native.Solver(p)
        s.fill(x, mode=0)
        dx, _, _ = s.solve(b.reshape(x.shape), tol=1e-12, max_iter=1000)
        s.close()
        assert np.abs(dx - out.a).max() <= 1e-8 * np.abs(ref).max()
    (L.dft_hardsphere_lin_prob_mgr_destruct if hardsphere else L.dft_linprobmgr_destruct)(h)


@pytest.mark.parametrize("name", ["lj1d_a22", "mix1d_fmt3"])
def test_legacy_ilu_preconditioner_of_a_nondiagonal_a22(name):
    """With seta22blockisdiagonal(0) the hard-sphere manager preconditions the Schur GMRES with ILU(2) of A22,
    as the reference does (src/dft_A22Matrix_Epetra_Operator.cpp:110-140): the solution equals a dense solve to
    1e-8, and on the attraction-in-A22 problem (lj1d_a22: the mean field summed into the Euler-Lagrange rows
    makes A22 non-diagonal) GMRES takes fewer iterations than with the diagonal; on a diagonal A22
    (mix1d_fmt3) the factors are that diagonal."""
    z, p = load(name)
    x = np.array(z["x0"])
    J = lm.dense_jacobian(orc.Oracle(p), x)
    b = np.sin(0.37 * np.arange(J.shape[0]))
    ref = np.linalg.solve(J, b)
    L = lm.lib()
    iters = {}
    for diag in (True, False):
        h, _ = lm.make_manager(L, p, z, hardsphere=True, a22_diagonal=diag)
        assert L.tgpu_legacy_set_solver(h, 1e-12, 1000) == 0
        lm.insert_matrix(L, h, J, p.nunk, p.nnodes, b=b)
        assert L.dft_linprobmgr_setupsolver(h) == 0, L.tgpu_legacy_last_error()
        assert L.dft_linprobmgr_solve(h) == 0, L.tgpu_legacy_last_error()
        out = lm.Rows(np.zeros((p.nunk, p.nnodes)))
        assert L.dft_linprobmgr_getlhs(h, out.ptrs) == 0
        it = lm.C.c_int(0)
        rr = lm.C.c_double(0.0)
        L.tgpu_legacy_last_solve(h, lm.C.byref(it), lm.C.byref(rr))
        iters[diag] = it.value
        err = np.abs(out.a.reshape(-1) - ref).max() / np.abs(ref).max()
        print(name, "diag(A22)" if diag else "ILU(2) of A22", "GMRES", it.value, "error", err)
        assert err <= 1e-8
        L.dft_hardsphere_lin_prob_mgr_destruct(h)
    if name == "lj1d_a22":
        assert iters[False] < iters[True]
    else:
        assert iters[False] == iters[True]
