"""The reference's linear-problem-manager ABI (include/tramonto_legacy.h): the host-side part -
block structure, scalar inserts as the reference's fill makes them, matrix read-back, J x and
the owned-to-box copy - against the Jacobian of the C oracle (pinned to the reference's assembled
matrix).  No GPU calls: the solve is tested in test_gpu_legacy.py."""
import numpy as np
import pytest

import legacy_mgr as lm
import orc
from goldens import load


@pytest.fixture(scope="module")
def assembled():
    z, p = load("hs1d_wall")
    x = np.array(z["x0"])
    J = lm.dense_jacobian(orc.Oracle(p), x)
    L = lm.lib()
    h, _ = lm.make_manager(L, p, z)
    lm.insert_matrix(L, h, J, p.nunk, p.nnodes, b=-np.arange(J.shape[0], dtype=float))
    yield L, h, J, p
    L.dft_hardsphere_lin_prob_mgr_destruct(h)


def test_inserted_matrix_reads_back(assembled):
    L, h, J, p = assembled
    N = p.nnodes
    rng = np.random.default_rng(0)
    nz = np.argwhere(J != 0)
    for r, c in nz[rng.choice(len(nz), 200, replace=False)]:
        u, i = divmod(int(r), N)
        ju, j = divmod(int(c), N)
        assert L.dft_linprobmgr_getmatrixvalue(h, u, i, ju, j) == J[r, c]


def test_applymatrix_and_rhs(assembled):
    L, h, J, p = assembled
    x = np.random.default_rng(1).standard_normal((p.nunk, p.nnodes))
    xr, br = lm.Rows(x), lm.Rows(np.zeros_like(x))
    assert L.dft_linprobmgr_applymatrix(h, xr.ptrs, br.ptrs) == 0
    assert np.abs(br.a.reshape(-1) - J @ x.reshape(-1)).max() <= 1e-12 * np.abs(J).sum(axis=1).max() * 10
    got = lm.Rows(np.zeros_like(x))
    assert L.dft_linprobmgr_getrhs(h, got.ptrs) == 0
    assert np.array_equal(got.a.reshape(-1), -np.arange(J.shape[0], dtype=float))
    box = lm.Rows(np.zeros_like(x))
    assert L.dft_linprobmgr_importr2c(h, xr.ptrs, box.ptrs) == 0
    assert np.array_equal(box.a, x)


def test_lhs_before_solve_is_an_error(assembled):
    L, h, J, p = assembled
    out = lm.Rows(np.zeros((p.nunk, p.nnodes)))
    assert L.dft_linprobmgr_getlhs(h, out.ptrs) != 0
    assert b"solve" in L.tgpu_legacy_last_error()


def test_matrix_market_output(assembled, tmp_path):
    L, h, J, p = assembled
    f = tmp_path / "J.mtx"
    assert L.dft_linprobmgr_writeMatrix(h, str(f).encode(), b"J", b"hs1d_wall") == 0
    lines = [ln for ln in f.read_text().splitlines() if not ln.startswith("%")]
    n, m, nnz = map(int, lines[0].split())
    assert n == m == J.shape[0] and nnz == np.count_nonzero(J)
    A = np.zeros_like(J)
    for ln in lines[1:]:
        r, c, v = ln.split()
        A[int(r) - 1, int(c) - 1] = float(v)
    assert np.array_equal(A, J)
