"""Quadrature zones and coarsened nodes as the fixtures carry them (no GPU).

calc_stencils (src/dft_stencil.c:96-109, 229-236) builds zone z's tables on elements 2^z times the mesh's and
scales their offsets by 2^z; set_mesh_coarsen_flag (src/dft_mesh.c:2788-2850) marks a node of zone z >= 1
that is off that zone's lattice with -(d + 1) for the first dimension d in which it is off.  The problem
parser and the native bindings must hand exactly these to the C ABI.
"""
import numpy as np
import pytest

from goldens import coarsened, load


@pytest.mark.parametrize("name", ["hs1d_zones", "hs1d_jaczones"])
def test_zone_fixture_structure(name):
    from tramonto_gb300.native import mesh_coarsened
    z, p = load(name)
    assert p.nzone == 4 and p.mesh_coarsening == 1 and p.nwall > 0
    assert coarsened(p) and mesh_coarsened(p)
    assert p.coarser_jac == (1 if name == "hs1d_jaczones" else 0)
    flag = np.asarray(p.zone_flag)
    assert flag.min() >= -p.ndim and flag.max() < p.nzone
    # zone tables: offsets on the zone's lattice, one table per stencil of zone 0
    assert sorted(p.zone_stencils) == [1, 2, 3]
    for zone, tabs in p.zone_stencils.items():
        assert sorted(tabs) == sorted(p.stencils)
        for (t, idx), (off, w, hw) in tabs.items():
            assert np.all(np.asarray(off) % (1 << zone) == 0), (zone, t, idx)
            assert len(w) == len(off) and np.all(np.isfinite(w))
    # a node that keeps zone z >= 1 lies on that zone's lattice
    x = np.arange(p.nnodes)
    on = flag >= 1
    assert np.all(x[on] % (1 << flag[on]) == 0)


def test_converged_reference_state_satisfies_the_averaged_rows():
    import orc
    z, p = load("hs1d_zones")
    R = orc.Oracle(p).resid(z["x_newton"])
    rows = np.asarray(p.zone_flag) < 0
    assert np.abs(R[:, rows]).max() <= 1e-10


def test_one_dimensional_boundary_fixture_structure():
    """fmt1_wca_3d_1dbc (L1D_bc = 1, X_1D_bc = 1 sigma, Grad_dim x): the nodes within 1 sigma of either x end are
    flagged -999 except the line y = z = 0, every other node keeps zone 0; the oracle's rows there are
    x(node) - x(line node) for every unknown (load_coarse_node_1dim)."""
    import orc
    z, p = load("fmt1_wca_3d_1dbc")
    assert p.l1d_bc == 1 and p.dim_1dbc == 0 and coarsened(p)
    flag = np.asarray(p.zone_flag)
    nx, ny, nz = p.nx
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ix, iy, iz = (a.transpose(2, 1, 0).reshape(-1) for a in (ix, iy, iz))   # node = x + nx (y + ny z)
    xpos = ix * p.esize[0]
    near = (xpos <= 1.0 + 1e-8) | (xpos >= (nx - 1) * p.esize[0] - (1.0 + 1e-8))
    line = (iy == 0) & (iz == 0)
    assert np.array_equal(flag == -999, near & ~line)
    assert np.all(flag[~(near & ~line)] == 0)
    x = np.asarray(z[f"x{len(z['states']) - 1}"])
    R = orc.Oracle(p).resid(x)
    nodes = np.nonzero(flag == -999)[0]
    want = x[:, nodes] - x[:, ix[nodes]]          # the line node of (x, y, z) is x itself
    assert np.array_equal(R[:, nodes], want)


@pytest.mark.parametrize("kind", ["bulk", "pb"])
def test_bulk_and_pb_zone_rows_in_the_oracle(kind):
    """The oracle's Euler-Lagrange rows at BULK_ZONE (-888) / PB_ZONE (-777) nodes: ln rho - ln rho_b
    (fill_bulk_density) / ln rho - ln rho_b + V_ext (the PB branches, no nonlocal terms); rows of other nodes and
    the other unknowns' rows as with zone 0 there."""
    import copy
    import orc
    z, p = load("lj1d_zones")
    q = copy.copy(p)
    f = np.asarray(p.zone_flag)
    q.zone_flag = np.where(f != 0, -888 if kind == "bulk" else -777, 0).astype(np.int32)
    q.mesh_coarsening = 2 if kind == "bulk" else 3
    x = np.asarray(z["x1"])
    R = orc.Oracle(q).resid(x)
    rho = x[q.first_rho]
    flagged = (q.zone_flag < 0) & (np.asarray(q.zero_density)[0] == 0) & (np.asarray(q.vext)[0] < q.vext_max)
    want = np.log(rho[flagged]) - np.log(q.rho_b[0])
    if kind == "pb":
        want = want + np.asarray(q.vext)[0][flagged]
    assert np.allclose(R[q.first_rho][flagged], want, rtol=0, atol=1e-13)
    # unflagged nodes: the same rows as the problem without the flags (zone 0 there)
    zq = copy.copy(p)
    zq.zone_flag = np.zeros_like(f)
    R0 = orc.Oracle(zq).resid(x)
    assert np.array_equal(R[:, q.zone_flag == 0], R0[:, q.zone_flag == 0])
