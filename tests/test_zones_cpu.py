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
