"""oracle/workload.py builds the 128^3 workload for the oracle alone (the CPU reference arm of bench.py) from the
reference's own tables and bulk constants; it must describe the same problem the GPU arm builds with
tramonto_gb300.setup.config2: the same external field (bit for bit), stencils and constants."""
import numpy as np

import workload
from tramonto_gb300 import setup


def test_workload_matches_the_gpu_arm_problem():
    n = 40
    q = workload.config2_problem(n)
    p, meta = setup.config2(n=n)
    v, _ = setup.rough_wall_vext(p.nx, p.esize, kT=1.2, seed=meta["seed"], device=False)
    assert np.array_equal(q.vext, v) and np.array_equal(q.zero_density, p.zero_density)
    assert q.nx == tuple(p.nx) and q.bc == tuple(p.bc) and np.allclose(q.esize, p.esize, rtol=0, atol=0)
    assert (q.nunk, q.first_rb, q.first_mf) == (p.nunk, p.first_rb, p.first_mf)
    for name in ("rho_b", "hs_diam", "betamu_hs_ex", "betamu_att", "inv_rad", "inv_4pir", "inv_4pirsq",
                 "fac_overlap", "dphi_bulk"):
        assert np.allclose(getattr(q, name), getattr(p, name), rtol=1e-13, atol=1e-15), name
    assert q.vext_max == p.vext_max
    for key, (off, w, _) in q.stencils.items():
        off2, w2, _ = p.stencils[key]
        assert np.array_equal(off, off2) and np.abs(w - w2).max() <= 1e-14 * np.abs(w).max(), key


def test_initial_state_rows_are_their_own_sums():
    """On the sampled planes the oracle's residual of the weighted-density and mean-field rows vanishes."""
    import orc
    q = workload.config2_problem(32)
    o = orc.Oracle(q)
    x = workload.initial_state(q, o, sample_planes=1, threads=2)
    nxy = q.nx[0] * q.nx[1]
    R = o.resid_rows(x, 0, nxy)
    assert np.abs(R[q.first_rb:, :nxy]).max() <= 1e-12
    assert np.abs(x[q.first_rb, :nxy]).max() > 0.1 and np.abs(x[q.first_mf, :nxy]).max() > 0.1
