"""The 128^3 workload's physics at 64^3 against the oracle, plane by plane.

The reference fixtures of the 3-D path are small boxes at dx = 0.25 (a 5 233-point attraction stencil).  This
test takes the workload's own geometry at dx = 0.1 (setup.config2: FMT1 + WCA with the 71 831-point
attraction stencil that tests/test_stencils_3d_cpu.py pins to the reference's calc_stencils, a rough 12-3
wall, bulk at the far x side, periodic y and z) on a 64^3 grid and compares every unknown's residual row on
three z-planes (each plane holds the wall-side, interior and bulk-side x nodes; z = 0 and z = 63 also read the
periodic images) with the oracle's (oracle/oracle.c, the reference's fill restated):

- at the initial state and at a seeded perturbation of it (each unknown times 1 + 0.02 U(-1, 1));
- the FP64 fill to 1e-12 absolute (the FP64 parity tolerance), the FP64-FFT and float-float fills (the
  accurate fills of the mixed solve) to 5e-12, the FP32 fill to 1e-4 of max(1, |R|).
"""
import numpy as np
import pytest

import orc
from goldens import RESID_ATOL

pytestmark = pytest.mark.gpu

PLANES = (0, 31, 63)


@pytest.fixture(scope="module")
def workload():
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=64)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    rng = np.random.default_rng(21)
    x1 = x0 * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, x0.shape))
    o = orc.Oracle(p)
    nxy = p.nx[0] * p.nx[1]
    ref = []
    for x in (x0, x1):
        R = np.zeros((p.nunk, p.nnodes))
        for z in PLANES:
            part = o.resid_rows(x, z * nxy, (z + 1) * nxy)
            R[:, z * nxy:(z + 1) * nxy] = part[:, z * nxy:(z + 1) * nxy]
        ref.append(R)
    rows = np.concatenate([np.arange(z * nxy, (z + 1) * nxy) for z in PLANES])
    yield p, s, (x0, x1), ref, rows
    s.close()


@pytest.mark.parametrize("arith,tol", [("FILL_FP64", RESID_ATOL), ("FILL_FFT", 5e-12), ("FILL_FF", 5e-12),
                                       ("FILL_FP32", 1e-4)])
def test_fill_planes_match_oracle(workload, arith, tol):
    from tramonto_gb300 import native
    p, s, states, ref, rows = workload
    s.set_fill_arithmetic(getattr(native, arith))
    for k, x in enumerate(states):
        R = s.fill(x, mode=1)
        err = np.abs(R[:, rows] - ref[k][:, rows]).max()
        scale = max(1.0, np.abs(ref[k][:, rows]).max()) if arith == "FILL_FP32" else 1.0
        print(arith, "state", k, "max |R - R_oracle| on the planes", err, "max |R|", np.abs(ref[k][:, rows]).max())
        assert err <= tol * scale, (arith, k, err)
    s.set_fill_arithmetic(native.FILL_FP64)
