"""Shared helpers for the golden-fixture tests (test infrastructure)."""
import os

import numpy as np

from tramonto_gb300.problem import from_golden

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
CASES = ["hs1d_wall", "hs1d_reflect", "lj1d_mf", "mix1d_fmt3", "fmt1_wca_3d", "hs1d_c1",
         "hs1d_fmt2", "hs1d_fmt4", "mix1d_fmt4", "rough3d_fmt2", "rough3d_fmt4",
         "lj1d_sigzero", "lj1d_jdc", "yuk1d_mf", "exp1d_mf", "sw1d_mf", "hslj1d_wall", "lj1d_a22",
         "lv1d_interface", "lv1d_bulkbc", "hs1d_zones", "hs1d_jaczones", "mix3_hw1d", "mix4_hw1d_fmt3",
         "lj1d_zones", "lj1d_zones_a22", "fmt1_wca_3d_1dbc"]

# The reference fills in IEEE FP64 with its own summation order; any other
# order differs by rounding.  Residual entries are compared with an absolute
# tolerance scaled by the size of the terms they sum (O(1..10) for log rho,
# the chemical potential and the stencil sums), products by their max norm.
RESID_ATOL = 1e-12
PROD_RTOL = 1e-12


def load(case):
    z = np.load(os.path.join(GOLDEN, f"{case}.npz"))
    return z, from_golden(z)


def coarsened(p):
    """True when some nodes' rows average their neighbours (mesh coarsening) or copy the 1-D line (L1D_bc)."""
    if p.zone_flag is None or not ((p.mesh_coarsening and p.nwall > 0) or p.l1d_bc):
        return False
    f = p.zone_flag
    return bool(((f < 0) & (f != -888) & (f != -777)).any())


def probe(n, k):
    """Same deterministic probe vectors as tests/golden/make_golden.py."""
    i = np.arange(n, dtype=np.float64)
    return np.sin(1.3 + 0.7071 * k + 0.61803 * (k + 1) * i)


def rel_err(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))
