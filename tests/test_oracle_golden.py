"""The C restatement oracle against golden vectors produced by the reference itself."""
import numpy as np
import pytest

import orc
from goldens import CASES, PROD_RTOL, RESID_ATOL, coarsened, load, probe, rel_err


@pytest.fixture(scope="module", params=CASES)
def case(request):
    z, p = load(request.param)
    return request.param, z, p, orc.Oracle(p)


def test_residual_matches_reference(case):
    name, z, p, o = case
    for k in range(len(z["states"])):
        R = o.resid(z[f"x{k}"])
        assert np.abs(R - z[f"R{k}"]).max() <= RESID_ATOL, name


def test_jacobian_products_match_reference(case):
    name, z, p, o = case
    N = p.nunk * p.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        assert rel_err(o.jv(x, probe(N, 0).reshape(x.shape)), z[f"Jv{k}"]) <= PROD_RTOL, name
        assert rel_err(o.jtv(x, probe(N, 1).reshape(x.shape)), z[f"JTw{k}"]) <= PROD_RTOL, name


def test_schur_product_matches_reference(case):
    name, z, p, o = case
    if coarsened(p):
        pytest.skip("the reference's Schur blocks move every unknown of a coarsened node into block 2")
    n2 = p.ncomp * p.nnodes
    for k in range(len(z["states"])):
        S = o.schur(z[f"x{k}"], probe(n2, 2).reshape(p.ncomp, p.nnodes))
        assert rel_err(S, z[f"schur_Sv{k}"]) <= PROD_RTOL, name


def test_converged_state_has_small_residual(case):
    name, z, p, o = case
    if z["states"][0] == 0:
        R = o.resid(z["x0"])
        assert np.abs(R).max() < 1e-6, name
