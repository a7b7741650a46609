"""External fields generated on the GPU (tgpu_wall_field_*) against the numpy construction of the
same walls: the rough 12-3 wall of the 128^3 and 256^3 workloads and the 9-3 slit pores of
configuration 5 (1-D and chemically patterned 2-D).  Values below vext_max agree to 1e-13
relative (the two evaluate powers differently); the clipped (zero-density) nodes are the same
except where a value lies within 1e-9 of vext_max."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _compare(a, b, vmax):
    a, b = np.asarray(a).ravel(), np.asarray(b).ravel()
    ca, cb = a >= vmax, b >= vmax
    border = np.abs(np.where(ca, b, a) - vmax) <= 1e-9
    assert np.all((ca == cb) | border)
    live = ~ca & ~cb
    assert live.any()
    err = np.abs(a[live] - b[live]) / np.maximum(1.0, np.abs(b[live]))
    assert err.max() <= 1e-13, err.max()


@pytest.mark.parametrize("n,dx", [(64, 0.1), (128, 0.1), (256, 0.08)])
def test_rough_wall_field(n, dx):
    from tramonto_gb300 import setup
    nx, es = (n, n, n), (dx, dx, dx)
    vd, md = setup.rough_wall_vext(nx, es, device=True)
    vh, mh = setup.rough_wall_vext(nx, es, device=False)
    assert md == mh
    _compare(vd, vh, 10.0)


@pytest.mark.parametrize("ndim,n,dx", [(1, 3001, 0.01), (1, 401, 0.01), (2, 200, 0.05), (2, 333, 0.05)])
def test_slit_pore_field(ndim, n, dx):
    from tramonto_gb300 import setup
    nx = (n,) * ndim
    es = (dx,) * ndim
    _compare(setup.slit_pore_vext(ndim, nx, es, device=True), setup.slit_pore_vext(ndim, nx, es, device=False), 10.0)
