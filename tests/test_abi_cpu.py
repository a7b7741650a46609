"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point include/*.h declares (no GPU calls)."""
import ctypes
import glob
import os
import re

import pytest

from tramonto_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            txt = f.read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b((?:tgpu|dft)_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "tgpu_fill" in names and "tgpu_schur_apply" in names and len(names) > 20
    assert "dft_linprobmgr_insertonematrixvalue" in names and "dft_hardsphere_lin_prob_mgr_create" in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_errors_without_gpu_are_status_codes(lib):
    # a null geometry is rejected before any CUDA call
    lib.tgpu_create.restype = ctypes.c_int
    lib.tgpu_last_error.restype = ctypes.c_char_p
    h = ctypes.c_void_p()
    assert lib.tgpu_create(None, 0, ctypes.byref(h)) == -1
    assert b"null" in lib.tgpu_last_error()


@pytest.mark.parametrize("bc,reach,n", [((1, 1), 50, 30), ((2, 2), 50, 30), ((2, 1), 12, 10)],
                         ids=["periodic-reach-past-box", "reflect-both-sides", "reflect-then-periodic"])
def test_noalloc_rejects_stencils_that_reach_past_the_box(lib, bc, reach, n):
    """A padded position the boundary rules cannot map (a periodic reach longer than the box, a mirrored point
    beyond a periodic or reflecting far side) is TGPU_ERR_UNSUPPORTED, decided on the host before any device
    work (the field pointers here are never read)."""
    import numpy as np
    lib.tgpu_stencil_sum_noalloc.restype = ctypes.c_int
    lib.tgpu_noalloc_last_error.restype = ctypes.c_char_p
    nx = np.array([n, 1, 1], np.int32)
    bcs = np.array(bc, np.int32)
    off = np.array([[-reach], [0], [reach]], np.int16)
    w = np.ones(3)
    rc = lib.tgpu_stencil_sum_noalloc(1, ctypes.c_void_p(nx.ctypes.data), ctypes.c_void_p(bcs.ctypes.data),
                                      ctypes.c_double(0.0), 3, ctypes.c_void_p(off.ctypes.data),
                                      ctypes.c_void_p(w.ctypes.data), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    assert rc == -4 and b"reaches past the box" in lib.tgpu_noalloc_last_error()


def test_surface_spec_errors_before_device_work(lib):
    """The surface builder checks its spec on the host: a mesh without a positive element size is
    TGPU_ERR_ARG, options it does not build (a 1-D sphere, a 2-D slit pore of orientation 0,
    Ipot_wf_n 4) TGPU_ERR_UNSUPPORTED; tgpu_surface_mesh gives the reference's node and element counts."""
    import numpy as np
    from tramonto_gb300 import surfaces
    lj = dict(sigma_wf=[1.0], eps_wf=[1.0], cut_wf=[2.0])
    ok = surfaces.make_spec(2, (9.4, 10.0), (0.2, 0.2), [(1, 1), (-1, 3)], 1, [(0, (0.0, 0.0))],
                            [dict(surf_type=surfaces.SURF_COLLOID, param=(1.0, 0, 0), ipot_wf=5, **lj)])
    nodes, els = (ctypes.c_int * 3)(), (ctypes.c_int * 3)()
    assert lib.tgpu_surface_mesh(ctypes.byref(ok), nodes, els) == 0
    assert list(nodes) == [47, 51, 1] and list(els) == [47, 50, 1]
    bad = [
        (surfaces.make_spec(2, (9.4, 10.0), (0.2, 0.0), [(1, 1), (-1, 3)], 1, [(0, (0.0, 0.0))],
                            [dict(surf_type=surfaces.SURF_COLLOID, param=(1.0, 0, 0), ipot_wf=5, **lj)]), -1),
        (surfaces.make_spec(1, (9.4,), (0.2,), [(-1, 0)], 1, [(0, (0.0,))],
                            [dict(surf_type=surfaces.SURF_COLLOID, param=(1.0, 0, 0), ipot_wf=5, **lj)]), -4),
        (surfaces.make_spec(2, (9.4, 10.0), (0.2, 0.2), [(1, 1), (-1, 3)], 1, [(0, (0.0, 0.0))],
                            [dict(surf_type=surfaces.SURF_FINITE_PORE, orientation=0, param=(1.0, 2.0, 0),
                                  ipot_wf=5, **lj)]), -4),
        (surfaces.make_spec(2, (9.4, 10.0), (0.2, 0.2), [(1, 1), (-1, 3)], 1, [(0, (0.0, 0.0))],
                            [dict(surf_type=surfaces.SURF_PLANAR, param=(1.0, 0, 0), ipot_wf=4, **lj)]), -4),
    ]
    v = np.zeros(4096)
    z = np.zeros(4096, np.int8)
    for spec, code in bad:
        assert lib.tgpu_surface_field_host(ctypes.byref(spec), ctypes.c_void_p(v.ctypes.data),
                                           ctypes.c_void_p(z.ctypes.data), None) == code
