"""Python side of the reference oracle (test infrastructure only).

``oracle/_ref/libtramonto_ref.so`` is the reference's own C physics (its
src/*.c files, compiled in place by ``oracle/refbuild/Makefile``) linked with
a serial MPI stand-in and a recording linear-problem manager.  This module
drives it:

* :func:`run_case` runs ``dftmain`` on an input deck (Newton to convergence
  plus the reference's post-processing) and returns the parsed
  ``dft_output.dat`` line;
* :func:`extract` runs the set-up half of ``dftmain``, optionally Newton, then
  calls ``fill_resid_and_matrix_control`` on chosen solution vectors and
  returns the problem description (stencils, bulk constants, V_ext, flags),
  residuals and the assembled Jacobian.

The library keeps the reference's global state, so every call runs in a
fresh child process.  Input decks are the reference's own
``Examples/*/dft_input.dat`` files, optionally edited line by line with
:func:`edit_deck`.  Nothing in the product imports this module.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libtramonto_ref.so")
# the reference checkout, read in place: TRAMONTO_REFERENCE overrides the default location
REFERENCE = os.environ.get("TRAMONTO_REFERENCE", "/root/reference")

# stencil type ids of the reference (src/dft_globals_const.h:152-161)
DELTA_FN_R, THETA_FN_R, THETA_PAIRPOT_RCUT = 0, 1, 2
NSTEN = 8


def reference_available() -> bool:
    return os.path.isdir(os.path.join(REFERENCE, "src"))


def build_ref(jobs: int = 8) -> str:
    """Compile the reference's C sources into oracle/_ref (needs the reference tree)."""
    if not reference_available():
        raise RuntimeError("reference tree not present; the reference oracle cannot be built")
    subprocess.run(["make", "-s", f"-j{jobs}", "-C", os.path.join(HERE, "refbuild"), f"REF={REFERENCE}"],
                   check=True)
    return REF_LIB


def example_dir(name: str) -> str:
    return os.path.join(REFERENCE, "Examples", name)


def read_deck(path: str) -> list[str]:
    with open(path) as f:
        return f.read().splitlines()


def edit_deck(lines: list[str], edits: dict[str, str]) -> list[str]:
    """Replace the data fields of '@' lines whose label contains a key.

    The reference parser (src/dft_input.c) reads the fields that follow '@'
    and ignores the rest of the line, so a line is rewritten as
    '@ <new fields>  <old label>'.  Keys must match exactly one '@' line.
    """
    out = list(lines)
    for key, val in edits.items():
        hits = [i for i, ln in enumerate(out) if ln.startswith("@") and key in ln]
        if len(hits) != 1:
            raise KeyError(f"deck key {key!r} matched {len(hits)} lines")
        i = hits[0]
        label = out[i][out[i].index(key):] if key in out[i] else ""
        out[i] = f"@ {val} \t{label}"
    return out


def _stage(deck_lines, surfaces_from: str | None, workdir: str):
    with open(os.path.join(workdir, "dft_input.dat"), "w") as f:
        f.write("\n".join(deck_lines) + "\n")
    if surfaces_from:
        src = os.path.join(surfaces_from, "dft_surfaces.dat")
        if os.path.exists(src):
            shutil.copy(src, workdir)


def _lib():
    import ctypes
    lib = ctypes.CDLL(REF_LIB)
    return lib


def _child_run(deck_lines, surfaces_from, q):
    import ctypes
    try:
        with tempfile.TemporaryDirectory() as wd:
            _stage(deck_lines, surfaces_from, wd)
            lib = _lib()
            e = ctypes.c_double(0.0)
            lib.tref_run(wd.encode(), ctypes.byref(e))
            with open(os.path.join(wd, "dft_output.dat")) as f:
                txt = f.read().splitlines()
            q.put({"header": txt[0].split(), "values": [float(v) for v in txt[1].split()]})
    except Exception as exc:  # pragma: no cover - reported to the parent
        q.put({"error": repr(exc)})


def _spawn(target, *args, timeout=900):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=target, args=(*args, q))
    p.start()
    import queue
    import time
    t0 = time.time()
    res = None
    try:
        while res is None:
            try:
                res = q.get(timeout=1.0)
            except queue.Empty:
                if not p.is_alive():
                    raise RuntimeError(f"reference child process died (exit code {p.exitcode})")
                if time.time() - t0 > timeout:
                    raise TimeoutError("reference child process timed out")
    finally:
        p.join(timeout=60)
        if p.is_alive():
            p.kill()
    if "error" in res:
        raise RuntimeError(res["error"])
    return res


def run_case(deck_lines, surfaces_from=None, timeout=900):
    """Run the reference end to end; returns {'header': [...], 'values': [...]}."""
    return _spawn(_child_run, deck_lines, surfaces_from, timeout=timeout)


def _child_extract(deck_lines, surfaces_from, opts, q):
    import ctypes
    try:
        with tempfile.TemporaryDirectory() as wd:
            _stage(deck_lines, surfaces_from, wd)
            lib = _lib()
            c_int_p = ctypes.POINTER(ctypes.c_int)
            c_dbl_p = ctypes.POINTER(ctypes.c_double)
            c_ll_p = ctypes.POINTER(ctypes.c_longlong)

            def ip(a):
                return a.ctypes.data_as(c_int_p)

            def dp(a):
                return a.ctypes.data_as(c_dbl_p)

            if lib.tref_setup(wd.encode()) != 0:
                raise RuntimeError("tref_setup failed")
            ints = np.zeros(64, np.int32)
            nint = lib.tref_info_ints(ip(ints))
            ints = ints[:nint].copy()
            dbls = np.zeros(512, np.float64)
            ndbl = lib.tref_info_doubles(dp(dbls))
            out = {"info_ints": ints, "info_doubles": dbls[:ndbl].copy()}
            ndim = int(ints[0])
            nnodes, nbox, nown, nunk, ncomp = (int(v) for v in ints[4:9])
            nlists = int(ints[14])
            nel_v = int(ints[39])   # Nnodes_per_el_V (tref_info_ints order)
            lhard = int(ints[13])
            l2b = np.zeros(nown, np.int32)
            b2g = np.zeros(nbox, np.int32)
            lib.tref_maps(ip(l2b), ip(b2g))
            out["l2b"], out["b2g"] = l2b, b2g
            vext = np.zeros(ncomp * nown)
            lib.tref_get_vext(dp(vext))
            out["vext"] = vext.reshape(ncomp, nown)
            zt = np.zeros(ncomp * nbox, np.int32)
            lib.tref_get_zero_density(ip(zt))
            out["zero_density"] = zt.reshape(ncomp, nbox)
            if int(ints[15]) > 0:   # Nwall: the surfaces (positions, images, wall-fluid parameters, elements)
                wi = np.zeros(64, np.int32)
                wd = np.zeros(4096, np.float64)
                lib.tref_wall_info(ip(wi), dp(wd))
                nwall, ntype, _, nel, nimg = (int(v) for v in wi[:5])
                out["wall_type"] = wi[5:5 + nwall].copy()
                k = 0
                out["wall_pos"] = wd[k:k + 3 * nwall].reshape(nwall, 3).copy()
                k += 3 * nwall
                for key in ("sigma_wf", "eps_wf", "cut_wf"):
                    out[key] = wd[k:k + ncomp * ntype].reshape(ncomp, ntype).copy()
                    k += ncomp * ntype
                out["wall_images"] = wd[k:k + 3 * nimg].reshape(nimg, 3).copy()
                we = np.zeros(nel, np.int32)
                if lib.tref_wall_elems(ip(we)) == 0:
                    out["wall_elems"] = we
            if lhard and nlists > 0:
                bn = np.zeros(nlists * nbox, np.int32)
                if lib.tref_get_boundary_nodes(ip(bn)) == 0:
                    out["boundary_nodes"] = bn.reshape(nlists, nbox)
                nrefl = 1 << ndim
                fm = np.zeros(nlists * nrefl * nbox, np.int32)
                if lib.tref_get_fluid_masks(ip(fm)) == 0:
                    out["fluid_masks"] = fm.reshape(nlists, nrefl, nbox)
            # stencils: zone 0; index = icomp (+ ncomp*jcomp for the pair stencil)
            sten = {}
            # delta/theta stencils exist per component (index icomp), the pair
            # stencil per component pair (index icomp + Ncomp*jcomp); the other
            # entries of the reference's Stencil array are never initialised.
            for isten, nidx in ((DELTA_FN_R, ncomp), (THETA_FN_R, ncomp), (THETA_PAIRPOT_RCUT, ncomp * ncomp)):
                for idx in range(nidx):
                    L = lib.tref_stencil_length(isten, 0, idx)
                    if L <= 0:
                        continue
                    off = np.zeros(L * ndim, np.int32)
                    w = np.zeros(L)
                    hw = np.zeros(L * nel_v) if lhard else None
                    lib.tref_stencil(isten, 0, idx, ip(off), dp(w), dp(hw) if hw is not None else None)
                    sten[(isten, idx)] = (off.reshape(L, ndim), w, None if hw is None else hw.reshape(L, nel_v))
            out["stencils"] = sten
            # quadrature zones above 0 (coarser elements, offsets in fine-node units) and the per-node
            # zone / coarsening flags
            nzone = int(ints[25])
            zsten = {}
            for zone in range(1, nzone):
                for isten, nidx in ((DELTA_FN_R, ncomp), (THETA_FN_R, ncomp), (THETA_PAIRPOT_RCUT, ncomp * ncomp)):
                    for idx in range(nidx):
                        L = lib.tref_stencil_length(isten, zone, idx)
                        if L <= 0:
                            continue
                        off = np.zeros(L * ndim, np.int32)
                        w = np.zeros(L)
                        hw = np.zeros(L * nel_v) if lhard else None
                        lib.tref_stencil(isten, zone, idx, ip(off), dp(w), dp(hw) if hw is not None else None)
                        zsten[(zone, isten, idx)] = (off.reshape(L, ndim), w,
                                                     None if hw is None else hw.reshape(L, nel_v))
            out["zone_stencils"] = zsten
            cf = np.zeros(nbox, np.int32)
            if lib.tref_get_coarsen_flag(ip(cf)) == 0:
                out["coarsen_flag"] = cf
            hit = np.zeros(ncomp * nown, np.int32)
            hit2 = np.zeros(ncomp * nown, np.int32)
            integ = np.zeros(6 + ncomp)
            lib.tref_integration(ip(hit), ip(hit2), dp(integ))
            out["nel_hit"], out["nel_hit2"], out["integ"] = hit.reshape(ncomp, nown), hit2.reshape(ncomp, nown), integ
            x0 = np.zeros(nunk * nbox)
            lib.tref_get_x(dp(x0))
            out["x_guess"] = x0.reshape(nunk, nbox).copy()
            if opts.get("newton"):
                out["newton_iters"] = lib.tref_newton()
                xc = np.zeros(nunk * nbox)
                lib.tref_get_x(dp(xc))
                out["x_newton"] = xc.reshape(nunk, nbox).copy()
            fills = []
            for xs in opts.get("fill_states", []):
                if isinstance(xs, str):
                    xs = out[xs]
                elif isinstance(xs, tuple):
                    key, seed, rel = xs
                    rng = np.random.default_rng(seed)
                    xs = out[key] * (1.0 + rel * rng.uniform(-1.0, 1.0, out[key].shape))
                xs = np.ascontiguousarray(xs, dtype=np.float64).reshape(-1)
                lib.tref_set_x(dp(xs))
                rs = ctypes.c_double(0.0)
                lib.tref_fill(1, 0, ctypes.byref(rs))
                sizes = np.zeros(8, np.int32)
                lib.tref_mgr_sizes(ip(sizes))
                nnz = int(sizes[4])
                ng = int(sizes[3])
                rhs = np.zeros(nunk * nown)
                lib.tref_mgr_rhs(dp(rhs))
                rows = np.zeros(nnz, np.int64)
                cols = np.zeros(nnz, np.int64)
                vals = np.zeros(nnz)
                lib.tref_mgr_matrix(rows.ctypes.data_as(c_ll_p), cols.ctypes.data_as(c_ll_p), dp(vals))
                lib.tref_set_x(dp(xs))
                om = ctypes.c_double(0.0)
                ads, ads_b = np.zeros(ncomp), np.zeros(ncomp)
                lib.tref_energy(ctypes.byref(om), dp(ads), dp(ads_b))
                fills.append({"x": xs.reshape(nunk, nbox), "rhs": rhs.reshape(nunk, nown), "rows": rows,
                              "cols": cols, "vals": vals, "nglobal": ng, "resid_sum": rs.value,
                              "omega_s": om.value, "ads": ads, "ads_b": ads_b})
            out["fills"] = fills
            q.put(out)
    except Exception as exc:  # pragma: no cover
        import traceback
        q.put({"error": traceback.format_exc()})


def extract(deck_lines, surfaces_from=None, newton=False, fill_states=(), timeout=1800):
    """Set up a case with the reference and read back its fill (see module doc)."""
    opts = {"newton": newton, "fill_states": list(fill_states)}
    return _spawn(_child_extract, deck_lines, surfaces_from, opts, timeout=timeout)
