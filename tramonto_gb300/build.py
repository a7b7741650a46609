"""In-tree build of the CUDA library (sm_103a only).

Each .cu file under csrc/ is compiled by nvcc in parallel and linked into
tramonto_gb300/_build/libtramonto_gpu.so (static CUDA runtime).  Rebuilds only
what changed.  Used by __graft_entry__.build() and by tests.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtramonto_gpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "--expt-relaxed-constexpr",
           "-diag-suppress", "550,177"]
# stencils.cu: the host and device stencil builders must perform the same IEEE operations;
# surfaces.cu: positions, distances and rule choices with the reference's operations
FILE_FLAGS = {"stencils.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
              "surfaces.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    files = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(f) for f in files), default=0.0)


def _compile(src: str, extra) -> str:
    base, ext = os.path.splitext(os.path.basename(src))
    obj = os.path.join(BUILD, base + (".o" if ext == ".cu" else "_host.o"))
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _deps_mtime()):
        return obj
    tmp = obj + f".tmp{os.getpid()}"
    if ext == ".cu":
        cmd = [nvcc(), *ARCH, *NVFLAGS, *FILE_FLAGS.get(os.path.basename(src), []), *extra, "-I", INCLUDE, "-c", src,
               "-o", tmp]
    else:  # host-only C++ (set-up code)
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-I", INCLUDE, "-c", src, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    os.replace(tmp, obj)
    return obj


def build(verbose: bool = False, extra=()) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra)), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
