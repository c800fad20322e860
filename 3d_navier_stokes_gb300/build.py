"""Build the sm_103a shared library libns3d.so in-tree (3d_navier_stokes_gb300/_build/).

Every translation unit under csrc/ is compiled by nvcc in parallel for
sm_103a only, then linked into one shared library that exports the C ABI of
include/ns3d.h. A unit is recompiled when it, any header, or the flags are
newer than its object.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.environ.get("NS3D_BUILD_DIR") or os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libns3d.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include")] + ARCH + \
    os.environ.get("NS3D_NVCC_EXTRA", "").split()


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libns3d.so")
    return cand


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]


def _flag_stamp() -> str:
    return hashlib.sha1(" ".join(NVCC_FLAGS).encode()).hexdigest()[:12]


def _compile(src: str, nvcc: str, verbose: bool) -> str:
    obj = os.path.join(OUT, src[:-3] + ".o")
    srcp = os.path.join(CSRC, src)
    stamp = obj + ".flags"
    newest = max([os.path.getmtime(srcp)] + [os.path.getmtime(h) for h in _headers()])
    fresh = (os.path.exists(obj) and os.path.getmtime(obj) >= newest and os.path.exists(stamp)
             and open(stamp).read() == _flag_stamp())
    if fresh:
        return obj
    cmd = [nvcc] + NVCC_FLAGS + ["-c", srcp, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(_flag_stamp())
    return obj


CC = os.environ.get("CC", "gcc")
C_FLAGS = ["-std=gnu11", "-O2", "-fPIC", "-Wall", "-I", os.path.join(ROOT, "include")]
DRIVER = os.path.join(HERE, "driver", "solver_main.c")
SOLVER = os.path.join(OUT, "solver")


def _compile_c(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT, os.path.basename(src)[:-2] + ".c.o")
    newest = max([os.path.getmtime(src)] + [os.path.getmtime(h) for h in _headers()])
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [CC] + C_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{CC} failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    """Build libns3d.so (CUDA + C units) and the `solver` driver; return the library path."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    srcs = _sources()
    csrcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".c"))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, verbose), srcs))
    objs += [_compile_c(s, verbose) for s in csrcs]
    if not os.path.exists(LIB) or max(os.path.getmtime(o) for o in objs) > os.path.getmtime(LIB):
        cmd = [nvcc] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if not os.path.exists(SOLVER) or max(os.path.getmtime(DRIVER), os.path.getmtime(LIB)) > os.path.getmtime(SOLVER):
        cmd = [CC] + C_FLAGS + [DRIVER, "-o", SOLVER, "-L", OUT, "-lns3d", "-lm", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"driver link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
