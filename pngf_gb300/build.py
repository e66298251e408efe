"""In-tree build of libpngf_gb300.so (sm_103a only).

Each translation unit is compiled in parallel with nvcc, then linked into
pngf_gb300/libpngf_gb300.so next to this file. Objects go to
pngf_gb300/_build/. Run as ``python -m pngf_gb300.build``.

``--bounds-check`` builds the bounds-checked variant instead
(-DPNGF_BOUNDS_CHECK, objects in _build/bc/, pngf_gb300/libpngf_gb300_bc.so):
the data-dependent gathers record out-of-range indices rather than reading
them (see csrc/bounds.cuh).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpngf_gb300.so")
LIB_BC = os.path.join(HERE, "libpngf_gb300_bc.so")

SOURCES = ["kernels_fp64.cu", "kernels_c64.cu", "kernels_f64tc.cu", "capi.cu", "dbs.cpp", "dbs_device.cu", "gfile.cpp", "noalloc.cu",
           "proposal.cu", "synth.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pngf_gb300")


def _compile(src: str, bounds_check: bool = False) -> str:
    obj = os.path.join(BUILD, "bc" if bounds_check else "", os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
            os.path.getmtime(path), *[os.path.getmtime(os.path.join(CSRC, h)) for h in os.listdir(CSRC)
                                      if h.endswith(".h") or h.endswith(".cuh")],
            os.path.getmtime(os.path.join(ROOT, "include", "pngf_gb300.h"))):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + (["-DPNGF_BOUNDS_CHECK"] if bounds_check else []) + ["-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose: bool = False, bounds_check: bool = False) -> str:
    os.makedirs(os.path.join(BUILD, "bc") if bounds_check else BUILD, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, bounds_check), srcs))
    out = LIB_BC if bounds_check else LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fopenmp", "-Xlinker", "--no-undefined", "-o", out] + objs + ["-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", out)
    return out


if __name__ == "__main__":
    build(verbose=True, bounds_check="--bounds-check" in sys.argv[1:])
    sys.exit(0)
