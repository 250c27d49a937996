"""Build recipe for the native engine (libsparq_gb300.so, sm_103a only).

Each CUDA translation unit under csrc/ is compiled separately and in
parallel, then linked into one shared library placed next to this file.
Amplitude arithmetic is compiled with --fmad=false (and host code with
-ffp-contract=off) so that no multiply-add is contracted: complex products,
butterflies and the host-side angle computations then round exactly like the
reference's CPU code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libsparq_gb300.so"

SOURCES = ["sq_core.cu", "elementwise.cu", "compact.cu", "radix_sort.cu", "group_ops.cu", "api.cu", "predictor.cu"]
# group_ops.cu is also compiled once per key width K (its kernels are templates
# on K), so that the objects build in parallel: (source, object stem, defines)
UNITS = [(s, Path(s).stem, []) for s in SOURCES] + \
        [("group_ops.cu", f"group_ops_k{k}", [f"-DSQ_GROUP_K={k}"]) for k in range(1, 9)]
HEADERS = ["sq_internal.cuh", "lookback.cuh"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--fmad=false", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
              "-I" + str(INCLUDE), "-I" + str(CSRC)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newest_input() -> float:
    files = [CSRC / s for s in SOURCES + HEADERS] + [INCLUDE / "sparq_gb300.h", Path(__file__)]
    return max(f.stat().st_mtime for f in files)


def _compile(unit) -> Path:
    src, stem, defines = unit
    obj = BUILD / (stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *defines, "-c", str(CSRC / src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = True) -> Path:
    """Compile csrc/*.cu for sm_103a and link libsparq_gb300.so; returns its path."""
    if LIB.exists() and not force and LIB.stat().st_mtime >= _newest_input():
        return LIB
    BUILD.mkdir(exist_ok=True)
    # longest units first so the pool stays busy
    units = sorted(UNITS, key=lambda u: (u[0] not in ("group_ops.cu", "elementwise.cu"), u[1]))
    with cf.ThreadPoolExecutor(max_workers=min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, units))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(tmp), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
