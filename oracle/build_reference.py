"""TEST INFRASTRUCTURE ONLY. Builds the reference's own CPU operator sources
(SparQ/src/*.cpp of IAI-USTC-Quantum/SparQSim, compiled unmodified from the
read-only checkout at /root/reference) together with oracle/refshim/ (a
stand-in for the header of the absent git submodule extern/qram-simulator)
and oracle/reference_driver.cpp into oracle/_ref/libsparq_ref.so.

The library pins the oracle: tests/test_reference_pin_cpu.py runs the same
operations on both and compares them bit for bit. It is built only where the
reference checkout exists (this returns None elsewhere), never by the engine's
own build, and nothing outside tests/ loads it.

Not built from the reference: its cmake build (fmt, Eigen and the submodule
are absent), the CUDA sources, and the OpenMP variant (the sources select
single-threaded loops in global_macros.h, which is not overridden).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
REFERENCE = Path("/root/reference")
SPARQ = REFERENCE / "SparQ"
OUT = HERE / "_ref"
LIB = OUT / "libsparq_ref.so"

# the CPU operator path (SparQ/src): registers and systems, arithmetic, QRAM
# load, Hadamard, gates, conditional rotations, sorting, ClearZero/Normalize
SOURCES = ["basic_components", "system_operations", "quantum_arithmetic", "qram", "hadamard", "basic_gates",
           "condrot", "sort_state", "dark_magic", "debugger", "quantum_interfere_basic", "partial_trace", "rot",
           "parallel_phase_operations"]
FLAGS = ["-std=c++20", "-O2", "-fPIC", "-ffp-contract=off", "-w"]


def available() -> bool:
    return (SPARQ / "src").is_dir() and (SPARQ / "include").is_dir()


def _inputs():
    return ([SPARQ / "src" / f"{s}.cpp" for s in SOURCES] + list((HERE / "refshim").rglob("*")) +
            [HERE / "reference_driver.cpp", ROOT / "include" / "sparq_gb300.h", Path(__file__)])


def build(force: bool = False, verbose: bool = False) -> Path | None:
    """Compile into oracle/_ref/ and return the library's path (None when the
    reference checkout is absent)."""
    if not available():
        return None
    gxx = shutil.which("g++") or "g++"
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(p.stat().st_mtime for p in _inputs() if p.is_file()):
        return LIB
    OUT.mkdir(exist_ok=True)
    inc = ["-I" + str(HERE / "refshim"), "-I" + str(SPARQ / "include"), "-I" + str(ROOT / "include")]

    def compile_one(src: Path) -> Path:
        obj = OUT / (src.stem + ".o")
        r = subprocess.run([gxx, *FLAGS, *inc, "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stderr[-4000:]}")
        return obj

    srcs = [SPARQ / "src" / f"{s}.cpp" for s in SOURCES] + [HERE / "reference_driver.cpp"]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    r = subprocess.run([gxx, "-shared", "-fPIC", *map(str, objs), "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
    os.replace(tmp, LIB)
    for o in objs:
        o.unlink()
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
