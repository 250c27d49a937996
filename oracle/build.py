"""Build the CPU oracle (test infrastructure): oracle/libsparq_oracle.so from
sparq_oracle.cpp with g++, no fused multiply-add (-ffp-contract=off)."""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "sparq_oracle.cpp"
LIB = HERE / "libsparq_oracle.so"


def build(force: bool = False) -> Path:
    header = ROOT / "include" / "sparq_gb300.h"
    if LIB.exists() and not force and LIB.stat().st_mtime >= max(SRC.stat().st_mtime, header.stat().st_mtime,
                                                                  Path(__file__).stat().st_mtime):
        return LIB
    cxx = shutil.which("g++") or "g++"
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I" + str(ROOT / "include"),
           str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(LIB)
