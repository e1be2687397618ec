"""Build recipe of the oracle's shared library (test infrastructure only).

Compiles oracle/gfe_oracle.cpp with g++ into oracle/libgfe_oracle.so.  Plain -O3 without
machine-specific flags and without FMA contraction, so the same recipe gives the same results on
x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "gfe_oracle.cpp"
LIB = HERE / "libgfe_oracle.so"


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and LIB.stat().st_mtime >= SRC.stat().st_mtime:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    # no FMA contraction: Iron's FP64 arithmetic rounds every product, and the oracle must give the
    # same bits on x86_64 (where -O3 has no FMA) and aarch64 (where contraction is the default)
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
