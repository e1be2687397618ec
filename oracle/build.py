"""Build recipe of the oracle's shared library (test infrastructure only).

Compiles oracle/gfe_oracle.cpp with g++ into oracle/libgfe_oracle.so (parity build: plain -O3
without machine-specific flags and without FMA contraction, so the same recipe gives the same
results on x86_64 and aarch64 hosts) and oracle/libgfe_oracle_timing.so (the compiler's default
contraction; timed as the CPU baseline).
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "gfe_oracle.cpp"
LIB = HERE / "libgfe_oracle.so"
LIB_TIMING = HERE / "libgfe_oracle_timing.so"


def _compile(out: Path, extra: list[str]) -> Path:
    tmp = out.with_suffix(".so.tmp")
    cmd = ["g++", "-O3", "-std=c++17", *extra, "-fPIC", "-shared", "-pthread", str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build(force: bool = False) -> Path:
    """Both builds of the same source.  The parity build (returned) has no FMA contraction: Iron's
    FP64 arithmetic rounds every product, and the oracle must give the same bits on x86_64 (where
    -O3 has no FMA) and aarch64 (where contraction is the compiler's default).  The timing build
    keeps the compiler's default, as a normal build of the reference's code would, and is the one
    the CPU baseline times."""
    for out, extra in ((LIB, ["-ffp-contract=off"]), (LIB_TIMING, [])):
        if force or not out.exists() or out.stat().st_mtime < SRC.stat().st_mtime:
            _compile(out, extra)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
