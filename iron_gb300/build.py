"""Build recipe of libgfe.so: every CUDA source of iron_gb300/csrc compiled for sm_103a.

The translation units are compiled in parallel (one nvcc per .cu) and linked into one shared
library next to this file, so the library is loaded from the source tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgfe.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgfe.so")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(objs: list[Path]) -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "gfe.h"]
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile all csrc/*.cu for sm_103a and link libgfe.so.  Returns the library path."""
    srcs = sources()
    BUILD.mkdir(exist_ok=True)
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    if not force and not _stale(objs):
        return LIB
    nvcc = _nvcc()
    flags = NVCC_FLAGS + ARCH + list(extra_flags or [])

    def compile_one(src: Path, obj: Path) -> str:
        cmd = [nvcc, *flags, "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        logs = list(ex.map(compile_one, srcs, objs))
    if verbose:
        for s, l in zip(srcs, logs):
            if l.strip():
                print(f"[{s.name}]\n{l}")
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link of libgfe.so failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
