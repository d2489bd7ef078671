"""Build libdem_gb300.so in-tree with nvcc for sm_103a.

One shared library, compiled from a handful of translation units in parallel:
the FP64 reference-formula kernels (build.cu, step64.cu) are compiled with
-fmad=false so their arithmetic rounds like the CPU oracle's; the mixed
precision kernel keeps FMA contraction and takes the hardware FP32 square
root, division and exponentials (-use_fast_math: errors of a few ulp, far
below its FP32 force tolerance; its FP64 arithmetic is unaffected).  The
step-chaining unit launches graphs from the device and is the one unit built
with relocatable device code (nvcc's link step adds the device link).  No cmake, no torch extension: the
library exposes a plain C ABI (include/heydem_gb300.h).
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
OUT = PKG / "libdem_gb300.so"
BUILD = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, extra flags)
UNITS = [
    ("errors.cpp", []),
    ("host_io.cpp", []),
    ("metrics.cpp", []),
    ("build.cu", ["-fmad=false"]),
    ("step64.cu", ["-fmad=false"]),
    ("compat.cu", []),
    ("engine.cu", []),
    ("mixed.cu", ["-use_fast_math"]),
    ("capnet.cu", []),
    ("tune.cu", []),
    ("feed.cu", []),
    ("chain.cu", ["-rdc=true"]),
]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libdem_gb300")
    return exe


def _compile(src: str, extra: list[str], verbose: bool) -> Path:
    s = CSRC / src
    obj = BUILD / (src + ".o")
    cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
           "-I", str(INCLUDE), "-I", str(CSRC), *ARCH, *extra, "-c", str(s), "-o", str(obj)]
    if src.endswith(".cu"):
        cmd[1:1] = ["-x", "cu", "--expt-relaxed-constexpr"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def sources_newer_than(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    for p in list(CSRC.iterdir()) + list(INCLUDE.iterdir()) + [Path(__file__)]:
        if p.is_file() and p.stat().st_mtime > t:
            return True
    return False


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and return the path of libdem_gb300.so."""
    if not force and not sources_newer_than(OUT):
        return OUT
    BUILD.mkdir(exist_ok=True)
    units = [(s, f) for s, f in UNITS if (CSRC / s).exists()]
    with cf.ThreadPoolExecutor(max_workers=min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), units))
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudadevrt", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
