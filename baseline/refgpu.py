"""ctypes binding of baseline/refgpu.cu: the reference's own kernels, compiled
for sm_103a from its sources, run on this GPU in main.cpp:433-568's order.

A reported baseline for the benchmark, not part of the product."""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CUBIN = HERE / "_ref" / "ref_kernels.cubin"
LIB = HERE / "_ref" / "librefgpu.so"


class RefGpuStats(C.Structure):
    _fields_ = [("step_ms", C.c_double), ("force_ms", C.c_double), ("wall_ms", C.c_double),
                ("update_ms", C.c_double), ("rebuilds", C.c_int), ("overflow", C.c_int),
                ("contacts", C.c_longlong)]


def available() -> tuple[bool, str]:
    if not CUBIN.exists():
        return False, "the reference kernels' cubin was not built (it needs the reference sources)"
    return True, ""


def build_harness() -> None:
    if not LIB.exists() or LIB.stat().st_mtime < (HERE / "refgpu.cu").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "harness"], check=True)


def run(setup, pos: np.ndarray, vel: np.ndarray, ang: np.ndarray, warmup: int, steps: int,
        flush_ptr: int = 0, flush_bytes: int = 0) -> tuple[dict, np.ndarray]:
    """warmup untimed + steps timed reference steps from (pos, vel, ang) with empty
    histories; returns the per-step means and the final positions."""
    build_harness()
    lib = C.CDLL(str(LIB))
    P = C.c_void_p
    lib.refgpu_run.argtypes = [C.c_char_p, P, P, P, P, P, P, P, C.c_int, C.c_int, P, C.c_size_t, P,
                               C.POINTER(RefGpuStats)]
    lib.refgpu_run.restype = C.c_int
    lib.refgpu_last_error.restype = C.c_char_p
    n = setup.n
    arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(n, 3) for a in (pos, vel, ang)]
    rad = np.ascontiguousarray(setup.rad, dtype=np.float64)
    plevel = np.ascontiguousarray(setup.plevel, dtype=np.int32)
    nidx = np.ascontiguousarray(setup.nidx, dtype=np.int32)
    out = np.zeros((n, 3), np.float64)
    st = RefGpuStats()
    p = lambda a: a.ctypes.data_as(P)  # noqa: E731
    rc = lib.refgpu_run(str(CUBIN).encode(), C.cast(C.byref(setup.s), P), p(arrs[0]), p(arrs[1]), p(arrs[2]),
                        p(rad), p(plevel), p(nidx), warmup, steps, P(flush_ptr or None), flush_bytes, p(out),
                        C.byref(st))
    if rc != 0:
        raise RuntimeError(f"refgpu_run failed ({rc}): {lib.refgpu_last_error().decode()}")
    return {k: getattr(st, k) for k, _ in RefGpuStats._fields_}, out
