"""Python handle on the native engine (dem_* C API of libdem_gb300).

Thin: every call goes straight to the C ABI; arrays cross as raw pointers to
NumPy buffers.  Units are the reference's reduced units on the device side.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import DemInput, DemOptions, DemSetup, DemStats, check, ptr


@dataclass
class Setup:
    """A derived set-up: dem_setup plus the per-particle radius (reduced),
    size level and level rank (the reference's Nebor_Idx)."""

    s: DemSetup
    rad: np.ndarray
    plevel: np.ndarray
    nidx: np.ndarray

    @property
    def n(self) -> int:
        return int(self.s.np)

    @classmethod
    def build(cls, inp: DemInput, dia_m: np.ndarray) -> "Setup":
        lib = _abi.load()
        dia = np.ascontiguousarray(dia_m, dtype=np.float64)
        n = int(inp.np)
        if dia.shape != (n,):
            raise ValueError(f"diameters: expected shape ({n},), got {dia.shape}")
        s = DemSetup()
        rad = np.zeros(n, np.float64)
        plevel = np.zeros(n, np.int32)
        nidx = np.zeros(n, np.int32)
        check(lib.dem_build_setup(C.byref(inp), ptr(dia), C.byref(s), ptr(rad), ptr(plevel), ptr(nidx)),
              "dem_build_setup")
        return cls(s, rad, plevel, nidx)

    @classmethod
    def from_files(cls, genfile: str) -> "Setup":
        """heyi.in-style keyword file (+ <genfile>_dia.dat) -> set-up."""
        lib = _abi.load()
        inp = DemInput()
        check(lib.dem_read_input(genfile.encode(), C.byref(inp), None), "dem_read_input")
        dia = np.zeros(inp.np, np.float64)
        check(lib.dem_read_input(genfile.encode(), C.byref(inp), ptr(dia)), "dem_read_input")
        return cls.build(inp, dia)

    def to_reduced(self, x_m: np.ndarray) -> np.ndarray:
        """SI lengths -> reduced lengths (divide by REALSIZE, UnitReduce.cpp:14)."""
        return np.asarray(x_m, np.float64) / self.s.unit.rlunit

    def memory(self, precision: str = "mixed", capillary: str = "formula") -> dict:
        """device bytes the engine allocates for this set-up (dem_memory_estimate)"""
        lib = _abi.load()
        m = _abi.DemMemory()
        check(lib.dem_memory_estimate(C.byref(self.s), C.byref(_options(precision, capillary)), C.byref(m)),
              "dem_memory_estimate")
        return {k: getattr(m, k) for k, _ in _abi.DemMemory._fields_}

    def scale_cells(self, factor: float) -> None:
        """multiply every level's cell size by factor >= 1 (dem_scale_cells)"""
        check(_abi.load().dem_scale_cells(C.byref(self.s), float(factor)), "dem_scale_cells")

    def fit_memory(self, budget_bytes: float, min_slots: int = 8, precision: str = "mixed",
                   capillary: str = "formula") -> float:
        """scale the neighbour slots so the engine fits budget_bytes (dem_fit_memory); returns the factor"""
        lib = _abi.load()
        f = C.c_double()
        check(lib.dem_fit_memory(C.byref(self.s), C.byref(_options(precision, capillary)), float(budget_bytes),
                                 int(min_slots), C.byref(f)), "dem_fit_memory")
        return f.value


def _options(precision: str = "mixed", capillary: str = "formula", reorder: bool = True, use_graph: bool = True,
             graph_steps: int = 0, block_size: int = 0, pairs: str = "auto") -> DemOptions:
    lib = _abi.load()
    opt = DemOptions()
    lib.dem_default_options(C.byref(opt))
    opt.precision = {"mixed": _abi.PREC_MIXED, "fp64": _abi.PREC_FP64}[precision]
    opt.capillary = {"formula": _abi.CAP_FORMULA, "mlp": _abi.CAP_MLP}[capillary]
    opt.reorder = 1 if reorder else 0
    opt.use_graph = 1 if use_graph else 0
    opt.graph_steps = int(graph_steps)
    opt.block_size = int(block_size)
    opt.pair_mode = {"auto": _abi.PAIRS_AUTO, "warp": _abi.PAIRS_WARP, "thread": _abi.PAIRS_THREAD}[pairs]
    return opt


def packing_metrics(setup: Setup, pos: np.ndarray) -> dict:
    """Packing fraction and mean coordination number of a bed (dem_packing_metrics)."""
    lib = _abi.load()
    p = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
    phi, z = C.c_double(), C.c_double()
    npb = C.c_int()
    check(lib.dem_packing_metrics(len(p), ptr(p), ptr(np.ascontiguousarray(setup.rad, np.float64)),
                                  C.byref(setup.s.cyl), C.byref(phi), C.byref(z), C.byref(npb)),
          "dem_packing_metrics")
    return {"phi": phi.value, "z": z.value, "n_probe": npb.value}


class Engine:
    """One simulation on one GPU (dem_ctx)."""

    def __init__(self, setup: Setup, precision: str = "mixed", reorder: bool = True, use_graph: bool = True,
                 capillary: str = "formula", graph_steps: int = 0, block_size: int = 0, pairs: str = "auto"):
        self.lib = _abi.load()
        self.setup = setup
        opt = _options(precision, capillary, reorder, use_graph, graph_steps, block_size, pairs)
        self.opt = opt
        h = C.c_void_p()
        check(self.lib.dem_create(C.byref(setup.s), ptr(setup.rad), ptr(setup.plevel), ptr(setup.nidx),
                                  C.byref(opt), C.byref(h)), "dem_create")
        self.h = h
        self.n = setup.n

    # ---- state ----
    def set_state(self, pos: np.ndarray, vel: np.ndarray | None = None, angvel: np.ndarray | None = None) -> None:
        p = np.ascontiguousarray(pos, np.float64).reshape(self.n, 3)
        v = None if vel is None else np.ascontiguousarray(vel, np.float64).reshape(self.n, 3)
        w = None if angvel is None else np.ascontiguousarray(angvel, np.float64).reshape(self.n, 3)
        check(self.lib.dem_set_state(self.h, ptr(p), None if v is None else ptr(v), None if w is None else ptr(w)),
              "dem_set_state")

    def get_state(self) -> dict[str, np.ndarray]:
        out = {k: np.zeros((self.n, 3), np.float64) for k in ("pos", "vel", "angvel", "force", "mom")}
        check(self.lib.dem_get_state(self.h, ptr(out["pos"]), ptr(out["vel"]), ptr(out["angvel"]),
                                     ptr(out["force"]), ptr(out["mom"])), "dem_get_state")
        return out

    def step(self, nsteps: int = 1) -> None:
        check(self.lib.dem_step(self.h, int(nsteps)), "dem_step")

    def sync(self) -> None:
        check(self.lib.dem_sync(self.h), "dem_sync")

    def stats(self) -> dict[str, float]:
        st = DemStats()
        check(self.lib.dem_get_stats(self.h, C.byref(st)), "dem_get_stats")
        return {k: getattr(st, k) for k, _ in DemStats._fields_ if k != "pad"}

    def stream(self) -> int:
        return int(self.lib.dem_stream(self.h) or 0)

    def step_chained(self) -> bool:
        """whether the steps launch one another on the device (after the first step)"""
        return bool(self.lib.dem_step_chained(self.h))

    def step_kernel_name(self) -> str:
        """the step kernel dem_step launches for this engine's options"""
        return self.lib.dem_step_kernel(self.h).decode()

    def neighbors(self, max_per: int = 256) -> tuple[np.ndarray, np.ndarray]:
        counts = np.zeros(self.n, np.int32)
        partners = np.full((self.n, max_per), -1, np.int32)
        check(self.lib.dem_get_neighbors(self.h, ptr(counts), ptr(partners), max_per), "dem_get_neighbors")
        return counts, partners

    def history(self, max_per: int = 256) -> tuple[np.ndarray, np.ndarray]:
        rec = np.zeros((self.n, max_per, 8), np.float64)
        brg = np.zeros((self.n, max_per), np.int32)
        check(self.lib.dem_get_history(self.h, ptr(rec), ptr(brg), max_per), "dem_get_history")
        return rec, brg

    # ---- learned capillary closure ----
    def set_capnet(self, net) -> None:
        """install a trained CapNet (the engine must use capillary="mlp")"""
        check(self.lib.dem_set_capnet(self.h, net.h), "dem_set_capnet")

    def set_liquid_model(self, mode: str = "per_contact", vol_min: float = 0.005, vol_max: float = 0.02,
                         theta_max: float = 0.5235987755982988, seed: int = 0) -> None:
        """dem_set_liquid_model: "reference" (the reference's per-particle liquid,
        zero contact angle) or "per_contact" (bridge volume a fraction in
        [vol_min, vol_max] of the smaller sphere, contact angle in [0, theta_max]
        radians per particle); before the first step"""
        m = _abi.DemLiquidModel()
        m.mode = {"reference": _abi.LIQUID_REFERENCE, "per_contact": _abi.LIQUID_PER_CONTACT}[mode]
        m.vol_min, m.vol_max, m.theta_max, m.seed = float(vol_min), float(vol_max), float(theta_max), int(seed)
        check(self.lib.dem_set_liquid_model(self.h, C.byref(m)), "dem_set_liquid_model")

    def set_contact_angles(self, theta_max_rad: float, seed: int = 0) -> None:
        check(self.lib.dem_set_contact_angles(self.h, float(theta_max_rad), int(seed)), "dem_set_contact_angles")

    # ---- batched systems ----
    def set_systems(self, system_of_particle: np.ndarray, cylinders: list, wet: np.ndarray | None = None) -> None:
        """independent packings stepped together (dem_set_systems); cylinders are
        CylinderBC structs in reduced units, one per system"""
        sysv = np.ascontiguousarray(system_of_particle, np.int32).reshape(self.n)
        arr = (_abi.CylinderBC * len(cylinders))(*cylinders)
        w = None if wet is None else np.ascontiguousarray(wet, np.int32).reshape(len(cylinders))
        check(self.lib.dem_set_systems(self.h, len(cylinders), ptr(sysv), C.cast(arr, C.c_void_p),
                                       None if w is None else ptr(w)), "dem_set_systems")

    def profile_kernels(self) -> list[tuple[str, float]]:
        """one step with a forced rebuild, timed kernel by kernel (dem_profile_kernels):
        [(kernel, device ms)] in launch order"""
        out = (_abi.DemKernelTime * 32)()
        n = C.c_int()
        check(self.lib.dem_profile_kernels(self.h, C.cast(out, C.c_void_p), 32, C.byref(n)), "dem_profile_kernels")
        return [(out[k].name.decode(), out[k].ms) for k in range(n.value)]

    def save(self, path: str | os.PathLike, nbatch: int = 1) -> None:
        check(self.lib.dem_save(self.h, str(path).encode(), nbatch), "dem_save")

    def load(self, path: str | os.PathLike) -> None:
        check(self.lib.dem_load(self.h, str(path).encode()), "dem_load")

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.dem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
