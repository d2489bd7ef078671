"""pyoracle -- ctypes access to the CPU oracle (oracle/libdem_oracle.so) and,
where it was built, to the reference's own kernels compiled for the CPU
(oracle/_ref/libdem_ref.so).  TEST INFRASTRUCTURE: only tests/, smoke() and
bench.py's CPU-baseline leg use it, as the checker or the timed CPU baseline."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from gpucode_gb300 import _abi
from gpucode_gb300._abi import LIQUID, PARAMETER, MatType, calPara

ROOT = Path(__file__).resolve().parents[1]  # repository root
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "libdem_oracle.so"
REF_LIB = ORACLE_DIR / "_ref" / "libdem_ref.so"


def reference_dir() -> Path:
    """The reference's source tree: $DEM_REF_DIR when set, else the tree checked out
    beside this repository (../reference).  It may be absent (then only the oracle
    and the golden fixtures are available)."""
    env = os.environ.get("DEM_REF_DIR")
    return Path(env) if env else ROOT.parent / "reference"


REF_SRC = reference_dir()


class OConsts(C.Structure):
    _fields_ = [("mat", MatType * 2), ("lqd", LIQUID), ("prm", PARAMETER), ("cal", calPara), ("pwcal", calPara),
                ("lqd_mode", C.c_int), ("lqd_theta_max", C.c_float), ("lqd_vol_min", C.c_double),
                ("lqd_vol_max", C.c_double), ("lqd_seed", C.c_ulonglong)]


def _declare(lib: C.CDLL) -> C.CDLL:
    P, I, L = C.c_void_p, C.c_int, C.c_long
    lib.orc_sim_new.restype = P
    lib.orc_sim_new.argtypes = [I, I, I, L]
    lib.orc_sim_free.argtypes = [P]
    lib.orc_sim_ptr.restype = P
    lib.orc_sim_ptr.argtypes = [P, C.c_char_p]
    lib.orc_sim_set_mode.argtypes = [P, I, I]
    lib.orc_sim_step.restype = I
    lib.orc_sim_step.argtypes = [P]
    lib.orc_sim_counter.restype = L
    lib.orc_sim_counter.argtypes = [P, C.c_char_p]
    lib.orc_sim_request_rebuild.argtypes = [P]
    lib.orc_sim_set_counter.argtypes = [P, C.c_char_p, L]
    lib.orc_sim_set_kernels.argtypes = [P, P]
    lib.orc_fcap.restype = C.c_double
    lib.orc_fcap.argtypes = [C.c_double, C.c_double, C.c_double, P]
    if hasattr(lib, "orc_willett"):
        lib.orc_willett.restype = C.c_double
        lib.orc_willett.argtypes = [C.c_double, C.c_double, C.c_double]
        lib.orc_rupture.restype = C.c_double
        lib.orc_rupture.argtypes = [C.c_double, C.c_double]
        lib.orc_theta.restype = C.c_float
        lib.orc_theta.argtypes = [I, C.c_ulonglong, C.c_float]
        lib.orc_pair_volume.restype = C.c_double
        lib.orc_pair_volume.argtypes = [P, I, I, C.c_double]
    return lib


_oracle = None
_ref = None


def build_oracle() -> None:
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "all"], check=True)


def oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not ORACLE_LIB.exists():
            build_oracle()
        _oracle = _declare(C.CDLL(str(ORACLE_LIB)))
    return _oracle


def ref_available() -> bool:
    if REF_LIB.exists():
        return True
    if (REF_SRC / "kernel.cu").exists():
        r = subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "ref", f"REF_DIR={REF_SRC}"], capture_output=True)
        return r.returncode == 0 and REF_LIB.exists()
    return False


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        lib = _declare(C.CDLL(str(REF_LIB)))
        lib.ref_kernels.restype = C.c_void_p
        lib.ref_fcap.restype = C.c_double
        lib.ref_fcap.argtypes = [C.c_double, C.c_double, C.c_double, C.c_void_p]
        _ref = lib
    return _ref


def consts_of(setup) -> OConsts:
    s = setup.s
    k = OConsts()
    k.mat[0] = s.mat[0]
    k.mat[1] = s.mat[1]
    k.lqd = s.lqd
    k.prm = s.prm
    k.cal = s.cal
    k.pwcal = s.pwcal
    return k


class OracleSim:
    """A whole simulation in the reference's layouts on the CPU (main.cpp:433-568)."""

    def __init__(self, setup, pos, vel=None, angvel=None, use_ref_kernels: bool = False, lib=None):
        self.lib = lib or (ref() if use_ref_kernels else oracle())
        s = setup.s
        self.setup = setup
        self.n = setup.n
        self.slots = int(s.n_pp_slots)
        self.h = self.lib.orc_sim_new(self.n, s.n_levels, s.sys_ncells, self.slots)
        if use_ref_kernels:
            self.lib.orc_sim_set_kernels(self.h, self.lib.ref_kernels())
        k = consts_of(setup)
        C.memmove(self.lib.orc_sim_ptr(self.h, b"consts"), C.byref(k), C.sizeof(k))
        cyl = _abi.CylinderBC()
        C.memmove(C.byref(cyl), C.byref(s.cyl), C.sizeof(cyl))
        C.memmove(self.lib.orc_sim_ptr(self.h, b"cylinder"), C.byref(cyl), C.sizeof(cyl))
        L = s.n_levels
        self.arr("Level_size", np.float64, L)[:] = list(s.level_size)[:L]
        self.arr("level_nNebors", np.int32, L)[:] = list(s.level_nnebors)[:L]
        self.arr("level_nPars", np.int32, L)[:] = list(s.level_npars)[:L]
        self.arr("Ncell_Idx", np.int32, L)[:] = list(s.ncell_idx)[:L]
        self.arr("numCells", np.int32, L)[:] = list(s.num_cells)[:L]
        self.arr("Cellsize", np.float64, L)[:] = list(s.cell_size)[:L]
        gs = self.arr("gridSize", np.int32, 3 * L).reshape(L, 3)
        for l in range(L):
            gs[l] = (s.grid_size[l].x, s.grid_size[l].y, s.grid_size[l].z)
        self.arr("rad", np.float64, self.n)[:] = setup.rad
        self.arr("pLevel", np.int32, self.n)[:] = setup.plevel
        self.arr("Nebor_Idx", np.int32, self.n)[:] = setup.nidx
        self.set_state(pos, vel, angvel)
        self.lib.orc_sim_set_mode(self.h, int(s.force_cap), int(s.load_stage))

    def set_liquid_model(self, mode: int, vol_min: float = 0.0, vol_max: float = 0.0, theta_max: float = 0.0,
                         seed: int = 0) -> None:
        """the per-contact liquid model (mode 1) or the reference's (mode 0); the
        same parameters as the library's dem_set_liquid_model"""
        k = OConsts.from_address(self.lib.orc_sim_ptr(self.h, b"consts"))
        k.lqd_mode = int(mode)
        k.lqd_vol_min, k.lqd_vol_max = float(vol_min), float(vol_max)
        k.lqd_theta_max = float(theta_max)
        k.lqd_seed = int(seed)

    def arr(self, name: str, dtype, count: int) -> np.ndarray:
        p = self.lib.orc_sim_ptr(self.h, name.encode())
        if not p:
            raise KeyError(name)
        ct = {np.float64: C.c_double, np.int32: C.c_int}[dtype]
        return np.ctypeslib.as_array(C.cast(p, C.POINTER(ct)), shape=(count,))

    def vec(self, name: str) -> np.ndarray:
        return self.arr(name, np.float64, 3 * self.n).reshape(self.n, 3)

    def set_state(self, pos, vel=None, angvel=None) -> None:
        self.vec("pos")[:] = pos
        self.vec("vel")[:] = 0.0 if vel is None else vel
        self.vec("angvel")[:] = 0.0 if angvel is None else angvel
        self.lib.orc_sim_request_rebuild(self.h)

    def step(self, k: int = 1) -> int:
        r = 0
        for _ in range(k):
            r = self.lib.orc_sim_step(self.h)
            if r < 0:
                raise RuntimeError("oracle: neighbour-slot overflow")
        return r

    def counter(self, name: str) -> int:
        return int(self.lib.orc_sim_counter(self.h, name.encode()))

    def state(self) -> dict[str, np.ndarray]:
        return {k: self.vec(k).copy() for k in ("pos", "vel", "angvel", "force", "mom")}

    def slot_base(self) -> np.ndarray:
        s = self.setup.s
        base = np.zeros(s.n_levels, np.int64)
        acc = 0
        for l in range(s.n_levels):
            base[l] = acc
            acc += s.level_nnebors[l] * s.level_npars[l]
        return base

    def lists_flat(self) -> tuple[np.ndarray, np.ndarray]:
        """(counts, every particle's partners end to end: particle-major, list order)."""
        num = self.arr("Num_Nebor", np.int32, self.n).copy()
        _, _, sl = self.slots_of(num)
        return num, self.arr("Nebor1", np.int32, self.slots)[sl].copy()

    def lists(self) -> tuple[np.ndarray, list[np.ndarray]]:
        """(counts, per-particle partner arrays in list order)."""
        num, flat = self.lists_flat()
        return num, np.split(flat, np.cumsum(num)[:-1]) if self.n else []

    def history_flat(self) -> np.ndarray:
        """(used slots, 9) records, particle-major in list order: dispt xyz, nDsp,
        nDsp_mx, plstRad, plstDfm, stage, lqdBrg."""
        num = self.arr("Num_Nebor", np.int32, self.n)
        _, _, idx = self.slots_of(num)
        f = {k: self.arr("pp." + k, np.float64, self.slots) for k in ("nDsp", "nDsp_mx", "plstRad", "plstDfm")}
        disp = self.arr("pp.dispt", np.float64, 3 * self.slots).reshape(-1, 3)
        stage = self.arr("pp.stage", np.int32, self.slots)
        brg = self.arr("pp.lqdBrg", np.int32, self.slots)
        return np.column_stack([disp[idx], f["nDsp"][idx], f["nDsp_mx"][idx], f["plstRad"][idx],
                                f["plstDfm"][idx], stage[idx].astype(np.float64), brg[idx].astype(np.float64)])

    def history(self) -> list[np.ndarray]:
        """per-particle (count, 9) records: dispt xyz, nDsp, nDsp_mx, plstRad, plstDfm, stage; plus lqdBrg."""
        num = self.arr("Num_Nebor", np.int32, self.n)
        return np.split(self.history_flat(), np.cumsum(num)[:-1]) if self.n else []

    def slots_of(self, counts: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(particle, list position, slot) of every used neighbour slot."""
        s = self.setup.s
        base = self.slot_base()
        npars = np.array(list(s.level_npars)[: s.n_levels], np.int64)
        counts = np.asarray(counts, np.int64)
        ii = np.repeat(np.arange(self.n), counts)
        start = np.cumsum(counts) - counts
        kk = np.arange(len(ii), dtype=np.int64) - np.repeat(start, counts)
        L = self.setup.plevel[ii]
        return ii, kk, base[L] + kk * npars[L] + self.setup.nidx[ii]

    def load_state(self, pos, vel, angvel, pmove, lqd, counts, partners, rec, brg, nwall, wlist, wrec, flag, it):
        """Resume from another implementation's full state (reference layouts).
        partners, rec (8 columns) and brg hold the used slots end to end,
        particle-major in list order (the order of slots_of)."""
        n = self.n
        self.vec("pos")[:] = pos
        self.vec("vel")[:] = vel
        self.vec("angvel")[:] = angvel
        self.arr("pMove", np.float64, n)[:] = pmove
        self.arr("lqdCnt", np.int32, n)[:] = lqd
        self.arr("Num_Nebor", np.int32, n)[:] = counts
        _, _, sl = self.slots_of(counts)
        self.arr("Nebor1", np.int32, self.slots)[sl] = partners
        r = np.asarray(rec).reshape(-1, 8)
        self.arr("pp.dispt", np.float64, 3 * self.slots).reshape(-1, 3)[sl] = r[:, 0:3]
        for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
            self.arr("pp." + f, np.float64, self.slots)[sl] = r[:, 3 + c]
        self.arr("pp.stage", np.int32, self.slots)[sl] = r[:, 7].astype(np.int32)
        self.arr("pp.lqdBrg", np.int32, self.slots)[sl] = brg
        self.arr("nwall", np.int32, n)[:] = nwall
        self.arr("wlist", np.int32, 3 * n)[:] = np.asarray(wlist).reshape(-1)
        wr = np.asarray(wrec).reshape(n, 3, 8)
        for a in range(3):
            rows = a * n + np.arange(n)
            self.arr("pw.dispt", np.float64, 9 * n).reshape(-1, 3)[rows] = wr[:, a, 0:3]
            for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
                self.arr("pw." + f, np.float64, 3 * n)[rows] = wr[:, a, 3 + c]
            self.arr("pw.stage", np.int32, 3 * n)[rows] = wr[:, a, 7].astype(np.int32)
        self.lib.orc_sim_set_counter(self.h, b"flag", int(flag))
        self.lib.orc_sim_set_counter(self.h, b"iter", int(it))
        self.lib.orc_sim_set_counter(self.h, b"need_build", 0)

    def wall_records(self) -> np.ndarray:
        n = self.n
        out = np.zeros((n, 3, 8))
        for a in range(3):
            rows = a * n + np.arange(n)
            out[:, a, 0:3] = self.arr("pw.dispt", np.float64, 9 * n).reshape(-1, 3)[rows]
            for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
                out[:, a, 3 + c] = self.arr("pw." + f, np.float64, 3 * n)[rows]
            out[:, a, 7] = self.arr("pw.stage", np.int32, 3 * n)[rows]
        return out

    def close(self) -> None:
        if self.h:
            self.lib.orc_sim_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sim_arrays(sim: OracleSim) -> dict[str, np.ndarray]:
    """Every array of an oracle simulation that a step writes (for bit-for-bit comparison)."""
    n, S, C_ = sim.n, sim.slots, sim.setup.s.sys_ncells
    out = {k: sim.vec(k).copy() for k in ("pos", "vel", "angvel", "force", "mom")}
    out["rmom"] = sim.arr("rmom", np.float64, n).copy()
    out["pMove"] = sim.arr("pMove", np.float64, n).copy()
    for k in ("lqdCnt", "hash", "index", "Num_Nebor", "nwall"):
        out[k] = sim.arr(k, np.int32, n).copy()
    out["wlist"] = sim.arr("wlist", np.int32, 3 * n).copy()
    out["cellStart"] = sim.arr("cellStart", np.int32, C_).copy()
    out["cellEnd"] = sim.arr("cellEnd", np.int32, C_).copy()
    num, lists = sim.lists()
    out["lists"] = np.concatenate(lists) if lists else np.zeros(0, np.int32)
    hist = sim.history()
    out["hist"] = np.vstack(hist) if hist else np.zeros((0, 9))
    wl = {k: sim.arr("pw." + k, np.float64, 3 * n).copy() for k in ("nDsp", "nDsp_mx", "plstRad", "plstDfm")}
    for k, v in wl.items():
        out["pw." + k] = v
    out["pw.dispt"] = sim.arr("pw.dispt", np.float64, 9 * n).copy()
    return out
