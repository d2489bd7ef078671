"""ctypes mirror of include/heydem_gb300.h and the loader of libdem_gb300.so.

The library is the product; this module only binds it.  Loading fails loudly
when the library has not been built: there is no Python or CPU fallback for
any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libdem_gb300.so"

MAX_LEVELS = 16

# status codes (heydem_gb300.h)
DEM_OK = 0
DEM_ERR_ARG = -1
DEM_ERR_CUDA = -2
DEM_ERR_OVERFLOW = -3
DEM_ERR_NONFINITE = -4
DEM_ERR_IO = -5
DEM_ERR_STATE = -6
DEM_ERR_NOMEM = -7
DEM_ERR_CELL = -8

PREC_FP64 = 0
PREC_MIXED = 1
CAP_FORMULA = 0
CAP_MLP = 1
PAIRS_AUTO = 0
PAIRS_WARP = 1
PAIRS_THREAD = 2


class double3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class int3(C.Structure):
    _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]


class CylinderBC(C.Structure):
    # double2 cir is 16-byte aligned in C: the struct is 64 bytes
    _fields_ = [("cir_x", C.c_double), ("cir_y", C.c_double), ("R", C.c_double), ("Tw", C.c_double),
                ("Bw", C.c_double), ("topv", C.c_double), ("btmv", C.c_double), ("_pad", C.c_double)]


class FeedZone(C.Structure):
    _fields_ = [("Lmax", C.c_double), ("Lmin", C.c_double)]


class UNIT(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("rlunit", "rmunit", "rfunit", "reunit", "rsunit", "rtunit", "rvunit")]


class MatType(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("density", "emod", "ymod", "pois", "dmpn", "sfrc", "rfrc", "yldp")]


class LIQUID(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("stension", "vol", "gapmn", "layer", "brknmx")]


class SIMULATION(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("dt", "dtFactor", "cutGap", "ctime", "simTime", "fdtime", "outtime",
                                          "dumptime", "outinterval", "fdinterval")] + \
               [("iter", C.c_int), ("Outs", C.c_int)]


class LOADMODE(C.Structure):
    _fields_ = [("stage", C.c_int), ("tPacking", C.c_double), ("nOutPacking", C.c_int)]


class PARAMETER(C.Structure):
    _fields_ = [("Origin", double3), ("EndPoint", double3), ("SearchGap", C.c_double), ("dt", C.c_double),
                ("NP", C.c_int)]


class calPara(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("emod", "pois", "sfrc", "ystress", "ydsp_t", "yforce_t", "ystiff_t")]


class SEARCHCELL(C.Structure):
    _fields_ = [("numCells", C.c_void_p), ("gridSize", C.c_void_p), ("Cellsize", C.c_void_p)]


class PPCONTACT_HISTORY(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("dispt", "ShrForB", "ShrMomB", "nOld", "nDsp", "nDsp_mx", "plstRad",
                                          "plstDfm", "bndRad", "NorForB", "NorMomB", "TenStrn", "ShrStrn",
                                          "stage", "lqdBrg", "Exbond")]


class PWCONTACT_HISTORY(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("dispt", "nDsp", "nDsp_mx", "plstRad", "plstDfm", "stage", "lqdBrg")]


class DemInput(C.Structure):
    _fields_ = [("np", C.c_int), ("n_levels", C.c_int), ("load_stage", C.c_int), ("t_packing", C.c_double),
                ("force_cap", C.c_int), ("real_size", C.c_double), ("cut_gap", C.c_double),
                ("expand_size", C.c_double), ("cyl_x", C.c_double), ("cyl_y", C.c_double), ("cyl_bw", C.c_double),
                ("cyl_r", C.c_double), ("cyl_h", C.c_double), ("feed_lmin", C.c_double), ("feed_lmax", C.c_double),
                ("mat", (C.c_double * 7) * 2), ("lqd", C.c_double * 3), ("dt_factor", C.c_double),
                ("n_out", C.c_int), ("level_input", C.c_int), ("level_dia", C.c_double * MAX_LEVELS),
                ("dt_override", C.c_double), ("gravity", C.c_double)]


class DemSetup(C.Structure):
    _fields_ = [("np", C.c_int), ("n_levels", C.c_int), ("force_cap", C.c_int), ("load_stage", C.c_int),
                ("init_par_size", C.c_double), ("_pad0", C.c_double), ("cyl", CylinderBC), ("feed", FeedZone),
                ("mat", MatType * 2), ("lqd", LIQUID), ("prm", PARAMETER), ("cal", calPara), ("pwcal", calPara),
                ("unit", UNIT), ("sim", SIMULATION), ("load", LOADMODE),
                ("level_size", C.c_double * MAX_LEVELS), ("level_nnebors", C.c_int * MAX_LEVELS),
                ("level_npars", C.c_int * MAX_LEVELS), ("cell_size", C.c_double * MAX_LEVELS),
                ("grid_size", int3 * MAX_LEVELS), ("num_cells", C.c_int * MAX_LEVELS),
                ("ncell_idx", C.c_int * MAX_LEVELS), ("sys_ncells", C.c_int), ("n_pp_slots", C.c_longlong),
                ("rad_min", C.c_double), ("rad_max", C.c_double), ("_pad1", C.c_double)]


class DemOptions(C.Structure):
    _fields_ = [("precision", C.c_int), ("capillary", C.c_int), ("block_size", C.c_int), ("reorder", C.c_int),
                ("use_graph", C.c_int), ("graph_steps", C.c_int), ("pair_mode", C.c_int)]


class DemStats(C.Structure):
    _fields_ = [("iter", C.c_longlong), ("rebuilds", C.c_longlong), ("nb_entries", C.c_longlong),
                ("contacts", C.c_longlong), ("bridges", C.c_longlong), ("wall_contacts", C.c_longlong),
                ("error_bits", C.c_int), ("pad", C.c_int), ("ctime", C.c_double), ("cap_mlp", C.c_longlong),
                ("cap_fallback", C.c_longlong)]


LIQUID_REFERENCE = 0
LIQUID_PER_CONTACT = 1


class DemLiquidModel(C.Structure):
    _fields_ = [("mode", C.c_int), ("pad", C.c_int), ("vol_min", C.c_double), ("vol_max", C.c_double),
                ("theta_max", C.c_double), ("seed", C.c_ulonglong)]


class DemMemory(C.Structure):
    _fields_ = [("per_particle", C.c_longlong), ("per_slot", C.c_longlong), ("per_cell", C.c_longlong),
                ("slots", C.c_longlong), ("total", C.c_longlong)]


class DemTuneSpace(C.Structure):
    _fields_ = [("n_skin", C.c_int), ("n_cell", C.c_int), ("n_block", C.c_int), ("pad", C.c_int),
                ("skin_scale", C.c_double * 8), ("cell_scale", C.c_double * 8), ("block_size", C.c_int * 4),
                ("warmup_steps", C.c_int), ("trial_steps", C.c_int)]


class DemTuneResult(C.Structure):
    _fields_ = [("skin_scale", C.c_double), ("cell_scale", C.c_double), ("block_size", C.c_int),
                ("n_tried", C.c_int), ("best_rate", C.c_double), ("rate", C.c_double * 64)]


class DemKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("ms", C.c_double)]


class CapnetFitOpts(C.Structure):
    _fields_ = [("epochs", C.c_int), ("batch", C.c_int), ("lr", C.c_float), ("val_frac", C.c_float),
                ("seed", C.c_ulonglong)]


class CapnetReport(C.Structure):
    _fields_ = [("epochs", C.c_int), ("n_train", C.c_int), ("n_val", C.c_int), ("pad", C.c_int),
                ("train_mse", C.c_float * 64), ("val_mse", C.c_float), ("val_force_rel_mean", C.c_float),
                ("val_force_rel_max", C.c_float), ("val_rupture_rel_max", C.c_float), ("seconds", C.c_double)]


# expected C layout, in the order dem_abi_layout reports it
_LAYOUT = [
    C.sizeof(CylinderBC), CylinderBC.R.offset, C.sizeof(MatType), C.sizeof(LIQUID), C.sizeof(PARAMETER),
    PARAMETER.SearchGap.offset, C.sizeof(calPara), C.sizeof(UNIT), C.sizeof(SIMULATION), C.sizeof(LOADMODE),
    C.sizeof(FeedZone), C.sizeof(DemInput), DemInput.mat.offset, DemInput.dt_override.offset, C.sizeof(DemSetup),
    DemSetup.cyl.offset, DemSetup.mat.offset, DemSetup.prm.offset, DemSetup.unit.offset, DemSetup.sim.offset,
    DemSetup.load.offset, DemSetup.level_size.offset, DemSetup.grid_size.offset, DemSetup.sys_ncells.offset,
    DemSetup.n_pp_slots.offset, DemSetup.rad_max.offset, C.sizeof(DemOptions), C.sizeof(DemStats),
    C.sizeof(PPCONTACT_HISTORY), C.sizeof(PWCONTACT_HISTORY), C.sizeof(SEARCHCELL), C.sizeof(DemLiquidModel),
    DemLiquidModel.seed.offset,
]

_lib = None


class DemError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: status {code}: {msg}")
        self.code = code


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libdem_gb300.so (RTLD_GLOBAL is not used) and check the struct layout."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is not built: run `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(the CUDA library is required; there is no fallback)")
    lib = C.CDLL(str(p))
    _declare(lib)
    buf = (C.c_longlong * 64)()
    n = lib.dem_abi_layout(buf, 64)
    got = list(buf[:n])
    if got != _LAYOUT:
        raise RuntimeError(f"libdem_gb300 struct layout mismatch: C {got} vs ctypes {_LAYOUT}")
    if path is None:
        _lib = lib
    return lib


def _declare(lib: C.CDLL) -> None:
    P = C.c_void_p
    I = C.c_int
    sig = {
        "dem_abi_layout": (I, [C.POINTER(C.c_longlong), I]),
        "dem_last_error": (C.c_char_p, []),
        "dem_version": (C.c_char_p, []),
        "dem_read_input": (I, [C.c_char_p, C.POINTER(DemInput), P]),
        "dem_build_setup": (I, [C.POINTER(DemInput), P, C.POINTER(DemSetup), P, P, P]),
        "dem_default_options": (None, [C.POINTER(DemOptions)]),
        "dem_create": (I, [C.POINTER(DemSetup), P, P, P, C.POINTER(DemOptions), C.POINTER(P)]),
        "dem_destroy": (I, [P]),
        "dem_set_state": (I, [P, P, P, P]),
        "dem_set_state_ex": (I, [P, P, P, P, I]),
        "dem_advance": (I, [P, P, P, P, P, I]),
        "dem_profile_step": (I, [P, I, P, C.c_size_t, C.POINTER(C.c_double)]),
        "dem_get_state": (I, [P, P, P, P, P, P]),
        "dem_step": (I, [P, I]),
        "dem_sync": (I, [P]),
        "dem_get_stats": (I, [P, C.POINTER(DemStats)]),
        "dem_stream": (P, [P]),
        "dem_step_chained": (I, [P]),
        "dem_step_kernel": (C.c_char_p, [P]),
        "dem_e2e_parts": (I, [P, P, P, P, P, I, P]),
        "dem_set_liquid_model": (I, [P, C.POINTER(DemLiquidModel)]),
        "dem_get_neighbors": (I, [P, P, P, I]),
        "dem_get_history": (I, [P, P, P, I]),
        "dem_get_aux": (I, [P, P, P, P, P, P, P]),
        "dem_save": (I, [P, C.c_char_p, I]),
        "dem_load": (I, [P, C.c_char_p]),
        "dem_set_feed_seed": (None, [C.c_ulonglong]),
        "dem_packing_metrics": (I, [I, P, P, P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(I)]),
        "dem_l2_flush": (I, [P, P, C.c_size_t]),
        "dem_compat_errors": (I, []),
        "dem_compat_set_precision": (I, [I]),
        "dem_compat_precision": (I, []),
        "dem_set_systems": (I, [P, I, P, P, P]),
        "dem_profile_kernels": (I, [P, P, I, C.POINTER(I)]),
        "dem_scale_cells": (I, [C.POINTER(DemSetup), C.c_double]),
        "dem_autotune": (I, [C.POINTER(DemInput), P, P, P, C.POINTER(DemOptions), C.POINTER(DemTuneSpace), I, P, P, P,
                             C.POINTER(DemSetup), C.POINTER(DemOptions), C.POINTER(DemTuneResult)]),
        "dem_pack_deposit": (I, [I, P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, I,
                                 C.c_ulonglong, P]),
        "dem_memory_estimate": (I, [C.POINTER(DemSetup), C.POINTER(DemOptions), C.POINTER(DemMemory)]),
        "dem_fit_memory": (I, [C.POINTER(DemSetup), C.POINTER(DemOptions), C.c_double, I, C.POINTER(C.c_double)]),
        "dem_capnet_create": (I, [C.c_ulonglong, C.POINTER(P)]),
        "dem_capnet_destroy": (None, [P]),
        "dem_capnet_get": (I, [P, P, P]),
        "dem_capnet_set": (I, [P, P, P]),
        "dem_capnet_samples": (I, [P, P, P, C.c_longlong, C.POINTER(C.c_longlong)]),
        "dem_capnet_fit": (I, [P, P, P, C.c_longlong, C.POINTER(CapnetFitOpts), C.POINTER(CapnetReport)]),
        "dem_capnet_grad": (I, [P, P, P, I, P, P]),
        "dem_capnet_infer": (I, [P, P, C.c_longlong, I, P]),
        "dem_capnet_formula": (I, [P, C.c_longlong, I, P]),
        "dem_set_capnet": (I, [P, P]),
        "dem_set_contact_angles": (I, [P, C.c_float, C.c_ulonglong]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def check(code: int, where: str) -> None:
    if code != DEM_OK:
        msg = load().dem_last_error().decode(errors="replace")
        raise DemError(code, where, msg)


def ptr(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return C.c_void_p(a.ctypes.data)
