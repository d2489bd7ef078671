"""The autotuner (dem_autotune of libdem_gb300): neighbour skin, cell size and
the step kernel's block size for a bed, chosen by timing short runs of the
engine itself on that bed."""
from __future__ import annotations

import copy
import ctypes as C

import numpy as np

from . import _abi
from ._abi import DemOptions, DemSetup, DemTuneResult, DemTuneSpace, check, ptr
from .engine import Setup, _options


def autotune(inp, dia, pos_reduced, vel_reduced=None, precision: str = "mixed", capillary: str = "formula",
             skins=(0.5, 1.0, 2.0), cells=(1.0, 1.3), blocks=(32, 64, 128), warmup: int = 20, trial: int = 200,
             systems=None) -> tuple[Setup, dict, dict]:
    """-> (the fastest set-up, Engine keyword options, report).  systems:
    (system_of_particle, cylinders, wet) for batched beds, else None."""
    lib = _abi.load()
    sp = DemTuneSpace()
    sp.n_skin, sp.n_cell, sp.n_block = len(skins), len(cells), len(blocks)
    for i, v in enumerate(skins):
        sp.skin_scale[i] = v
    for i, v in enumerate(cells):
        sp.cell_scale[i] = v
    for i, v in enumerate(blocks):
        sp.block_size[i] = v
    sp.warmup_steps, sp.trial_steps = warmup, trial
    n = int(inp.np)
    d = np.ascontiguousarray(dia, np.float64)
    p = np.ascontiguousarray(pos_reduced, np.float64).reshape(n, 3)
    v = None if vel_reduced is None else np.ascontiguousarray(vel_reduced, np.float64).reshape(n, 3)
    base = _options(precision, capillary)
    best_s, best_o, rep = DemSetup(), DemOptions(), DemTuneResult()
    ns, sysp, cylp, wetp = 0, None, None, None
    keep = []
    if systems is not None:
        sysv = np.ascontiguousarray(systems[0], np.int32)
        cyl = (_abi.CylinderBC * len(systems[1]))(*systems[1])
        keep += [sysv, cyl]
        ns, sysp, cylp = len(systems[1]), ptr(sysv), C.cast(cyl, C.c_void_p)
        if systems[2] is not None:
            w = np.ascontiguousarray(systems[2], np.int32)
            keep.append(w)
            wetp = ptr(w)
    check(lib.dem_autotune(C.byref(inp), ptr(d), ptr(p), None if v is None else ptr(v), C.byref(base), C.byref(sp),
                           ns, sysp, cylp, wetp, C.byref(best_s), C.byref(best_o), C.byref(rep)), "dem_autotune")
    # the chosen set-up with its per-particle tables
    chosen_in = copy.copy(inp)
    chosen_in.cut_gap = inp.cut_gap * rep.skin_scale
    setup = Setup.build(chosen_in, d)
    setup.scale_cells(rep.cell_scale)
    assert setup.s.sys_ncells == best_s.sys_ncells and setup.s.n_pp_slots == best_s.n_pp_slots
    table = []
    k = 0
    for s in skins:
        for c in cells:
            for b in blocks:
                table.append({"skin_scale": s, "cell_scale": c, "block_size": b, "particle_steps_per_s": rep.rate[k]})
                k += 1
    report = {"skin_scale": rep.skin_scale, "cell_scale": rep.cell_scale, "block_size": rep.block_size,
              "particle_steps_per_s": rep.best_rate, "trials": table}
    return setup, {"block_size": rep.block_size, "precision": precision, "capillary": capillary}, report
