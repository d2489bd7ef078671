"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own kernels (kernel.cu compiled for the CPU by
`make -C oracle ref`, in place from the reference tree) on the seeded parity
states of tests/_workloads.py and stores, per workload: the set-up (the
dem_setup bytes, radii, levels, level ranks), the start state, and every
array the step writes at a few checkpoints (after the first build, after
later rebuilds, at the end).  test_oracle_golden.py replays the oracle from
the stored inputs and compares.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
sys.path.insert(0, str(HERE.parent))

import _harness  # noqa: E402
import _workloads  # noqa: E402

CASES = {
    "pin_dry300": (_workloads.small_dry, 600, (1, 200, 600)),
    "pin_wet400": (_workloads.small_wet, 600, (1, 200, 600)),
}
KEEP = ("pos", "vel", "angvel", "force", "mom", "rmom", "pMove", "lqdCnt", "hash", "index", "Num_Nebor", "nwall",
        "wlist", "lists", "hist", "pw.dispt", "pw.nDsp", "pw.nDsp_mx", "pw.plstRad", "pw.plstDfm")


def main() -> None:
    if not _harness.ref_available():
        raise SystemExit("the reference sources are needed to regenerate the golden fixtures")
    for name, (make, steps, marks) in CASES.items():
        w = make()
        pos, vel, ang = _workloads.stirred(w)
        sim = _harness.OracleSim(w.setup, pos, vel, ang, use_ref_kernels=True)
        out = {
            "setup_bytes": np.frombuffer(C.string_at(C.addressof(w.setup.s), C.sizeof(w.setup.s)), np.uint8),
            "rad": w.setup.rad, "plevel": w.setup.plevel, "nidx": w.setup.nidx,
            "pos0": pos, "vel0": vel, "ang0": ang, "marks": np.array(marks),
        }
        for t in range(1, steps + 1):
            sim.step()
            if t in marks:
                arrs = _harness.sim_arrays(sim)
                for k in KEEP:
                    out[f"s{t}:{k}"] = arrs[k]
        out["rebuilds"] = np.array(sim.counter("rebuilds"))
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(name, "rebuilds", int(out["rebuilds"]), "bytes", (HERE / f"{name}.npz").stat().st_size)


if __name__ == "__main__":
    main()
