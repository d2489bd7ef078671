"""Make the packed 200,000-sphere wet bed (tests/golden/packed_wet200k.npz).

The bench's wet workload and the large-bed parity tests start from this bed, and
so does the benchmark's reference arm (the FP64 oracle on the host cores), which
reads it from the file and never loads the GPU library.

Recipe (needs a GPU; the library steps the bed):
  1. the wet workload's set-up and seeded sequential deposit (200,000 log-normal
     spheres, median 1 mm, sigma_ln 0.2 in [0.5, 2] mm, cylinder R = 25 mm): a
     loose bed, packing fraction ~0.39;
  2. the same spheres without friction, rolling resistance or liquid settle under
     gravity (dt 1e-6 s) until the packing fraction stops rising: frictionless
     spheres slide into the holes of the deposit and jam densely;
  3. the wet set-up itself (friction 0.3, capillary bridges, dt 5e-7 s) takes the
     bed over from rest for --wet-steps, so its bridges and springs form and the
     bed relaxes under them.
The file holds the final positions (float64, reduced units, caller order) and
the wet set-up (the dem_setup struct's bytes, the per-particle radius, size level
and level rank); the diameters are the wet workload's seeded draw
(configs.lognormal_diameters), which a reader can repeat to check the set-up.
Velocities and contact histories are not kept: a run starts from this bed at rest
with empty histories.

    python tests/golden/make_packed_bed.py --out tests/golden/packed_wet200k.npz
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(ROOT / "tests" / "golden" / "packed_wet200k.npz"))
    ap.add_argument("--n", type=int, default=200_000)
    ap.add_argument("--cyl-r", type=float, default=25e-3)
    ap.add_argument("--chunk", type=int, default=20_000, help="dry steps between packing-fraction checks")
    ap.add_argument("--max-dry-steps", type=int, default=1_200_000)
    ap.add_argument("--wet-steps", type=int, default=20_000)
    args = ap.parse_args()

    from gpucode_gb300 import configs
    from gpucode_gb300.engine import Engine, Setup, packing_metrics

    t0 = time.time()
    w = configs.wet(n=args.n, cyl_r=args.cyl_r)
    wi = w.inp
    # the same spheres and container without friction, rolling resistance or liquid
    prep = configs.make_input(wi.np, wi.n_levels, wi.real_size, wi.cut_gap, wi.cyl_r, wi.cyl_h, configs.RHO,
                              configs.E_YOUNG, configs.NU, 0.0, wi.mat[0][5], wi.mat[0][6], 0, dt=1e-6, rfrc=0.0)
    ps = Setup.build(prep, w.dia)
    e = Engine(ps, precision="mixed")
    e.set_state(w.pos0_reduced)
    log = []
    m0 = packing_metrics(w.setup, w.pos0_reduced)
    log.append({"phase": "deposit", "steps": 0, **m0})
    done, best = 0, m0["phi"]
    stall = 0
    while done < args.max_dry_steps:
        e.step(args.chunk)
        e.sync()
        done += args.chunk
        st = e.get_state()
        m = packing_metrics(w.setup, st["pos"])
        vmax = float(np.abs(st["vel"]).max())
        log.append({"phase": "dry", "steps": done, "vmax": vmax, **m})
        print(json.dumps(log[-1]), flush=True)
        stall = stall + 1 if m["phi"] < best * (1 + 2e-4) else 0
        best = max(best, m["phi"])
        if stall >= 3 and vmax < 0.05:
            break
    pos = e.get_state()["pos"]
    e.close()

    e = Engine(w.setup, precision="mixed")
    e.set_state(pos)
    for k in range(0, args.wet_steps, args.chunk):
        e.step(min(args.chunk, args.wet_steps - k))
        st = e.get_state()
        m = packing_metrics(w.setup, st["pos"])
        log.append({"phase": "wet", "steps": k + min(args.chunk, args.wet_steps - k),
                    "vmax": float(np.abs(st["vel"]).max()), **m})
        print(json.dumps(log[-1]), flush=True)
    pos = e.get_state()["pos"]
    e.close()
    s = w.setup
    np.savez_compressed(
        args.out, pos=pos.astype(np.float64), rad=s.rad, plevel=s.plevel, nidx=s.nidx,
        setup=np.frombuffer(C.string_at(C.addressof(s.s), C.sizeof(s.s)), np.uint8),
        setup_size=np.int64(C.sizeof(s.s)), log=np.array(json.dumps(log)),
        recipe=np.array(json.dumps({"n": args.n, "cyl_r_m": args.cyl_r, "dry_steps": done, "dry_dt_s": 1e-6,
                                    "wet_steps": args.wet_steps, "wet_dt_s": 5e-7, "seconds": time.time() - t0})))
    print(json.dumps({"out": args.out, "final": log[-1], "seconds": time.time() - t0}), flush=True)


if __name__ == "__main__":
    main()
