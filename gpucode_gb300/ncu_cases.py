"""Small, host-launched cases of the hot kernels, for Nsight Compute captures.

Every kernel launch of these cases comes from the host (no CUDA graphs, no
device-launched steps), so a profiler's launch counting (-s / -c) addresses
them directly, and each case holds a few GB on the device at most.

    python -m gpucode_gb300.ncu_cases step [--pairs thread|warp] [--steps 4] [--io]
        the packed 200,000-sphere wet bed: `steps` host-launched mixed steps
        (the first rebuilds the lists); one step kernel per step; with --io
        then an export, an import and one more step through page-locked host
        arrays
    python -m gpucode_gb300.ncu_cases closure [--rows 1000000]
        the packed bed with the per-contact liquid model: a network trained
        for 3 epochs on the bridges of one step, 3 host-launched steps with it
        fused in the step kernel, then the network's inference on `rows`
        bridges: twice on the tcgen05 path, once on the warp tiles
    python -m gpucode_gb300.ncu_cases dropin [--precision fp64|mixed] [--steps 3]
        the packed bed through the reference's entry points in main.cpp's
        order (gpucode_gb300.dropin): `steps` steps, the first one building
        the lists, in the chosen mode of PpInterCalc / CirPWCalc / UpdateSystem
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
BED = ROOT / "tests" / "golden" / "packed_wet200k.npz"
LIQUID = {"vol_min": 0.005, "vol_max": 0.02, "theta_max": 0.5235987755982988, "seed": 2}


def step_case(pairs: str, steps: int, io: bool = False) -> None:
    from . import configs
    from .engine import Engine

    w = configs.load_bed(BED)
    e = Engine(w.setup, precision="mixed", use_graph=False, pairs=pairs)
    e.set_state(w.pos0_reduced)
    e.step(steps)
    e.sync()
    if io:
        # one end-to-end round trip through page-locked host arrays: the
        # state import and export kernels that read and write them directly
        import torch

        from ._abi import check, ptr

        n = w.setup.n
        h = [torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
        check(e.lib.dem_get_state(e.h, ptr(h[0]), ptr(h[1]), ptr(h[2]), None, None), "dem_get_state")
        check(e.lib.dem_set_state_ex(e.h, ptr(h[0]), ptr(h[1]), ptr(h[2]), 0), "dem_set_state_ex")
        e.step(1)
        check(e.lib.dem_get_state(e.h, ptr(h[0]), ptr(h[1]), ptr(h[2]), ptr(h[3]), None), "dem_get_state")
    print("ok", e.step_kernel_name(), e.stats())
    e.close()


def closure_case(rows: int) -> None:
    import torch

    from . import capnet as cn
    from . import configs
    from .engine import Engine

    w = configs.load_bed(BED)
    e = Engine(w.setup, precision="mixed", use_graph=False)
    e.set_liquid_model("per_contact", **LIQUID)
    e.set_state(w.pos0_reduced)
    e.step(1)
    x, y = cn.collect_samples(e, max(rows, 100_000))
    x, y = x.clone(), y.clone()
    e.close()
    net = cn.CapNet(seed=0)
    net.fit(x, y, epochs=3, batch=8192, lr=1e-3, val_frac=0.1, seed=1)
    m = Engine(w.setup, precision="mixed", capillary="mlp", use_graph=False)
    m.set_capnet(net)
    m.set_liquid_model("per_contact", **LIQUID)
    m.set_state(w.pos0_reduced)
    m.step(3)
    m.sync()
    big = x[:rows].contiguous()
    a = net.infer(big, "tcgen05")
    b = net.infer(big, "tcgen05")
    c = net.infer(big, True)
    torch.cuda.synchronize()
    print("ok", m.step_kernel_name(), m.stats(), "tcgen05 vs warp tiles", float((a - c).abs().max()),
          "repeat", float((a - b).abs().max()))
    m.close()
    net.close()


def dropin_case(precision: str, steps: int) -> None:
    import torch

    from . import configs
    from ._abi import check
    from .dropin import DropInDriver

    w = configs.load_bed(BED)
    z = w.pos0_reduced * 0.0
    drv = DropInDriver(w, w.pos0_reduced, z, z, torch)
    check(drv.lib.dem_compat_set_precision(1 if precision == "mixed" else 0), "dem_compat_set_precision")
    for _ in range(steps):
        drv.step()
    torch.cuda.synchronize()
    print("ok", precision, steps, "steps, compat errors", drv.lib.dem_compat_errors())


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case", choices=["step", "closure", "dropin"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--pairs", default="auto", choices=["auto", "warp", "thread"])
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--rows", type=int, default=1_000_000)
    ap.add_argument("--io", action="store_true", help="step: then a round trip through page-locked host arrays")
    a = ap.parse_args(argv)
    if a.case == "step":
        step_case(a.pairs, a.steps, a.io)
    elif a.case == "dropin":
        dropin_case(a.precision, a.steps)
    else:
        closure_case(a.rows)


if __name__ == "__main__":
    sys.exit(main())
