#!/usr/bin/env python
"""Benchmark: particle-steps/s of the wet polydisperse packing (200,000 spheres)
on one GB300, FP32-force / FP64-state path.

The bed is tests/golden/packed_wet200k.npz: the wet workload's 200,000
log-normal spheres (median 1 mm, sigma_ln 0.2 in [0.5, 2] mm, cylinder R =
25 mm, capillary bridges, dt 5e-7 s) packed to a packing fraction of 0.662 and
a mean coordination number of 6.6 (tests/golden/make_packed_bed.py), at rest,
contact histories empty.  Both arms read it from the file: --impl reference
runs the FP64 oracle (the reference's algorithm on the host cores) and never
loads the GPU library.  Each arm takes --warmup steps from the bed (the first
builds the neighbour lists), then times --steps steps.

One bench "step" is one DEM time step of the whole bed (rebuild when flagged,
p-p contact + capillary, wall contact, integration).  The timed steps run as a
run runs them: chained on the device in one dem_step call (each step graph
launches the next, the rebuild decided on the device), CUDA events around the
call.  A step moves ~233 MB through DRAM (ncu), more than the 129 MB L2, so the
timed region evicts nothing: inputs larger than L2 (a chained step measures
113.3 us, the step kernel alone with L2 evicted before it 113.8 us).  The same
steps launched one at a time with L2 evicted before each (a 256 MB write and a
256 MB read outside the per-step events) are reported beside it
(run.one_step_l2_evicted_ms_per_step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (launched by torchrun) every rank runs its own replica of the bed:
the path does not shard across GPUs here (replicas only); value sums all ranks'
particle-steps over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s, 200k wet spheres, vs FP64 plain; packing-frac & Z error"
UNIT = "particle-steps/s"
BED = ROOT / "tests" / "golden" / "packed_wet200k.npz"
DATA = "synthetic (seeded log-normal sizes, packed bed from tests/golden/packed_wet200k.npz)"
# the configured liquid: bridge volume per contact uniform in [0.5 %, 2 %] of the
# smaller sphere's volume, contact angle per particle uniform in [0, 30 deg]
LIQUID_CFG = {"vol_min": 0.005, "vol_max": 0.02, "theta_max": 0.5235987755982988, "seed": 2}


def bed_config(w) -> dict:
    """the workload both arms time (identical in both lines)"""
    return {"workload": "wet200k-packed", "particles": w.setup.n, "levels": int(w.setup.s.n_levels), "dt_s": 5e-7,
            "bed": "tests/golden/packed_wet200k.npz (phi 0.662, Z 6.6; at rest, empty histories)",
            "start": "warm-up steps from the bed (the first builds the lists), then the timed steps",
            "l2": "inputs larger than L2: one step moves ~233 MB through DRAM, the L2 holds 129 MB; no eviction"}


def _peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self, gpu_index: int = 0) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(gpu_index):
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def slowest(local: float, ws: int, device: str = "cuda") -> float:
    """the largest of every rank's value (a time): the job is as fast as its
    slowest replica"""
    if ws <= 1:
        return local
    import torch
    import torch.distributed as dist

    t = torch.tensor([local], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def algorithmic_bytes(n_nb: float, n_c: float, n_w: float, n_wall: float) -> float:
    """DRAM bytes one particle-step of the fused step kernel must move, from the
    per-particle counts of the step: the state read and written (position,
    velocity, spin, radius: 152), 4 per neighbour-list entry, 128 per p-p
    contact and per wall contact (the 64-byte record read and written), 16 per
    wet non-contact bridge (flag and volume)"""
    return 152 + 4 * n_nb + 128 * n_c + 16 * n_w + 128 * n_wall


def replica_rate(local_s: float, particles: int, steps: int, ws: int, device: str = "cuda") -> tuple[float, float]:
    """whole-job particle-steps/s of `ws` independent replicas, each stepping
    `particles` particles `steps` times: all ranks' particle-steps over the
    slowest rank's time; -> (rate, slowest time [s])"""
    t = slowest(local_s, ws, device)
    return ws * particles * steps / t, t


def cpu_oracle_rate(w, pos, steps: int, threads: int) -> tuple[float, str]:
    """The FP64 oracle (reference algorithm on the host cores, OpenMP) on the same bed."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    if not pyoracle.ORACLE_LIB.exists():
        pyoracle.build_oracle()
    sim = pyoracle.OracleSim(w.setup, pos)
    sim.step(1)  # first neighbour build, untimed
    t0 = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t0
    sim.close()
    return w.setup.n * steps / dt, f"{steps} steps of the {w.setup.n}-sphere bed after its first list build"


def run_reference(args, ws, rank):
    """The reference's algorithm (the FP64 oracle restating kernel.cu and the
    main.cpp step) on the host cores, on the same bed file as the GPU arm; the
    GPU library is not loaded."""
    if rank != 0:
        return
    from gpucode_gb300 import configs

    w = configs.load_bed(BED)
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    if not pyoracle.ORACLE_LIB.exists():
        pyoracle.build_oracle()
    sim = pyoracle.OracleSim(w.setup, w.pos0_reduced)
    sim.step(args.warmup)
    t0 = time.perf_counter()
    sim.step(args.steps)
    dt = time.perf_counter() - t0
    val = w.setup.n * args.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": DATA, "config": bed_config(w),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} steps of the full bed after {args.warmup} warm-up steps, on the "
                                   "host cores (FP64 oracle restating the reference kernels, pinned bit for bit to "
                                   "the reference's kernels compiled for the CPU)"},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def checksum(pos: np.ndarray) -> dict:
    """FP64 sum of x + 2y + 3z, and a hash of the positions rounded to 1e-9 reduced units"""
    p = np.asarray(pos, np.float64)
    r = np.round(p * 1e9).astype(np.int64)
    h = np.bitwise_xor.reduce((r[:, 0] * 73856093) ^ (r[:, 1] * 19349663) ^ (r[:, 2] * 83492791))
    return {"sum": float((p[:, 0] + 2 * p[:, 1] + 3 * p[:, 2]).sum()), "hash": int(h)}


def run_dry(args):
    """The dry monodisperse gravity packing (5,000 spheres, 20,000 steps of
    1e-6 s): this library's FP64 and mixed paths on the GPU and the oracle (the
    reference's algorithm, FP64, all host cores) on the same start, each run
    whole; packing fraction, coordination number and a positions checksum."""
    import torch

    from gpucode_gb300 import configs
    from gpucode_gb300.engine import Engine, packing_metrics

    w = configs.dry()
    n, steps = w.setup.n, args.dry_steps
    out = {}
    for prec in ("mixed", "fp64"):
        e = Engine(w.setup, precision=prec, pairs=args.pairs)
        e.set_state(w.pos0_reduced)
        e.step(16)
        e.sync()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.step(steps - 16)
        e.sync()
        dt = time.perf_counter() - t0
        pos = e.get_state()["pos"]
        st = e.stats()
        e.close()
        m = packing_metrics(w.setup, pos)
        out[prec] = {"particle_steps_per_s": n * (steps - 16) / dt, "wall_s": dt, "phi": m["phi"], "z": m["z"],
                     "n_probe": m["n_probe"], "rebuilds": st["rebuilds"], "checksum": checksum(pos)}
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    if not pyoracle.ORACLE_LIB.exists():
        pyoracle.build_oracle()
    sim = pyoracle.OracleSim(w.setup, w.pos0_reduced)
    t0 = time.perf_counter()
    sim.step(steps)
    dt = time.perf_counter() - t0
    pos = sim.state()["pos"]
    sim.close()
    m = packing_metrics(w.setup, pos)
    out["cpu_oracle"] = {"particle_steps_per_s": n * steps / dt, "wall_s": dt, "cores": threads, "phi": m["phi"],
                         "z": m["z"], "n_probe": m["n_probe"], "checksum": checksum(pos)}
    ref = out["cpu_oracle"]
    for prec in ("mixed", "fp64"):
        out[prec]["phi_rel_err_vs_oracle"] = abs(out[prec]["phi"] - ref["phi"]) / ref["phi"]
        out[prec]["z_rel_err_vs_oracle"] = abs(out[prec]["z"] - ref["z"]) / ref["z"]
    print(json.dumps({"metric": "particle-steps/s, 5k dry spheres, 20k steps; packing-frac & Z vs the oracle",
                      "workload": "dry5k", "particles": n, "steps": steps, "dt_s": 1e-6, "data": "synthetic "
                      "(seeded jittered hexagonal lattice)", "results": out}), flush=True)


def run_ensemble(args):
    """Batched ensemble: independent dry and wet packings of uneven sizes stepped
    together by the same launches, block size / cell size / skin picked by the
    autotuner on the batch; aggregate particle-steps/s, and each sampled
    system's packing fraction against the same system run alone."""
    import torch

    from gpucode_gb300 import configs
    from gpucode_gb300.autotune import autotune
    from gpucode_gb300.engine import Engine, packing_metrics

    t0 = time.perf_counter()
    e = configs.ensemble(n_systems=args.ens_systems, steps=args.ens_steps)
    t_build = time.perf_counter() - t0
    comb = e.combined
    systems = (e.system, e.cylinders, e.wet)
    t0 = time.perf_counter()
    setup, opts, tune = autotune(comb.inp, comb.dia, comb.pos0_reduced, None, skins=(0.5, 1.0, 2.0),
                                 cells=(1.0, 1.3), blocks=(32, 64, 128), warmup=10, trial=100, systems=systems)
    t_tune = time.perf_counter() - t0
    n = setup.n
    eng = Engine(setup, precision="mixed", block_size=opts["block_size"])
    eng.set_state(comb.pos0_reduced)
    eng.set_systems(*systems)
    eng.step(16)
    eng.sync()
    clk = Clocks()
    clk.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    eng.step(args.ens_steps - 16)
    eng.sync()
    dt = time.perf_counter() - t0
    ck = clk.stop()
    st = eng.stats()
    pos = eng.get_state()["pos"]
    eng.close()
    rl = setup.s.unit.rlunit
    picks = sorted(set(np.linspace(0, len(e.members) - 1, max(1, args.ens_alone)).astype(int).tolist()))
    per_sys, alone_steps, alone_time = [], 0, 0.0
    for k in picks:
        m = configs.member_setup(e.members[k])
        a = Engine(m.setup, precision="mixed")
        a.set_state(m.pos0_reduced)
        a.sync()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        a.step(args.ens_steps)
        a.sync()
        alone_time += time.perf_counter() - t1
        alone_steps += m.setup.n * args.ens_steps
        pa = a.get_state()["pos"]
        a.close()
        shift = np.array([e.offsets[k][0] / rl, e.offsets[k][1] / rl, 0.0])
        mb = packing_metrics(m.setup, pos[e.system == k] - shift)
        ma = packing_metrics(m.setup, pa)
        per_sys.append({"system": k, "particles": m.setup.n, "wet": int(e.wet[k]), "phi_batched": mb["phi"],
                        "phi_alone": ma["phi"], "phi_rel_diff": abs(mb["phi"] - ma["phi"]) / ma["phi"],
                        "z_batched": mb["z"], "z_alone": ma["z"]})
    diffs = [p["phi_rel_diff"] for p in per_sys]
    print(json.dumps({
        "metric": "aggregate particle-steps/s, batched ensemble of independent packings",
        "workload": f"ensemble{args.ens_systems}", "value": n * (args.ens_steps - 16) / dt, "unit": UNIT,
        "systems": args.ens_systems, "particles": n, "steps": args.ens_steps, "dt_s": 5e-7,
        "data": "synthetic (seeded per-system deposits, log-normal sizes, counts uniform in [1000, 50000])",
        "clocks": ck, "rebuilds": st["rebuilds"], "build_s": t_build, "autotune_s": t_tune, "autotune": tune,
        "device_bytes": setup.memory()["total"],
        "alone": {"systems_compared": len(per_sys), "particle_steps_per_s": alone_steps / max(alone_time, 1e-9),
                  "phi_rel_diff_mean": float(np.mean(diffs)), "phi_rel_diff_max": float(np.max(diffs)),
                  "per_system": per_sys}}), flush=True)


def train_closure(samples: int, epochs: int, settle: int = 2000, snaps: int = 11):
    """The learned capillary closure as the wet workloads deploy it: samples of
    the plain formula (the configured per-contact liquid, contact-angle terms
    included) logged from the packed 200,000-sphere wet bed over `settle`
    steps (`snaps` points), then trained on the GPU by the library's own
    kernels (seeded 90/10 split, Adam lr 1e-3, batch 8192).
    Returns (network, fit report, samples used)."""
    import torch

    from gpucode_gb300 import capnet as cn
    from gpucode_gb300 import configs
    from gpucode_gb300.engine import Engine

    w = configs.load_bed(BED)
    e = Engine(w.setup, precision="mixed")
    e.set_liquid_model("per_contact", **LIQUID_CFG)
    e.set_state(w.pos0_reduced)
    per = -(-samples // snaps)
    xs, ys = [], []
    e.step(settle - snaps * (settle // (snaps + 1)))
    for _ in range(snaps):
        e.step(settle // (snaps + 1))
        x, y = cn.collect_samples(e, per)
        xs.append(x.clone())
        ys.append(y.clone())
    e.close()
    x, y = torch.cat(xs).contiguous(), torch.cat(ys).contiguous()
    net = cn.CapNet(seed=0)
    rep = net.fit(x, y, epochs=epochs, batch=8192, lr=1e-3, val_frac=0.1, seed=2024)
    return net, rep, int(len(x))


def run_span(e, steps: int) -> tuple[float, dict]:
    """`steps` graph-replayed steps of engine e, timed on the host around a
    synchronised span (rebuilds included); -> (wall s, clocks)"""
    import torch

    e.sync()
    clk = Clocks()
    clk.start()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.step(steps)
    e.sync()
    dt = time.perf_counter() - t0
    return dt, clk.stop()


def closure_error(e, net, capacity: int = 8_000_000) -> dict:
    """per-contact error of the network against the plain formula it learned
    (FP64, the per-contact liquid model's regression with its contact-angle
    terms) over every bridge of engine e's current bed"""
    import torch

    from gpucode_gb300 import capnet as cn

    x, _ = cn.collect_samples(e, capacity)
    if len(x) == 0:
        return {"bridges": 0}
    # the step kernel evaluates the network only inside its training box (the
    # formula takes the rest): the error is the network's over those bridges
    _, norm = net.get()
    lo = torch.tensor(norm[12:16], device=x.device)
    hi = torch.tensor(norm[16:20], device=x.device)
    inside = ((x >= lo) & (x <= hi)).all(dim=1)
    n_all = len(x)
    x = x[inside].contiguous()
    if len(x) == 0:
        return {"bridges": n_all, "outside_training_box": n_all}
    yn = net.infer(x, True).double()
    yf = cn.formula(x, True, angle=True).double()
    fe = (yn[:, 0] - yf[:, 0]).abs() / yf[:, 0].abs().clamp_min(1e-30)
    re = (yn[:, 1] - yf[:, 1]).abs() / yf[:, 1].abs().clamp_min(1e-30)
    q = torch.tensor([0.5, 0.99, 0.999], dtype=torch.float64, device=fe.device)
    fq = torch.quantile(fe[: 10_000_000], q).tolist()
    return {"bridges": n_all, "outside_training_box": n_all - int(len(x)),
            "force_rel_err_mean": float(fe.mean()), "force_rel_err_p50": fq[0],
            "force_rel_err_p99": fq[1], "force_rel_err_p999": fq[2], "force_rel_err_max": float(fe.max()),
            "rupture_rel_err_mean": float(re.mean()), "rupture_rel_err_max": float(re.max())}


def run_wet_full(args):
    """The 200,000-sphere wet packing run whole (50,000 steps of 5e-7 s) three
    ways from the same packed bed, with the configured per-contact liquid:
    FP32 forces / FP64 state with the plain capillary formula, the same with
    the learned closure fused in the step kernel, and the all-FP64 engine (the
    reference's formulas with the contact-angle terms).  Packing fraction and
    coordination number at checkpoints along the run; the error of each fast
    path against the FP64 run at the end."""
    from gpucode_gb300 import configs
    from gpucode_gb300.engine import Engine, packing_metrics

    w = configs.load_bed(BED)
    n, total = w.setup.n, args.full_steps
    every = max(1, total // 5)
    net, rep, used = train_closure(args.capnet_samples, args.capnet_epochs)
    runs = {}
    for name, prec, cap in (("mixed_formula", "mixed", "formula"), ("mixed_mlp", "mixed", "mlp"),
                            ("fp64", "fp64", "formula")):
        e = Engine(w.setup, precision=prec, capillary=cap)
        if cap == "mlp":
            e.set_capnet(net)
        e.set_liquid_model("per_contact", **LIQUID_CFG)
        e.set_state(w.pos0_reduced)
        done, wall, marks, clocks = 0, 0.0, [], []
        while done < total:
            k = min(every, total - done)
            dt, ck = run_span(e, k)
            wall += dt
            done += k
            clocks.append(ck)
            m = packing_metrics(w.setup, e.get_state()["pos"])
            marks.append({"step": done, "phi": m["phi"], "z": m["z"], "n_probe": m["n_probe"]})
        st = e.stats()
        runs[name] = {"particle_steps_per_s": n * total / wall, "wall_s": wall, "rebuilds": st["rebuilds"],
                      "checkpoints": marks, "clocks": clocks[-1]}
        if cap == "mlp":
            runs[name]["network_evaluations"] = st["cap_mlp"]
            runs[name]["formula_fallbacks"] = st["cap_fallback"]
            runs[name]["closure_error_final_bed"] = closure_error(e, net)
        e.close()
    net.close()
    ref = runs["fp64"]["checkpoints"][-1]
    for name in ("mixed_formula", "mixed_mlp"):
        fin = runs[name]["checkpoints"][-1]
        runs[name]["phi_rel_err_vs_fp64"] = abs(fin["phi"] - ref["phi"]) / ref["phi"]
        runs[name]["z_rel_err_vs_fp64"] = abs(fin["z"] - ref["z"]) / max(ref["z"], 1e-300)
        runs[name]["speedup_vs_fp64"] = runs[name]["particle_steps_per_s"] / runs["fp64"]["particle_steps_per_s"]
    print(json.dumps({
        "metric": METRIC, "workload": "wet200k-full", "unit": UNIT, "particles": n, "steps": total, "dt_s": 5e-7,
        "data": DATA, "liquid": LIQUID_CFG,
        "timing": "host wall time around graph-replayed spans of steps, rebuilds included, metrics outside",
        "closure_training": {"samples": used, "epochs": rep["epochs"], "fit_seconds": rep["seconds"],
                             "val_force_rel_err_mean": rep["val_force_rel_mean"],
                             "val_force_rel_err_max": rep["val_force_rel_max"]},
        "targets": {"phi_rel_err": 0.002, "z_rel_err": 0.01}, "runs": runs}), flush=True)


def run_wet_large(args, which: str):
    """wet2m: 2,000,000 wet spheres in a 60 mm cylinder, 10,000 steps, the
    learned closure (trained on the 200,000-sphere bed's samples) fused in the
    step kernel with the plain formula outside its training box; per-contact
    error of the network against the formula on the final bed, and the same
    bed with the FP32 formula for comparison.
    wet16m: 16,000,000 wet spheres in a 150 mm cylinder, 5,000 steps, slots
    fitted to 180 GB, fused closure; the step kernel's HBM roofline on it; and
    packing fraction / coordination number of a 1,000,000-sphere sub-cylinder
    of the same set-up (37.5 mm: the same fill height) with the fused closure
    against its all-FP64 plain run."""
    import ctypes as C

    import torch

    from gpucode_gb300 import configs
    from gpucode_gb300._abi import check
    from gpucode_gb300.engine import Engine, packing_metrics

    net, rep, used = train_closure(args.capnet_samples, args.capnet_epochs)
    if which == "wet2m":
        n_big, r_big, steps = 2_000_000, 60e-3, args.large_steps or 10000
    else:
        n_big, r_big, steps = 16_000_000, 150e-3, args.large_steps or 5000
    t0 = time.perf_counter()
    w = configs.wet(n=n_big, cyl_r=r_big, steps=steps)
    t_gen = time.perf_counter() - t0
    fit = None
    if which == "wet16m":
        budget = 180e9
        full = w.setup.memory("mixed", "mlp")["total"]
        fit = {"budget_bytes": budget, "unfitted_bytes": full, "slot_factor": 1.0}
        if full > budget:
            fit["slot_factor"] = w.setup.fit_memory(budget, min_slots=8, precision="mixed", capillary="mlp")
        fit["device_bytes"] = w.setup.memory("mixed", "mlp")["total"]
        fit["slots_per_level"] = list(w.setup.s.level_nnebors)[: w.setup.s.n_levels]
    n = w.setup.n
    out = {}
    for name, cap in (("mixed_mlp", "mlp"), ("mixed_formula", "formula")):
        e = Engine(w.setup, precision="mixed", capillary=cap)
        if cap == "mlp":
            e.set_capnet(net)
        e.set_liquid_model("per_contact", **LIQUID_CFG)
        e.set_state(w.pos0_reduced)
        e.step(16)
        s0 = e.stats()
        dt, ck = run_span(e, steps - 16)
        s1 = e.stats()
        ps = n * (steps - 16)
        cnt = {k: (s1[k] - s0[k]) / ps for k in ("nb_entries", "contacts", "bridges", "wall_contacts")}
        bpp = algorithmic_bytes(cnt["nb_entries"], cnt["contacts"], cnt["bridges"], cnt["wall_contacts"])
        ms_k = C.c_double()
        check(e.lib.dem_profile_step(e.h, 5, None, 0, C.byref(ms_k)), "dem_profile_step")
        peak, peak_kind = _peaks()
        ach = n * bpp / (ms_k.value * 1e-3) / 1e9
        m = packing_metrics(w.setup, e.get_state()["pos"])
        r = {"particle_steps_per_s": ps / dt, "wall_s": dt, "rebuilds": s1["rebuilds"] - s0["rebuilds"],
             "clocks": ck, "per_step_counts": cnt, "phi": m["phi"], "z": m["z"], "n_probe": m["n_probe"],
             "roofline": {"kernel": e.step_kernel_name(), "kernel_ms": ms_k.value, "bytes_per_particle": bpp,
                          "achieved": ach, "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                          "frac": ach / peak, "l2": "working set far above L2 (no eviction needed)"}}
        if cap == "formula":
            r["kernels"] = kernel_table(e, n)
            r["kernels_note"] = ("one step with a forced rebuild timed kernel by kernel (CUDA events); DRAM bytes "
                                 "scaled from the 200,000-sphere ncu capture by particle count")
        if cap == "mlp":
            r["network_evaluations_per_step"] = (s1["cap_mlp"] - s0["cap_mlp"]) / (steps - 16)
            r["formula_fallback_fraction"] = (s1["cap_fallback"] - s0["cap_fallback"]) / max(
                1, (s1["cap_mlp"] - s0["cap_mlp"]) + (s1["cap_fallback"] - s0["cap_fallback"]))
            r["closure_error_final_bed"] = closure_error(e, net)
        out[name] = r
        e.close()
        torch.cuda.empty_cache()
    sub = None
    if which == "wet16m":
        ws_ = configs.wet(n=1_000_000, cyl_r=37.5e-3, steps=steps)
        sub = {"particles": ws_.setup.n, "cyl_r_m": 37.5e-3, "steps": steps}
        for name, prec, cap in (("mixed_mlp", "mixed", "mlp"), ("fp64", "fp64", "formula")):
            e = Engine(ws_.setup, precision=prec, capillary=cap)
            if cap == "mlp":
                e.set_capnet(net)
            e.set_liquid_model("per_contact", **LIQUID_CFG)
            e.set_state(ws_.pos0_reduced)
            dt, _ = run_span(e, steps)
            m = packing_metrics(ws_.setup, e.get_state()["pos"])
            sub[name] = {"particle_steps_per_s": ws_.setup.n * steps / dt, "phi": m["phi"], "z": m["z"],
                         "n_probe": m["n_probe"]}
            e.close()
        sub["phi_rel_err"] = abs(sub["mixed_mlp"]["phi"] - sub["fp64"]["phi"]) / sub["fp64"]["phi"]
        sub["z_rel_err"] = abs(sub["mixed_mlp"]["z"] - sub["fp64"]["z"]) / max(sub["fp64"]["z"], 1e-300)
    net.close()
    print(json.dumps({
        "metric": "particle-steps/s, wet spheres, fused learned capillary closure", "workload": which,
        "unit": UNIT, "particles": n, "steps": steps, "dt_s": 5e-7, "cyl_r_m": r_big,
        "data": "synthetic (seeded deposited bed, log-normal sizes)", "generate_s": t_gen,
        "timing": "host wall time around one graph-replayed span of steps after 16 warm-up, rebuilds included",
        "closure_training": {"samples": used, "epochs": rep["epochs"], "fit_seconds": rep["seconds"],
                             "bed": "the packed 200,000-sphere wet bed, per-contact liquid, 2,000 steps"},
        "memory_plan": fit, "runs": out, "sub_cylinder_vs_fp64": sub}), flush=True)


CELL_SORT = ("k_hash_count", "k_tile_sums", "k_scan_tiles", "k_cell_ranges", "k_scatter", "k_cell_order")


def kernel_bytes_per_particle() -> dict:
    """DRAM bytes per particle of each kernel of a rebuild + step, from the
    committed ncu table of the deposited 200,000-sphere bed (MB per launch /
    200,000; the large beds are deposited too); the cell sort's launches summed
    under the group name the library reports"""
    p = ROOT / "profiles" / "launches_deposit200k.md"
    out = {}
    if not p.exists():
        return out
    for line in p.read_text().splitlines():
        f = [x.strip() for x in line.strip().strip("|").split("|")]
        if len(f) == 6 and f[0].startswith("k_") and f[2].replace(".", "").isdigit():
            try:
                out[f[0]] = float(f[3]) * 1e6 / 200_000
            except ValueError:
                pass
    out["cell sort (k_hash_count .. k_cell_order)"] = sum(out.get(k, 0.0) for k in CELL_SORT)
    return out


def kernel_table(e, n: int) -> list:
    """one rebuild + step of engine e timed kernel by kernel, with achieved GB/s
    from the 200k bed's measured bytes per particle scaled to n particles"""
    bpp = kernel_bytes_per_particle()
    peak, _ = _peaks()
    rows = []
    for name, ms in e.profile_kernels():
        key = "k_step_coop<1,0>" if name == "step kernel" else name
        b = bpp.get(key)
        gbs = None if (b is None or ms <= 0) else b * n / (ms * 1e-3) / 1e9
        rows.append({"kernel": name, "ms": ms, "dram_bytes_scaled": None if b is None else b * n,
                     "achieved_gbs": gbs, "frac": None if gbs is None else gbs / peak})
    return rows


def traffic_from_profiles(kernel: str) -> float | None:
    """DRAM bytes per launch of the fused step kernel on the packed bed, from the
    committed ncu summary of the same kernel (None for a kernel without one)"""
    name = {"k_step_mixed<1,0>": "step_mixed_packed200k.md"}.get(kernel)
    if name is None:
        return None
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip())
            except ValueError:
                return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--profile-reps", type=int, default=20)
    ap.add_argument("--accuracy-steps", type=int, default=2000,
                    help="steps of the mixed and FP64 engines from the bed for the packing-fraction / Z errors "
                         "(0: skip)")
    ap.add_argument("--oracle-steps", type=int, default=300,
                    help="steps of the CPU oracle from the bed, compared with both engines (0: skip)")
    ap.add_argument("--capnet-samples", type=int, default=5_000_000,
                    help="training samples for the learned capillary closure, logged from the bed (0: skip it)")
    ap.add_argument("--capnet-epochs", type=int, default=20)
    ap.add_argument("--sample-steps", type=int, default=2000,
                    help="steps of the bed over which the closure's training samples are logged")
    ap.add_argument("--ref-gpu-steps", type=int, default=40,
                    help="timed steps of the reference's own kernels on this GPU (0: skip)")
    ap.add_argument("--host-steps", action="store_true",
                    help="launch every step's kernels directly instead of from CUDA graphs")
    ap.add_argument("--workload", default="wet200k",
                    choices=["wet200k", "wet200k-full", "dry5k", "ensemble", "wet2m", "wet16m"],
                    help="wet200k: the headline bench on the packed bed; wet200k-full: the wet deposit's whole "
                         "run, FP64 against the fast paths; dry5k: the dry lattice packing run whole on GPU and "
                         "CPU; ensemble: independent packings batched in one engine; wet2m / wet16m: large wet "
                         "beds with the fused learned closure")
    ap.add_argument("--pairs", default="auto", choices=["auto", "warp", "thread"],
                    help="pair loop of the step kernel: warp-cooperative, one thread per particle, or auto (the "
                         "library's choice)")
    ap.add_argument("--block-size", type=int, default=0, help="threads per block of the step kernel (0: default)")
    ap.add_argument("--full-steps", type=int, default=50000)
    ap.add_argument("--large-steps", type=int, default=0, help="steps of wet2m / wet16m (0: 10,000 / 5,000)")
    ap.add_argument("--dry-steps", type=int, default=20000)
    ap.add_argument("--ens-systems", type=int, default=256)
    ap.add_argument("--ens-steps", type=int, default=10000)
    ap.add_argument("--ens-alone", type=int, default=16, help="systems also run alone for the comparison")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank = _dist()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.workload == "dry5k":
        if rank == 0:
            run_dry(args)
        return
    if args.workload == "ensemble":
        if rank == 0:
            run_ensemble(args)
        return
    if args.workload == "wet200k-full":
        if rank == 0:
            run_wet_full(args)
        return
    if args.workload in ("wet2m", "wet16m"):
        if rank == 0:
            run_wet_large(args, args.workload)
        return
    run_headline(args, ws, rank)


def run_headline(args, ws, rank):
    import ctypes as C

    import torch

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")

    from gpucode_gb300 import configs
    from gpucode_gb300._abi import check, ptr
    from gpucode_gb300.engine import Engine, packing_metrics

    w = configs.load_bed(BED)
    n = w.setup.n
    pos0 = w.pos0_reduced

    eng = Engine(w.setup, precision="mixed", use_graph=not args.host_steps, graph_steps=1, pairs=args.pairs,
                 block_size=args.block_size)
    eng.set_state(pos0)
    # L2 eviction between timed steps: write 256 MB, then read another 256 MB,
    # so each step starts with a cold L2 holding clean, unrelated lines
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    eng.lib.dem_l2_flush.restype = C.c_int
    eng.lib.dem_l2_flush.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]

    def l2_flush(e):
        """evict L2 on engine e's stream, so the eviction finishes before e's next step starts"""
        check(e.lib.dem_l2_flush(C.c_void_p(e.stream()), C.c_void_p(flush.data_ptr()), flush.numel()),
              "dem_l2_flush")

    def timed_steps(e, steps, all_ranks=True):
        """`steps` steps of engine e chained on the device in one call (dem_step),
        as a run steps, CUDA events on its stream around the call; no L2 eviction:
        a step's working set is ~233 MB against the 129 MB L2 (the chained step
        measures the same as the step kernel alone with L2 evicted before it).
        Returns (ms total, wall s, clocks, stats before, after)"""
        st = torch.cuda.ExternalStream(e.stream())
        e.sync()
        before = e.stats()
        clk = Clocks()
        clk.start()
        if ws > 1 and all_ranks:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        e.step(steps)
        b.record(st)
        torch.cuda.synchronize()
        if ws > 1 and all_ranks:
            torch.distributed.barrier()
        wall = time.perf_counter() - t0
        ckk = clk.stop(local)
        e.sync()
        return a.elapsed_time(b), wall, ckk, before, e.stats()

    def one_step_evicted(e, steps):
        """the same steps launched one at a time, L2 evicted before each, CUDA
        events around each launch: ms per step"""
        st = torch.cuda.ExternalStream(e.stream())
        e.sync()
        tot = 0.0
        for _ in range(steps):
            l2_flush(e)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(st)
            e.step(1)
            b.record(st)
            b.synchronize()
            tot += a.elapsed_time(b)
        return tot / steps

    eng.step(args.warmup)
    ms, t_wall, ck, s0, s1 = timed_steps(eng, args.steps)
    value, t_slow = replica_rate(ms / 1000.0, n, args.steps, ws)
    ms = 1000.0 * t_slow
    one_step_ms = one_step_evicted(eng, args.steps)

    # measured pair counts per particle-step over the timed region
    d = {k: s1[k] - s0[k] for k in ("nb_entries", "contacts", "bridges", "wall_contacts", "rebuilds")}
    ps = n * args.steps
    n_nb, n_c, n_w, n_wall = d["nb_entries"] / ps, d["contacts"] / ps, d["bridges"] / ps, d["wall_contacts"] / ps
    bytes_per_particle = algorithmic_bytes(n_nb, n_c, n_w, n_wall)

    # the fused step kernel alone, cold L2 per launch
    ms_k = C.c_double()
    check(eng.lib.dem_profile_step(eng.h, args.profile_reps, C.c_void_p(flush.data_ptr()), flush.numel(),
                                   C.byref(ms_k)), "dem_profile_step")
    peak, peak_kind = _peaks()
    achieved = n * bytes_per_particle / (ms_k.value * 1e-3) / 1e9
    kname = eng.step_kernel_name()
    traffic = traffic_from_profiles(kname)
    rebuild = rebuild_cost(eng, n)

    # end to end through the public API with host buffers: H2D state, one step, D2H state + force
    e2e, e2e_parts = end_to_end(eng, n, args.e2e_steps, ws)
    eng.sync()

    # accuracy against FP64 runs of the reference's formulas from the same bed:
    # this library's FP64 engine (pinned to the oracle step by step) over a long
    # window, and the CPU oracle itself over a shorter one
    accuracy = None
    if rank == 0 and (args.accuracy_steps > 0 or args.oracle_steps > 0):
        accuracy = accuracy_runs(w, args, torch)
        nrb = accuracy.get("rebuilds_after_the_first", {}).get("mixed")
        if nrb is not None and args.accuracy_steps > 1:
            rebuild["rebuilds_in_accuracy_run"] = {"steps": args.accuracy_steps - 1, "rebuilds": nrb}
            rebuild["amortised_ms_per_step"] = rebuild["rebuild_ms"] * nrb / (args.accuracy_steps - 1)

    # the learned capillary closure: samples of the plain formula logged from
    # the bed, trained by the library's own kernels, then the same bed stepped
    # with the network fused in the step kernel (BF16 tensor-core tiles)
    closure = None
    liquid = None
    if rank == 0 and not args.host_steps:
        liquid = per_contact_liquid(w, args, timed_steps, flush)
    if rank == 0 and args.capnet_samples > 0 and not args.host_steps:
        closure = learned_closure(w, args, timed_steps, torch, flush)

    # the reference's own kernels (kernel.cu built for sm_103a) on this GPU, same bed
    ref_gpu = None
    if rank == 0 and args.ref_gpu_steps > 0:
        ref_gpu = reference_kernels(w, args, flush, value, closure, ms_k.value)

    if rank == 0:
        threads = os.cpu_count() or 1
        if args.cpu_steps > 0:
            cpu_val, cpu_sample = cpu_oracle_rate(w, pos0, args.cpu_steps, threads)
        else:
            cpu_val, cpu_sample = None, "skipped (--cpu-steps 0)"
        launches_per_step = 2  # fused step kernel + k_chain (each step graph launches the next)
        # a step that finds the rebuild request set: its gated step kernel + k_chain, then the rebuild graph
        # (clear request, bridge counts, copy_old, hash, 3 scan, scatter, order, permute, copy_back, shadows,
        # neighbour, wall list, carry, inverse), then the step again (counted in launches_per_step)
        rebuild_launches = 2 + 16
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32-force/f64-state", "data": DATA, "config": bed_config(w),
            "run": {"capillary": "formula", "pair_loop": kname, "parallelism": "replicas" if ws > 1 else "single",
                    "timing": "the timed steps chained on the device in one dem_step call, CUDA events around it",
                    "one_step_l2_evicted_ms_per_step": one_step_ms,
                    "per_step_counts": {"n_nb": n_nb, "n_c": n_c, "n_w": n_w, "n_wall": n_wall,
                                        "rebuilds": d["rebuilds"]},
                    "wall_s": t_wall},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": kname + " (fused contact + capillary + wall + integrate)",
                         "bytes_per_particle": bytes_per_particle, "kernel_ms": ms_k.value},
            "rebuild": rebuild,
            "cpu_baseline": {"value": cpu_val, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": cpu_sample},
            "contact_evaluations_per_s": value * n_c,
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": n * 72, "d2h_bytes_per_step": n * 96},
            "e2e_parts_ms": e2e_parts,
            "gpu_launches": launches_per_step * args.steps + rebuild_launches * d["rebuilds"],
            "clocks": ck,
            "accuracy_vs_fp64": accuracy,
            "reference_kernels_gpu": ref_gpu,
            "per_contact_liquid": liquid,
            "learned_closure": closure,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def rebuild_cost(eng, n: int) -> dict:
    """one forced rebuild of engine e timed kernel by kernel (its share of a step
    follows from the rebuild interval of a longer run: accuracy_runs)"""
    prof = eng.profile_kernels()
    ms = sum(t for name, t in prof if name != "step kernel")
    return {"rebuild_ms": ms, "kernels": {name: t for name, t in prof}}


def end_to_end(eng, n: int, steps: int, ws: int) -> tuple[float, dict]:
    """particle-steps/s through the public C-ABI with pinned host buffers, one
    step per round trip (state in, one step, state and force out): dem_advance,
    which queues the import, the step and the export and waits once; the same
    through the three calls dem_set_state_ex + dem_step + dem_get_state; and
    where the time of the three-call step goes (dem_e2e_parts)"""
    import ctypes as C

    import torch

    from gpucode_gb300._abi import check, ptr

    hp = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hv = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hw = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    hf = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
    check(eng.lib.dem_get_state(eng.h, ptr(hp), ptr(hv), ptr(hw), None, None), "dem_get_state")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        check(eng.lib.dem_advance(eng.h, ptr(hp), ptr(hv), ptr(hw), ptr(hf), 1), "dem_advance")
    e2e_t = time.perf_counter() - t0
    rate, _ = replica_rate(e2e_t, n, steps, ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        check(eng.lib.dem_set_state_ex(eng.h, ptr(hp), ptr(hv), ptr(hw), 0), "dem_set_state_ex")
        check(eng.lib.dem_step(eng.h, 1), "dem_step")
        check(eng.lib.dem_get_state(eng.h, ptr(hp), ptr(hv), ptr(hw), ptr(hf), None), "dem_get_state")
    three_t = time.perf_counter() - t0
    out = (C.c_double * 9)()
    check(eng.lib.dem_e2e_parts(eng.h, ptr(hp), ptr(hv), ptr(hw), ptr(hf), 10, out), "dem_e2e_parts")
    names = ["host_total", "dev_upload_copies", "dev_import_shadows", "dev_to_step_end", "dev_step_to_export",
             "dev_export_gather_copies", "host_in_set_state", "host_in_step", "host_in_get_state"]
    parts = {k: out[i] for i, k in enumerate(names)}
    parts["ms_per_step_dem_advance"] = 1000.0 * e2e_t / steps
    parts["ms_per_step_three_calls"] = 1000.0 * three_t / steps
    return rate, parts


def accuracy_runs(w, args, torch) -> dict:
    """packing fraction and coordination number of the mixed engine against
    FP64 runs of the reference's formulas from the same bed"""
    from gpucode_gb300.engine import Engine, packing_metrics

    out = {}
    runs = {}
    for name, prec in (("mixed", "mixed"), ("fp64", "fp64")):
        if args.accuracy_steps <= 0:
            break
        e = Engine(w.setup, precision=prec, use_graph=True)
        e.set_state(w.pos0_reduced)
        t0 = time.perf_counter()
        short = min(args.oracle_steps, args.accuracy_steps)
        if short > 0:
            e.step(short)
            runs[name + "_short"] = e.get_state()["pos"]
        e.step(args.accuracy_steps - short)
        e.sync()
        runs[name] = (e.get_state()["pos"], time.perf_counter() - t0)
        out.setdefault("rebuilds_after_the_first", {})[name] = int(e.stats()["rebuilds"]) - 1
        e.close()
    if runs:
        mm, mr = packing_metrics(w.setup, runs["mixed"][0]), packing_metrics(w.setup, runs["fp64"][0])
        out["engines"] = {"steps": args.accuracy_steps, "phi_mixed": mm["phi"], "phi_fp64": mr["phi"],
                          "phi_rel_err": abs(mm["phi"] - mr["phi"]) / mr["phi"], "z_mixed": mm["z"],
                          "z_fp64": mr["z"], "z_rel_err": abs(mm["z"] - mr["z"]) / max(mr["z"], 1e-300),
                          "n_probe": mr["n_probe"],
                          "fp64_particle_steps_per_s": w.setup.n * args.accuracy_steps / runs["fp64"][1],
                          "max_position_diff": float(np.abs(runs["mixed"][0] - runs["fp64"][0]).max())}
    if args.oracle_steps > 0:
        threads = os.cpu_count() or 1
        os.environ["OMP_NUM_THREADS"] = str(threads)
        sys.path.insert(0, str(ROOT / "oracle"))
        import pyoracle

        if not pyoracle.ORACLE_LIB.exists():
            pyoracle.build_oracle()
        sim = pyoracle.OracleSim(w.setup, w.pos0_reduced)
        t0 = time.perf_counter()
        sim.step(args.oracle_steps)
        t_or = time.perf_counter() - t0
        po = sim.state()["pos"]
        sim.close()
        mo = packing_metrics(w.setup, po)
        o = {"steps": args.oracle_steps, "phi_oracle": mo["phi"], "z_oracle": mo["z"], "cores": threads,
             "oracle_particle_steps_per_s": w.setup.n * args.oracle_steps / t_or}
        for name in ("mixed", "fp64"):
            key = name + "_short"
            if key in runs:
                m = packing_metrics(w.setup, runs[key])
                o[f"phi_{name}"] = m["phi"]
                o[f"z_{name}"] = m["z"]
                o[f"phi_rel_err_{name}"] = abs(m["phi"] - mo["phi"]) / mo["phi"]
                o[f"z_rel_err_{name}"] = abs(m["z"] - mo["z"]) / max(mo["z"], 1e-300)
                o[f"max_position_diff_{name}"] = float(np.abs(runs[key] - po).max())
        out["oracle"] = o
    return out


def per_contact_liquid(w, args, timed_steps, flush) -> dict:
    """The bed with the configured per-contact liquid model (FP32 formula with
    the contact-angle terms): step rate and kernel time, and packing fraction /
    coordination number against the FP64 engine with the same model"""
    import ctypes as C

    from gpucode_gb300._abi import check
    from gpucode_gb300.engine import Engine, packing_metrics

    n = w.setup.n
    e = Engine(w.setup, precision="mixed", graph_steps=1, pairs=args.pairs, block_size=args.block_size)
    e.set_liquid_model("per_contact", **LIQUID_CFG)
    e.set_state(w.pos0_reduced)
    e.step(args.warmup)
    ms, _, ck, s0, s1 = timed_steps(e, args.steps, all_ranks=False)
    ms_k = C.c_double()
    check(e.lib.dem_profile_step(e.h, args.profile_reps, C.c_void_p(flush.data_ptr()), flush.numel(),
                                 C.byref(ms_k)), "dem_profile_step")
    ps = n * args.steps
    out = {"model": LIQUID_CFG, "value": n * args.steps / (ms / 1000.0), "unit": UNIT,
           "ms_per_step": ms / args.steps, "kernel": e.step_kernel_name(), "kernel_ms": ms_k.value, "clocks": ck,
           "bridges_per_particle_step": (s1["bridges"] - s0["bridges"]) / ps,
           "contacts_per_particle_step": (s1["contacts"] - s0["contacts"]) / ps}
    e.close()
    if args.accuracy_steps > 0:
        pos = {}
        for prec in ("mixed", "fp64"):
            e = Engine(w.setup, precision=prec)
            e.set_liquid_model("per_contact", **LIQUID_CFG)
            e.set_state(w.pos0_reduced)
            e.step(args.accuracy_steps)
            pos[prec] = e.get_state()["pos"]
            e.close()
        mm, mr = packing_metrics(w.setup, pos["mixed"]), packing_metrics(w.setup, pos["fp64"])
        out["accuracy_vs_fp64"] = {"steps": args.accuracy_steps, "phi_mixed": mm["phi"], "phi_fp64": mr["phi"],
                                   "phi_rel_err": abs(mm["phi"] - mr["phi"]) / mr["phi"], "z_mixed": mm["z"],
                                   "z_fp64": mr["z"], "z_rel_err": abs(mm["z"] - mr["z"]) / max(mr["z"], 1e-300),
                                   "max_position_diff": float(np.abs(pos["mixed"] - pos["fp64"]).max())}
    return out


def learned_closure(w, args, timed_steps, torch, flush) -> dict:
    """The learned capillary closure under the configured per-contact liquid
    model: samples of the plain formula (with its contact-angle terms) logged
    from the bed, trained by the library's own kernels, then the bed stepped
    with the network fused in the step kernel"""
    import ctypes as C

    from gpucode_gb300 import capnet as cn
    from gpucode_gb300._abi import check
    from gpucode_gb300.engine import Engine, packing_metrics

    n = w.setup.n
    n_snap = 11
    per_snap = -(-args.capnet_samples // n_snap)
    xs, ys = [], []
    e = Engine(w.setup, precision="mixed")
    e.set_liquid_model("per_contact", **LIQUID_CFG)
    e.set_state(w.pos0_reduced)
    gap = max(1, args.sample_steps // (n_snap + 1))
    e.step(args.sample_steps - n_snap * gap)
    for _ in range(n_snap):
        e.step(gap)
        x, y = cn.collect_samples(e, per_snap)
        xs.append(x.clone())
        ys.append(y.clone())
    e.close()
    x = torch.cat(xs).contiguous()
    y = torch.cat(ys).contiguous()
    xs, ys = [], []
    net = cn.CapNet(seed=0)
    rep = net.fit(x, y, epochs=args.capnet_epochs, batch=8192, lr=1e-3, val_frac=0.1, seed=2024)
    em = Engine(w.setup, precision="mixed", capillary="mlp", graph_steps=1, pairs=args.pairs,
                block_size=args.block_size)
    em.set_capnet(net)
    em.set_liquid_model("per_contact", **LIQUID_CFG)
    em.set_state(w.pos0_reduced)
    em.step(args.warmup)
    ms_m, _, ck_m, m0, m1 = timed_steps(em, args.steps, all_ranks=False)
    value_m = n * args.steps / (ms_m / 1000.0)
    ms_km = C.c_double()
    check(em.lib.dem_profile_step(em.h, args.profile_reps, C.c_void_p(flush.data_ptr()), flush.numel(),
                                  C.byref(ms_km)), "dem_profile_step")
    kname = em.step_kernel_name()
    evals, falls = m1["cap_mlp"] - m0["cap_mlp"], m1["cap_fallback"] - m0["cap_fallback"]
    em.close()

    def per_call_ms(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps

    big = x[: min(len(x), 2_000_000)].contiguous()
    nb = len(big)
    rates = {"network_bf16_tensor_cores": nb / per_call_ms(lambda: net.infer(big, True)) * 1e3,
             "network_fp32": nb / per_call_ms(lambda: net.infer(big, False)) * 1e3,
             "formula_fp64": nb / per_call_ms(lambda: cn.formula(big, True, angle=True)) * 1e3,
             "formula_fp32_step_kernel": nb / per_call_ms(lambda: cn.formula(big, False, angle=True)) * 1e3}
    yn = net.infer(big, True).double()
    yf = cn.formula(big, True, angle=True).double()
    y32 = cn.formula(big, False, angle=True).double()
    rel = lambda a, b: ((a[:, 0] - b[:, 0]).abs() / b[:, 0].abs().clamp_min(1e-30))  # noqa: E731
    errors = {"network_force_rel_err_mean": float(rel(yn, yf).mean()),
              "network_force_rel_err_max": float(rel(yn, yf).max()),
              "fp32_formula_force_rel_err_mean": float(rel(y32, yf).mean()),
              "fp32_formula_force_rel_err_max": float(rel(y32, yf).max())}
    net.close()
    return {"value": value_m, "unit": UNIT, "ms_per_step": ms_m / args.steps, "kernel": kname,
            "kernel_ms": ms_km.value, "clocks": ck_m, "samples": len(x), "epochs": rep["epochs"],
            "fit_seconds": rep["seconds"], "val_mse_standardised": rep["val_mse"],
            "val_force_rel_err_mean": rep["val_force_rel_mean"], "val_force_rel_err_max": rep["val_force_rel_max"],
            "val_rupture_rel_err_max": rep["val_rupture_rel_max"], "rebuilds": m1["rebuilds"] - m0["rebuilds"],
            "network_evaluations_per_step": evals / args.steps,
            "formula_fallback_fraction": falls / max(evals + falls, 1), "evaluations_per_s": rates,
            "errors_vs_fp64_formula": errors, "model": LIQUID_CFG}


def reference_kernels(w, args, flush, value, closure, kernel_ms) -> dict:
    """the reference's kernel.cu, built for sm_103a, driven in main.cpp's step
    order from the same bed (after the same warm-up) on this GPU"""
    from baseline import refgpu

    from gpucode_gb300.engine import Engine

    n = w.setup.n
    ok, why = refgpu.available()
    if not ok:
        return {"unavailable": why}
    e = Engine(w.setup, precision="mixed")
    e.set_state(w.pos0_reduced)
    e.step(args.warmup)
    stt = e.get_state()
    e.close()
    try:
        r, _ = refgpu.run(w.setup, stt["pos"], stt["vel"], stt["angvel"], 5, args.ref_gpu_steps,
                          flush.data_ptr(), flush.numel())
    except RuntimeError as ex:
        return {"unavailable": str(ex)}
    rv = n / (r["step_ms"] * 1e-3)
    drop_in = {p: drop_in_path(w, stt, args, flush, p) for p in ("fp64", "mixed")}
    for d in drop_in.values():
        d["vs_reference_kernels"] = d["value"] / rv
    return {"value": rv, "unit": UNIT, "ms_per_step": r["step_ms"], "drop_in_path": drop_in["fp64"],
            "drop_in_path_mixed": drop_in["mixed"],
            "kernel_ms": {"PPForceCalcG": r["force_ms"], "CirPWInterG": r["wall_ms"],
                          "UpdateSystemG": r["update_ms"]},
            "rebuilds": r["rebuilds"], "slot_overflow": bool(r["overflow"]), "speedup": value / rv,
            "speedup_with_learned_closure": closure["value"] / rv if closure else None,
            "kernel_speedup": (r["force_ms"] + r["wall_ms"] + r["update_ms"]) / kernel_ms,
            "sample": f"{args.ref_gpu_steps} steps after 5 warm-up from the bed after {args.warmup} steps of this "
                      "library, histories empty, L2 evicted before each step, main.cpp step order (per-step flag "
                      "read, VarInit memsets)"}


def drop_in_path(w, stt, args, flush, precision: str) -> dict:
    """the reference's API driven in main.cpp's order (gpucode_gb300.dropin:
    what the reference's unchanged main.cpp gets from this library; "fp64"
    the default FP64 kernels, "mixed" what DEM_COMPAT_PRECISION=mixed selects)
    from the same state as the reference's kernels, timed the same way: L2
    evicted before each step, CUDA events around it, the per-step flag read
    included"""
    import ctypes as C

    import torch

    from gpucode_gb300._abi import check
    from gpucode_gb300.dropin import DropInDriver

    n = w.setup.n
    drv = DropInDriver(w, stt["pos"], stt["vel"], stt["angvel"], torch)
    lib = drv.lib
    check(lib.dem_compat_set_precision(1 if precision == "mixed" else 0), "dem_compat_set_precision")
    try:
        for _ in range(5):
            drv.step()
        torch.cuda.synchronize()
        tot, rebuilds = 0.0, 0
        for _ in range(args.ref_gpu_steps):
            check(lib.dem_l2_flush(None, C.c_void_p(flush.data_ptr()), flush.numel()), "dem_l2_flush")
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            rebuilds += int(drv.step())
            b.record()
            b.synchronize()
            tot += a.elapsed_time(b)
    finally:
        check(lib.dem_compat_set_precision(0), "dem_compat_set_precision")
    ms = tot / args.ref_gpu_steps
    return {"value": n / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "rebuilds": rebuilds,
            "precision": precision,
            "sample": f"{args.ref_gpu_steps} steps after 5 warm-up, the same state and method as the reference's "
                      f"kernels ({precision} kernels behind heydem.h's API, main.cpp's step order)"}


if __name__ == "__main__":
    main()
