"""Parity at the benchmark's sizes, against the oracle.

* The packed 200,000-sphere wet bed (tests/golden/packed_wet200k.npz: 4 size
  levels, ~20.6 M neighbour slots, 6.6 contacts per sphere):
  - the reference-compatible entry points driven in main.cpp's order (the
    first step builds the lists): sorted hashes and indices, CellStart /
    CellEnd and every neighbour slot bit-exact against the oracle
    (kernel.cu:617-855), forces, state and histories to 1e-12 (FP64 mode) or
    within the mixed tolerances (mixed mode), for a few steps in lockstep;
  - the native engine in both precisions after 20 steps from the bed, a
    rebuild forced by re-importing its own state, then steps in lockstep with
    the oracle (tests/_lockstep.py): lists bit-exact after the rebuild, FP64 to
    1e-12, mixed to the mixed tolerances;
  - packing fraction and coordination number of the mixed engine against the
    FP64 engine after 2,000 steps: within 0.2 % and 1 %.
* The dry 5,000-sphere lattice (20,000 steps of 1e-6 s; the lattice starts
  2 mm above the floor and falls freely for 20.2 ms, so the configured run ends
  just before its first layer lands): the whole run free-running on the FP64
  engine, the mixed engine and the oracle, with packing fraction, coordination
  number and a positions checksum compared; and the FP64 engine in lockstep
  with the oracle over 600 steps past the configured run, in which the first
  layer lands on the floor."""
from pathlib import Path

import numpy as np
import pytest

import _harness
import _lockstep
from gpucode_gb300 import _abi, configs
from gpucode_gb300.engine import Engine, packing_metrics

pytestmark = pytest.mark.gpu

BED = Path(__file__).resolve().parent / "golden" / "packed_wet200k.npz"
FP64_TOL = {"force": 1e-12, "pos": 1e-14, "vel": 1e-12, "hist": 1e-12}
MIXED_TOL = {"force": 2e-5, "pos": 1e-9, "vel": 1e-5, "angvel": 2e-5, "hist": 1e-5}


@pytest.fixture(scope="module")
def bed():
    return configs.load_bed(BED)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_drop_in_entry_points_at_200k_match_the_oracle(cuda, bed, precision):
    """the reference's entry points in main.cpp's order, in either mode of
    PpInterCalc / CirPWCalc / UpdateSystem (dem_compat_set_precision): the
    list build bit-exact in both, the step to 1e-12 (FP64, from the bed at
    rest) or within the mixed tolerances with at most 1 % of stage or bridge
    labels flipped (mixed, from the bed after 20 steps of the mixed engine, as
    the engine's own mixed lockstep starts: at exact rest every contact sits
    on its loading turning point, where FP32 and FP64 pick the load stage
    differently for many contacts at once)"""
    import torch

    from test_gpu_compat import FP64_TOL as COMPAT_TOL
    from test_gpu_compat import RefDriver, _declare, _load_oracle_from, _snap

    w = bed
    n = w.setup.n
    lib = _abi.load()
    _declare(lib)
    mixed = precision == "mixed"
    tol, budget = (MIXED_TOL, 0.01) if mixed else (COMPAT_TOL, 0.0)
    _abi.check(lib.dem_compat_set_precision(1 if mixed else 0), "dem_compat_set_precision")
    try:
        pos = w.pos0_reduced
        vel = ang = np.zeros_like(pos)
        if mixed:
            eng = Engine(w.setup, precision="mixed")
            eng.set_state(pos)
            eng.step(20)
            st = eng.get_state()
            eng.close()
            pos, vel, ang = (np.ascontiguousarray(st[k]) for k in ("pos", "vel", "angvel"))
        drv = RefDriver(w, pos, vel, ang, torch)
        sim = _harness.OracleSim(w.setup, pos, vel, ang)
        g = lambda x: x.detach().cpu().numpy()  # noqa: E731
        for t in range(3):
            torch.cuda.synchronize()
            _load_oracle_from(drv, sim)
            rb = sim.step()
            ra = drv.step()
            torch.cuda.synchronize()
            assert ra == bool(rb), f"rebuild decision differs at step {t}"
            if t == 0:
                assert rb
                assert np.array_equal(g(drv.hash), sim.arr("hash", np.int32, n))
                assert np.array_equal(g(drv.index), sim.arr("index", np.int32, n))
                assert np.array_equal(g(drv.cs), sim.arr("cellStart", np.int32, drv.C))
                assert np.array_equal(g(drv.ce), sim.arr("cellEnd", np.int32, drv.C))
            _lockstep.compare_step(_snap(drv, sim, w), sim, w, tol, f"step {t}", mismatch_budget=budget)
        assert g(drv.num).mean() > 8.0
        assert lib.dem_compat_errors() == 0
        sim.close()
    finally:
        _abi.check(lib.dem_compat_set_precision(0), "dem_compat_set_precision")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_engine_at_200k_after_a_forced_rebuild_matches_the_oracle(cuda, bed, precision):
    w = bed
    eng = Engine(w.setup, precision=precision)
    eng.set_state(w.pos0_reduced)
    eng.step(20)
    st = eng.get_state()
    # the same state back in, with the rebuild request set: the next step
    # rebuilds the lists and carries the histories over
    p, v, a = (np.ascontiguousarray(st[k]) for k in ("pos", "vel", "angvel"))
    _abi.check(eng.lib.dem_set_state_ex(eng.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(a), 1), "dem_set_state_ex")
    sim = _harness.OracleSim(w.setup, p, v, a)
    mp = _lockstep.max_per(w)
    tol, budget = (FP64_TOL, 0.0) if precision == "fp64" else (MIXED_TOL, 0.01)
    worst = {"force_err": 0.0, "hist_err": 0.0}
    it0 = int(eng.stats()["iter"])
    for t in range(4):
        before = _lockstep.snapshot(eng, mp)
        _lockstep.load_into(sim, before, it0 + t, first=(t == 0))
        r_sim = sim.step()
        r0 = eng.stats()["rebuilds"]
        eng.step(1)
        r_eng = eng.stats()["rebuilds"] - r0
        assert r_eng == r_sim, f"step {t}: rebuild decision {r_eng} vs {r_sim}"
        if t == 0:
            assert r_sim == 1
        res = _lockstep.compare_step(_lockstep.snapshot(eng, mp), sim, w, tol, f"{precision} step {t}", budget)
        for k in worst:
            worst[k] = max(worst[k], res[k])
    s = eng.stats()
    assert s["error_bits"] == 0
    eng.close()
    sim.close()


def test_mixed_packing_metrics_at_200k_match_fp64(cuda, bed):
    """the accuracy targets on the packed bed: packing fraction
    within 0.2 % and coordination number within 1 % of the FP64 run of the
    reference's formulas, after 2,000 steps from the same bed"""
    w = bed
    out = {}
    for prec in ("mixed", "fp64"):
        e = Engine(w.setup, precision=prec)
        e.set_state(w.pos0_reduced)
        e.step(2000)
        e.sync()
        out[prec] = packing_metrics(w.setup, e.get_state()["pos"])
        assert e.stats()["error_bits"] == 0
        e.close()
    phi_err = abs(out["mixed"]["phi"] - out["fp64"]["phi"]) / out["fp64"]["phi"]
    z_err = abs(out["mixed"]["z"] - out["fp64"]["z"]) / out["fp64"]["z"]
    assert phi_err < 2e-3 and z_err < 1e-2, (out, phi_err, z_err)


def test_dry_lattice_lands_in_lockstep_with_the_oracle(cuda):
    """the 5,000-sphere lattice from the dry workload, FP64 engine: free fall to
    just above the floor (20,100 steps), then 600 steps in lockstep while the
    bottom layer lands (wall contacts, plastic loading, rebounds)"""
    w = configs.dry()
    eng = Engine(w.setup, precision="fp64")
    eng.set_state(w.pos0_reduced)
    eng.step(20_100)
    st = eng.get_state()
    p, v, a = (np.ascontiguousarray(st[k]) for k in ("pos", "vel", "angvel"))
    _abi.check(eng.lib.dem_set_state_ex(eng.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(a), 1), "dem_set_state_ex")
    sim = _harness.OracleSim(w.setup, p, v, a)
    mp = _lockstep.max_per(w)
    it0 = int(eng.stats()["iter"])
    walls = 0
    for t in range(600):
        before = _lockstep.snapshot(eng, mp)
        _lockstep.load_into(sim, before, it0 + t, first=(t == 0))
        r_sim = sim.step()
        c0 = eng.stats()
        eng.step(1)
        c1 = eng.stats()
        assert c1["rebuilds"] - c0["rebuilds"] == r_sim, f"step {t}: rebuild decision"
        walls += c1["wall_contacts"] - c0["wall_contacts"]
        _lockstep.compare_step(_lockstep.snapshot(eng, mp), sim, w, FP64_TOL, f"step {t}")
    assert walls > 1000, walls
    eng.close()
    sim.close()


def test_dry_lattice_whole_run_matches_the_oracle(cuda):
    """the dry workload run whole (20,000 steps): the FP64 engine's packing
    fraction, coordination number and positions checksum against the oracle's
    free-running result, and the mixed engine within the accuracy targets"""
    w = configs.dry()
    n = w.setup.n
    res = {}
    for prec in ("fp64", "mixed"):
        e = Engine(w.setup, precision=prec)
        e.set_state(w.pos0_reduced)
        e.step(20_000)
        e.sync()
        res[prec] = e.get_state()["pos"]
        assert e.stats()["error_bits"] == 0
        e.close()
    sim = _harness.OracleSim(w.setup, w.pos0_reduced)
    sim.step(20_000)
    res["oracle"] = sim.state()["pos"]
    sim.close()
    m = {k: packing_metrics(w.setup, v) for k, v in res.items()}
    ck = {k: float((v[:, 0] + 2 * v[:, 1] + 3 * v[:, 2]).sum()) for k, v in res.items()}
    assert n == 5000 and m["oracle"]["phi"] > 0.5, m
    dev = {k: np.abs(res[k] - res["oracle"]).max(axis=1) for k in ("fp64", "mixed")}
    info = (m, ck, {k: (float(v.max()), float(np.mean(v > 1e-9))) for k, v in dev.items()})
    # The lattice falls freely but for the pairs its jitter starts overlapping:
    # they push apart and a few collide on; those few-body collisions are
    # chaotic (last-ulp pow differences grow), the free fall is not.
    # (mixed: every particle differs from the oracle by the FP32 rounding of
    # its gravity increments, ~1e-7 relative; the colliding few by more)
    for k, t in (("fp64", 1e-9), ("mixed", 1e-5)):
        assert np.mean(dev[k] > t) < 0.05, info
    # FP64: packing fraction, coordination number and checksum of the same formulas
    assert abs(m["fp64"]["phi"] - m["oracle"]["phi"]) <= 1e-7 * m["oracle"]["phi"], info
    assert abs(m["fp64"]["z"] - m["oracle"]["z"]) <= 2.0 / m["oracle"]["n_probe"], info
    assert abs(ck["fp64"] - ck["oracle"]) <= 1e-7 * np.abs(res["oracle"]).sum(), info
    # mixed: the accuracy targets (0.2 % packing fraction, 1 % coordination)
    assert abs(m["mixed"]["phi"] - m["oracle"]["phi"]) <= 2e-3 * m["oracle"]["phi"], info
    assert abs(m["mixed"]["z"] - m["oracle"]["z"]) <= 1e-2 * max(m["oracle"]["z"], 2.0 / m["oracle"]["n_probe"]), info
