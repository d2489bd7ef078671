"""The reference-compatible entry points (heydem.h:366-613) on the GPU, driven in
main.cpp:433-568's order on the reference's own layouts, against the oracle in
lockstep (tests/_lockstep.py).

Integer outputs (sorted hashes and indices, CellStart/CellEnd, neighbour slots,
wall lists, load stages, bridge flags) must be bit-exact.  Floating-point
outputs are FP64 with the reference's formulas on both sides: 1e-12 relative
per step (last-ulp differences of CUDA's and glibc's pow/log/exp), except at
contacts whose spring sits exactly on its slip limit, where those differences
legitimately select the other friction branch."""
import numpy as np
import pytest

import _harness
import _lockstep
import _workloads
from gpucode_gb300 import _abi
from gpucode_gb300.dropin import DropInDriver, declare

pytestmark = pytest.mark.gpu


# the reference driver's step loop over the drop-in entry points (the
# package's own main.cpp-order driver; the tests drive it step by step)
RefDriver = DropInDriver
_declare = declare


FP64_TOL = {"force": 1e-12, "pos": 1e-14, "vel": 1e-12, "hist": 1e-12}
# the mixed engine's per-step tolerances (forces relative to the step's force scale)
MIXED_TOL = {"force": 2e-5, "pos": 1e-9, "vel": 1e-5, "angvel": 2e-5, "hist": 1e-5}


def _snap(drv, sim, w):
    """the driver's device state (reference layouts) in the lockstep comparison's
    terms: lists and contact records as the used slots end to end"""
    g = lambda x: x.detach().cpu().numpy()  # noqa: E731
    n = drv.n
    num = g(drv.num)
    _, _, sl = sim.slots_of(num)
    pp = {k: g(v) for k, v in drv.pp[0].items()}
    rec = np.zeros((len(sl), 8))
    rec[:, 0:3] = pp["dispt"][sl]
    for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
        rec[:, 3 + c] = pp[f][sl]
    rec[:, 7] = pp["stage"][sl]
    pw = {k: g(v) for k, v in drv.pw[0].items()}
    wrec = np.zeros((n, 3, 8))
    for a in range(3):
        rows = a * n + np.arange(n)
        wrec[:, a, 0:3] = pw["dispt"][rows]
        for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
            wrec[:, a, 3 + c] = pw[f][rows]
        wrec[:, a, 7] = pw["stage"][rows]
    return dict(pos=g(drv.pos), vel=g(drv.vel), angvel=g(drv.ang), force=g(drv.force), pmove=g(drv.pmove),
                lqd=g(drv.lqd), counts=num, partners=g(drv.neb)[sl], rec=rec, brg=pp["lqdBrg"][sl],
                nwall=g(drv.nw), wlist=g(drv.wl), wrec=wrec, flag=int(drv.flag.item()))


def _load_oracle_from(drv, sim):
    """the oracle resumes from the driver's device state (same layouts)"""
    n, S = drv.n, drv.S
    g = lambda x: x.detach().cpu().numpy()  # noqa: E731
    sim.vec("pos")[:] = g(drv.pos)
    sim.vec("vel")[:] = g(drv.vel)
    sim.vec("angvel")[:] = g(drv.ang)
    sim.arr("pMove", np.float64, n)[:] = g(drv.pmove)
    sim.arr("lqdCnt", np.int32, n)[:] = g(drv.lqd)
    sim.arr("Num_Nebor", np.int32, n)[:] = g(drv.num)
    sim.arr("Nebor1", np.int32, S)[:] = g(drv.neb)
    for tag, h, m in (("pp", drv.pp[0], S), ("pw", drv.pw[0], 3 * n)):
        sim.arr(tag + ".dispt", np.float64, 3 * m)[:] = g(h["dispt"]).reshape(-1)
        for f in ("nDsp", "nDsp_mx", "plstRad", "plstDfm"):
            sim.arr(f"{tag}.{f}", np.float64, m)[:] = g(h[f])
        for f in ("stage", "lqdBrg"):
            sim.arr(f"{tag}.{f}", np.int32, m)[:] = g(h[f])
    sim.arr("nwall", np.int32, n)[:] = g(drv.nw)
    sim.arr("wlist", np.int32, 3 * n)[:] = g(drv.wl).reshape(-1)
    sim.lib.orc_sim_set_counter(sim.h, b"flag", int(drv.flag.item()))
    sim.lib.orc_sim_set_counter(sim.h, b"iter", drv.iter)
    sim.lib.orc_sim_set_counter(sim.h, b"need_build", 1 if drv.rebuild_pending else 0)


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_compat_step_loop_matches_oracle(cuda, make):
    """main.cpp's loop through the C ABI, in lockstep with the oracle: each step
    starts both from the driver's state; sorted order, cell ranges, neighbour
    slots, wall lists, stages and bridge flags bit-exact after every step;
    forces, state and histories to 1e-12 relative."""
    import torch

    w = make()
    _declare(_abi.load())
    pos, vel, ang = _workloads.stirred(w)
    drv = RefDriver(w, pos, vel, ang, torch)
    sim = _harness.OracleSim(w.setup, pos, vel, ang)
    n = w.setup.n
    g = lambda x: x.detach().cpu().numpy()  # noqa: E731
    rebuilds = 0
    for t in range(250):
        torch.cuda.synchronize()
        _load_oracle_from(drv, sim)
        rb = sim.step()
        ra = drv.step()
        torch.cuda.synchronize()
        assert ra == bool(rb), f"rebuild decision differs at step {t}"
        rebuilds += rb
        if rb:
            assert np.array_equal(g(drv.hash), sim.arr("hash", np.int32, n)), t
            assert np.array_equal(g(drv.index), sim.arr("index", np.int32, n)), t
            assert np.array_equal(g(drv.cs), sim.arr("cellStart", np.int32, drv.C)), t
            assert np.array_equal(g(drv.ce), sim.arr("cellEnd", np.int32, drv.C)), t
        _lockstep.compare_step(_snap(drv, sim, w), sim, w, FP64_TOL, f"step {t}")
    assert rebuilds >= 2
    assert _abi.load().dem_compat_errors() == 0


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_compat_mixed_step_loop_matches_oracle(cuda, make):
    """The same loop with the entry points in mixed precision
    (dem_compat_set_precision(DEM_PREC_MIXED), what DEM_COMPAT_PRECISION=mixed
    selects for an unchanged main.cpp): sorted order, cell ranges and
    neighbour slots still bit-exact, forces, state and histories within the
    mixed engine's tolerances, at most 1 % of stage or bridge labels flipped
    where FP32 and FP64 round a turning point differently."""
    import torch

    w = make()
    lib = _abi.load()
    _declare(lib)
    _abi.check(lib.dem_compat_set_precision(1), "dem_compat_set_precision")
    try:
        assert lib.dem_compat_precision() == 1
        pos, vel, ang = _workloads.stirred(w)
        drv = RefDriver(w, pos, vel, ang, torch)
        sim = _harness.OracleSim(w.setup, pos, vel, ang)
        n = w.setup.n
        g = lambda x: x.detach().cpu().numpy()  # noqa: E731
        rebuilds = 0
        for t in range(250):
            torch.cuda.synchronize()
            _load_oracle_from(drv, sim)
            rb = sim.step()
            ra = drv.step()
            torch.cuda.synchronize()
            assert ra == bool(rb), f"rebuild decision differs at step {t}"
            rebuilds += rb
            if rb:
                assert np.array_equal(g(drv.index), sim.arr("index", np.int32, n)), t
                assert np.array_equal(g(drv.cs), sim.arr("cellStart", np.int32, drv.C)), t
            _lockstep.compare_step(_snap(drv, sim, w), sim, w, MIXED_TOL, f"step {t}", mismatch_budget=0.01)
        assert rebuilds >= 2
        assert lib.dem_compat_errors() == 0
    finally:
        _abi.check(lib.dem_compat_set_precision(0), "dem_compat_set_precision")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_compat_moving_top_wall_lockstep(cuda, precision):
    """CirPWCalc with a descending lid (CylinderBC.topv < 0, kernel.cu:966-969):
    the entry point moves the top wall once per call before any sphere meets
    it, in both modes, and the loop follows the oracle step by step while the
    lid presses into the top layer (wall lists bit-exact, wall histories and
    forces to the mode's tolerances)."""
    import torch

    w = _workloads.small_dry()
    lib = _abi.load()
    _declare(lib)
    mixed = precision == "mixed"
    tol, budget = (MIXED_TOL, 0.01) if mixed else (FP64_TOL, 0.0)
    pos, vel, ang = _workloads.stirred(w)
    s = w.setup.s
    s.cyl.Tw = float((pos[:, 2] + w.setup.rad).max()) + 0.01
    s.cyl.topv = -0.05 / (250 * s.prm.dt)  # 0.05 diameters over the run
    _abi.check(lib.dem_compat_set_precision(1 if mixed else 0), "dem_compat_set_precision")
    try:
        drv = RefDriver(w, pos, vel, ang, torch)
        sim = _harness.OracleSim(w.setup, pos, vel, ang)
        rebuilds, touched = 0, 0
        for t in range(250):
            torch.cuda.synchronize()
            _load_oracle_from(drv, sim)
            rb = sim.step()
            ra = drv.step()
            torch.cuda.synchronize()
            assert ra == bool(rb), f"rebuild decision differs at step {t}"
            rebuilds += rb
            _lockstep.compare_step(_snap(drv, sim, w), sim, w, tol, f"{precision} step {t}", mismatch_budget=budget)
            # spheres in contact with the lid: a wall-list entry of kind 0 whose record has a stage
            wl, nw = drv.wl, drv.nw
            stage = drv.pw[0]["stage"].view(3, drv.n).t()
            slot = torch.arange(3, device=wl.device).unsqueeze(0) < nw.unsqueeze(1)
            touched = max(touched, int(((wl == 0) & slot & (stage != 0)).sum().item()))
        assert rebuilds >= 2
        assert touched > 0  # the lid reached the top layer
        assert lib.dem_compat_errors() == 0
    finally:
        _abi.check(lib.dem_compat_set_precision(0), "dem_compat_set_precision")


def test_first_step_forces_match_oracle_tightly(cuda):
    """One step from the same state: no chaotic growth, so FP64 forces agree to 1e-12."""
    import torch

    w = _workloads.small_wet()
    _declare(_abi.load())
    pos, vel, ang = _workloads.stirred(w)
    drv = RefDriver(w, pos, vel, ang, torch)
    sim = _harness.OracleSim(w.setup, pos, vel, ang)
    drv.step()
    sim.step()
    torch.cuda.synchronize()
    st = sim.state()
    scale = np.abs(st["force"]).max()
    np.testing.assert_allclose(drv.force.cpu().numpy(), st["force"], rtol=1e-12, atol=1e-14 * scale)
    np.testing.assert_allclose(drv.mom.cpu().numpy(), st["mom"], rtol=1e-12, atol=1e-14 * np.abs(st["mom"]).max())
    np.testing.assert_allclose(drv.pos.cpu().numpy(), st["pos"], rtol=1e-15, atol=1e-15)
    assert np.array_equal(drv.lqd.cpu().numpy(), sim.arr("lqdCnt", np.int32, w.setup.n))
