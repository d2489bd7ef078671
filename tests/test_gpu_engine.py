"""The native engine (dem_* API) on the GPU against the oracle, in lockstep
(tests/_lockstep.py): before every step the oracle resumes from the engine's
exact state, both step, the outputs are compared.

FP64 mode (the reference formulas): neighbour lists (partner ids in the
reference's list order), wall lists, load stages and bridge flags bit-exact,
with or without cell reordering; forces, state and history to 1e-12 relative
(last-ulp pow/log/exp differences between CUDA and glibc).
Mixed mode (FP32 pair forces, Kahan-summed; FP64 state and spring history):
forces to 2e-5 of the step's force scale, positions to 1e-9, velocities 2e-6,
spins 2e-5, history to 1e-5;
stage / bridge labels may differ where FP32 and FP64 round a comparison
differently (a contact at its turning point), budgeted at 1%.
Graph replay must equal host-driven stepping bit for bit, and a resumed
checkpoint must equal the continuous run bit for bit."""
import ctypes as C

import numpy as np
import pytest

import _lockstep
import _workloads
from gpucode_gb300 import _abi
from gpucode_gb300.engine import Engine

pytestmark = pytest.mark.gpu

FP64_TOL = {"force": 1e-12, "pos": 1e-14, "vel": 1e-12, "hist": 1e-12}
# spins: a small sphere's moment of inertia 0.1 (2r)^5 is ~1e-4 of the largest,
# so FP32 moment rounding shows amplified in its spin increment; velocities take
# one FP32-rounded force increment per step, relative to the stirred speed scale
MIXED_TOL = {"force": 2e-5, "pos": 1e-9, "vel": 1e-5, "angvel": 2e-5, "hist": 1e-5}


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
@pytest.mark.parametrize("reorder", [False, True])
def test_fp64_engine_lockstep(cuda, make, reorder):
    w = make()
    pos, vel, ang = _workloads.stirred(w)
    eng = Engine(w.setup, precision="fp64", reorder=reorder, use_graph=False)
    worst = _lockstep.run(eng, w, pos, vel, ang, steps=250, tol=FP64_TOL)
    assert worst["rebuilds"] >= 2, worst
    eng.close()


@pytest.mark.parametrize("pairs", ["warp", "thread"])
@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_mixed_engine_lockstep(cuda, make, pairs):
    w = make()
    pos, vel, ang = _workloads.stirred(w)
    eng = Engine(w.setup, precision="mixed", pairs=pairs)
    worst = _lockstep.run(eng, w, pos, vel, ang, steps=250, tol=MIXED_TOL, mismatch_budget=0.01)
    assert worst["rebuilds"] >= 2, worst
    eng.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_moving_top_wall_lockstep(cuda, precision):
    """A lid descending onto the bed (CylinderBC.topv < 0; the reference moves
    the top wall by topv dt every step, kernel.cu:966-969): the wall moves once
    per step before any particle meets it, and forces, state, wall lists and
    wall histories follow the oracle step by step while the lid presses into
    the top layer."""
    w = _workloads.small_dry()
    pos, vel, ang = _workloads.stirred(w)
    s = w.setup.s
    top = float((pos[:, 2] + w.setup.rad).max())
    s.cyl.Tw = top + 0.01
    s.cyl.topv = -0.05 / (250 * s.prm.dt)  # 0.05 diameters over the run
    eng = Engine(w.setup, precision=precision, use_graph=False)
    tol, budget = (FP64_TOL, 0.0) if precision == "fp64" else (MIXED_TOL, 0.01)
    worst = _lockstep.run(eng, w, pos, vel, ang, steps=250, tol=tol, mismatch_budget=budget)
    assert worst["rebuilds"] >= 2, worst
    assert eng.stats()["wall_contacts"] > 0
    eng.close()


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_pair_loops_agree(cuda, make):
    """The warp-cooperative pair loop and the thread-per-particle one evaluate
    the same pairs with the same FP32 formulas and sum them in the same
    neighbour order, but each kernel's instruction selection is its own (FMA
    contraction, approximate division), and a wet contact's and its bridge's
    forces are added into one FP32 value before the Kahan sum.  One step from
    the same state: forces agree to FP32 rounding, state to the rounding of
    one FP32 increment, and the labels (contacts, bridges, flags) but for
    comparisons that land on their turning point."""
    w = make()
    pos, vel, ang = _workloads.stirred(w)
    a = Engine(w.setup, precision="mixed", pairs="warp")
    b = Engine(w.setup, precision="mixed", pairs="thread")
    for e in (a, b):
        e.set_state(pos, vel, ang)
        e.step(1)
        e.sync()
    sa, sb = a.get_state(), b.get_state()
    scale = float(np.abs(sb["force"]).max())
    assert float(np.abs(sa["force"] - sb["force"]).max()) <= 1e-6 * scale
    for k, tol in (("pos", 1e-12), ("vel", 1e-6)):
        assert np.allclose(sa[k], sb[k], rtol=0, atol=tol * max(1.0, float(np.abs(sb[k]).max()))), k
    # labels: a comparison at its turning point may round either way in the
    # two kernels; allowed on at most 0.5% of the contacts
    mp = _lockstep.max_per(w)
    ha, hb = a.history(mp), b.history(mp)
    budget = max(1, int(0.005 * max(1, int(np.count_nonzero(hb[0][..., 7])))))
    assert int(np.count_nonzero(ha[1] != hb[1])) <= budget  # bridge flags
    assert int(np.count_nonzero(ha[0][..., 7] != hb[0][..., 7])) <= budget  # load stages
    sa_, sb_ = a.stats(), b.stats()
    for k in ("contacts", "bridges", "wall_contacts"):
        assert abs(sa_[k] - sb_[k]) <= budget, k
    a.close()
    b.close()


@pytest.mark.parametrize("pairs, sizes", [("warp", (32, 64, 96, 128)), ("thread", (32, 64, 128))])
def test_block_size_does_not_change_results(cuda, pairs, sizes):
    """The step kernel's block size (the default, 32 for the warp loop and 128
    for the thread loop, or the option) only changes which warps share a
    block: every warp's particles and arithmetic are the same, so 60 steps
    with rebuilds give the same bits at every size."""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    out = {}
    for bs in (0,) + tuple(sizes):
        e = Engine(w.setup, precision="mixed", pairs=pairs, block_size=bs)
        e.set_state(pos, vel, ang)
        e.step(60)
        e.sync()
        out[bs] = (e.get_state(), e.stats()["rebuilds"], e.history(_lockstep.max_per(w)))
        e.close()
    s0, r0, h0 = out[0]
    assert r0 >= 1
    for bs in sizes:
        s, r, h = out[bs]
        assert r == r0, bs
        for k in ("pos", "vel", "angvel", "force"):
            assert np.array_equal(s[k], s0[k]), (bs, k)
        assert np.array_equal(h[0], h0[0]) and np.array_equal(h[1], h0[1]), bs


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_equals_host_stepping(cuda, precision):
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    a = Engine(w.setup, precision=precision, use_graph=True)
    b = Engine(w.setup, precision=precision, use_graph=False)
    for e in (a, b):
        e.set_state(pos, vel, ang)
        e.step(96)
        e.sync()
    sa, sb = a.get_state(), b.get_state()
    for k in ("pos", "vel", "angvel"):
        assert np.array_equal(sa[k], sb[k]), k
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"] >= 1
    mp = _lockstep.max_per(w)
    ha, hb = a.history(mp), b.history(mp)
    assert np.array_equal(ha[0], hb[0]) and np.array_equal(ha[1], hb[1])


def test_device_chained_steps_equal_single_and_host_steps(cuda):
    """mixed precision with graphs chains its steps on the device (the step
    graph tail-launches the rebuild and the next step): one 240-step call,
    240 one-step calls, calls of uneven lengths and host-driven stepping give
    the same bits, with the rebuilds at the same steps"""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    runs = {"chain": [240], "single": [1] * 240, "uneven": [100, 1, 37, 1, 101], "host": [240]}
    out = {}
    for name, calls in runs.items():
        e = Engine(w.setup, precision="mixed", use_graph=name != "host")
        e.set_state(pos, vel, ang)
        for k in calls:
            e.step(k)
        e.sync()
        assert e.step_chained() == (name != "host")
        out[name] = (e.get_state(), e.stats()["rebuilds"], e.history(_lockstep.max_per(w)))
        e.close()
    s0, r0, h0 = out["host"]
    assert r0 >= 2
    for name in ("chain", "single", "uneven"):
        s, r, h = out[name]
        assert r == r0, name
        for k in ("pos", "vel", "angvel", "force"):
            assert np.array_equal(s[k], s0[k]), (name, k)
        assert np.array_equal(h[0], h0[0]) and np.array_equal(h[1], h0[1]), name


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_checkpoint_resume_is_bit_exact(cuda, tmp_path, precision):
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    a = Engine(w.setup, precision=precision)
    a.set_state(pos, vel, ang)
    a.step(64)
    path = tmp_path / "heyi_dump.dat"
    a.save(path, nbatch=3)
    a.step(64)
    b = Engine(w.setup, precision=precision)
    b.load(path)
    b.step(64)
    sa, sb = a.get_state(), b.get_state()
    for k in ("pos", "vel", "angvel"):
        assert np.array_equal(sa[k], sb[k]), k
    # the dump keeps the reference's text header (DumpLoad.cpp:14-17)
    lib = _abi.load()
    x, y, z = C.c_int(), C.c_int(), C.c_int()
    lib.LoadPara(str(path).encode(), C.byref(x), C.byref(y), C.byref(z))
    assert (x.value, y.value, z.value) == (w.setup.n, 3, w.setup.n)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_state_round_trip_without_rebuild_is_bit_exact(cuda, precision):
    """dem_get_state then dem_set_state_ex(..., request_rebuild = 0) with the same
    arrays (the end-to-end path: the import gathers into cell order and, in
    mixed precision, rewrites the shadows and bridge counts in one pass) leaves
    the run as if it had not been interrupted"""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    a = Engine(w.setup, precision=precision)
    b = Engine(w.setup, precision=precision)
    for e in (a, b):
        e.set_state(pos, vel, ang)
        e.step(37)
    st = b.get_state()
    p, v, g = (np.ascontiguousarray(st[k]) for k in ("pos", "vel", "angvel"))
    for _ in range(3):
        _abi.check(b.lib.dem_set_state_ex(b.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(g), 0), "dem_set_state_ex")
        b.step(9)
        a.step(9)
        st = b.get_state()
        p, v, g = (np.ascontiguousarray(st[k]) for k in ("pos", "vel", "angvel"))
    sa, sb = a.get_state(), b.get_state()
    for k in ("pos", "vel", "angvel", "force"):
        assert np.array_equal(sa[k], sb[k]), k
    assert a.stats()["rebuilds"] == b.stats()["rebuilds"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("rebuild", [0, 1])
def test_page_locked_host_arrays_give_the_same_state(cuda, precision, rebuild):
    """Page-locked caller arrays are read and written by the import and export
    kernels directly over the host link (no staging copy; 16-byte accesses, or
    8-byte ones for arrays that are not 16-byte aligned); pageable ones go
    through the copy engines and device staging.  All routes move the same
    bits: three rounds of import, 7 steps and export (positions, velocities,
    spins and forces) give identical states and rebuild counts."""
    torch = pytest.importorskip("torch")
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    n = w.setup.n
    pinned = [torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
    # page-locked arrays that start 8 bytes into their allocation: the import
    # and export take their 8-byte (not 16-byte) host accesses
    odd = [torch.empty(3 * n + 1, dtype=torch.float64, pin_memory=True).numpy()[1:].reshape(n, 3) for _ in range(4)]
    assert all(a.ctypes.data % 16 == 8 for a in odd)
    out = {}
    for route in ("pageable", "page-locked", "page-locked, 8-byte aligned"):
        e = Engine(w.setup, precision=precision)
        e.set_state(pos, vel, ang)
        e.step(20)
        st = e.get_state()
        bufs = [np.ascontiguousarray(st[k]) for k in ("pos", "vel", "angvel")] + [np.zeros((n, 3))]
        if route != "pageable":
            locked = pinned if route == "page-locked" else odd
            for dst, src in zip(locked, bufs):
                dst[...] = src
            bufs = locked
        p, v, g, f = bufs
        for _ in range(3):
            _abi.check(e.lib.dem_set_state_ex(e.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(g), rebuild), "set_state_ex")
            e.step(7)
            _abi.check(e.lib.dem_get_state(e.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(g), _abi.ptr(f), None),
                       "get_state")
        out[route] = ([b.copy() for b in (p, v, g, f)], e.stats()["rebuilds"])
        e.close()
    for route in ("page-locked", "page-locked, 8-byte aligned"):
        for k, (a, b) in enumerate(zip(out["pageable"][0], out[route][0])):
            assert np.array_equal(a, b), (route, ("pos", "vel", "angvel", "force")[k])
        assert out["pageable"][1] == out[route][1], route


@pytest.mark.parametrize("locked", [False, True])
def test_advance_equals_import_step_export(cuda, locked):
    """dem_advance (import, steps and export with one wait) against the three
    calls it queues, on page-locked and on pageable arrays: the same bits in
    the same arrays, four rounds of 9 steps"""
    torch = pytest.importorskip("torch")
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    n = w.setup.n
    out = {}
    for call in ("three calls", "dem_advance"):
        e = Engine(w.setup, precision="mixed")
        e.set_state(pos, vel, ang)
        e.step(30)
        st = e.get_state()
        if locked:
            bufs = [torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
        else:
            bufs = [np.empty((n, 3)) for _ in range(4)]
        for dst, k in zip(bufs, ("pos", "vel", "angvel", "force")):
            dst[...] = st[k]
        p, v, g, f = bufs
        for _ in range(4):
            if call == "dem_advance":
                _abi.check(e.lib.dem_advance(e.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(g), _abi.ptr(f), 9), "advance")
            else:
                _abi.check(e.lib.dem_set_state_ex(e.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(g), 0), "set_state_ex")
                e.step(9)
                _abi.check(e.lib.dem_get_state(e.h, _abi.ptr(p), _abi.ptr(v), _abi.ptr(g), _abi.ptr(f), None), "get")
        out[call] = ([b.copy() for b in bufs], e.stats()["rebuilds"], e.stats()["iter"])
        e.close()
    a, b = out["three calls"], out["dem_advance"]
    for k in range(4):
        assert np.array_equal(a[0][k], b[0][k]), ("pos", "vel", "angvel", "force")[k]
    assert a[1:] == b[1:]


def test_slot_overflow_is_reported_not_written(cuda):
    """A level whose slot capacity is too small: the build stops at capacity and
    dem_sync reports DEM_ERR_OVERFLOW (the reference would write past the end)."""
    w = _workloads.small_dry()
    s = w.setup
    s.s.level_nnebors[0] = 2
    s.s.n_pp_slots = 2 * s.s.level_npars[0]
    pos, vel, ang = _workloads.stirred(w)
    e = Engine(s, precision="mixed")
    e.set_state(pos, vel, ang)
    e.step(1)
    with pytest.raises(_abi.DemError) as ei:
        e.sync()
    assert ei.value.code == _abi.DEM_ERR_OVERFLOW
    counts, _ = e.neighbors(2)
    assert counts.max() <= 2


def test_nonfinite_state_is_reported(cuda):
    w = _workloads.small_dry()
    pos, vel, ang = _workloads.stirred(w)
    vel[5, 1] = np.nan
    e = Engine(w.setup, precision="mixed")
    e.set_state(pos, vel, ang)
    e.step(2)
    with pytest.raises(_abi.DemError) as ei:
        e.sync()
    assert ei.value.code == _abi.DEM_ERR_NONFINITE


@pytest.mark.parametrize("n", [1, 2, 37])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tiny_and_ragged_beds_lockstep(cuda, n, precision):
    """A single sphere (no neighbours: the floor and the side wall only), a
    pair, and a bed that fills neither a warp nor a block: the pair loops'
    partial warps and empty lists follow the oracle step by step."""
    w = _workloads.small_dry(n=n, seed=5)
    pos, vel, ang = _workloads.stirred(w, vscale=2.0)
    eng = Engine(w.setup, precision=precision, use_graph=False)
    tol, budget = (FP64_TOL, 0.0) if precision == "fp64" else (MIXED_TOL, 0.01)
    worst = _lockstep.run(eng, w, pos, vel, ang, steps=120, tol=tol, mismatch_budget=budget)
    assert worst["rebuilds"] >= 1, worst
    eng.close()


def test_empty_setup_is_rejected():
    """no particles: dem_create refuses the set-up instead of launching empty grids"""
    w = _workloads.small_dry(n=8)
    w.setup.s.np = 0
    with pytest.raises(_abi.DemError) as ei:
        Engine(w.setup, precision="mixed")
    assert ei.value.code == _abi.DEM_ERR_ARG


def test_particle_outside_the_grid_is_reported(cuda):
    """a particle far outside the domain hashes past the last cell: the build
    keeps it in the last cell instead of writing past the cell arrays (the
    reference clamps to the grid size, kernel.cu:627-629, one past the end)
    and dem_sync reports DEM_ERR_CELL"""
    w = _workloads.small_dry()
    pos, vel, ang = _workloads.stirred(w)
    pos[7, 2] = 1.0e4
    e = Engine(w.setup, precision="mixed")
    e.set_state(pos, vel, ang)
    e.step(1)
    with pytest.raises(_abi.DemError) as ei:
        e.sync()
    assert ei.value.code == _abi.DEM_ERR_CELL
    e.close()


def test_profile_kernels_times_a_rebuild_and_a_step(cuda):
    """dem_profile_kernels: one step with a forced rebuild, an event after each
    kernel; it counts as a step and stepping goes on from it"""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    e = Engine(w.setup, precision="mixed")
    e.set_state(pos, vel, ang)
    e.step(2)
    e.sync()
    s0 = e.stats()
    rows = e.profile_kernels()
    names = [r[0] for r in rows]
    for k in ("k_copy_old", "k_permute", "k_neighbor_find", "k_wall_list", "k_carry"):
        assert k in names, names
    assert names[-1] == "step kernel"
    assert all(ms >= 0.0 for _, ms in rows) and sum(ms for _, ms in rows) > 0.0
    s1 = e.stats()
    assert s1["iter"] == s0["iter"] + 1 and s1["rebuilds"] == s0["rebuilds"] + 1
    e.step(5)
    e.sync()
    assert e.stats()["iter"] == s1["iter"] + 5
    e.close()
