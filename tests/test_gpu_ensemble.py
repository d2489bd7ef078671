"""Batched ensembles on the GPU: every system stepped inside the batch against
the same system stepped alone, and the autotuner.

The batch translates each system to its place in the shared domain, so the
FP32 shadows round differently from the stand-alone run: one step agrees to
the FP32 force tolerance (2e-5 of the force scale), a short run to a small
fraction of a particle radius."""
import numpy as np
import pytest

import _workloads
from gpucode_gb300 import _abi, configs
from gpucode_gb300.autotune import autotune
from gpucode_gb300.engine import Engine

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ens(cuda):
    return configs.ensemble(n_systems=6, n_range=(300, 1200), seed=9, threads=4)


def _batched(e, steps):
    eng = Engine(e.combined.setup, precision="mixed")
    eng.set_state(e.combined.pos0_reduced)
    eng.set_systems(e.system, e.cylinders, e.wet)
    eng.step(steps)
    eng.sync()
    return eng


def _alone(m, steps):
    m = configs.member_setup(m)
    eng = Engine(m.setup, precision="mixed")
    eng.set_state(m.pos0_reduced)
    eng.step(steps)
    eng.sync()
    return eng


def test_each_system_in_the_batch_steps_as_it_does_alone(ens):
    e = ens
    b = _batched(e, 1)
    fb = b.get_state()["force"]
    for k, m in enumerate(e.members):
        a = _alone(m, 1)
        fa = a.get_state()["force"]
        err = np.abs(fb[e.system == k] - fa).max() / np.abs(fa).max()
        assert err < 2e-5, (k, err)
        a.close()
    b.step(99)
    pb = b.get_state()["pos"]
    rl = e.combined.setup.s.unit.rlunit
    for k, m in enumerate(e.members):
        a = _alone(m, 100)
        pa = a.get_state()["pos"]
        shift = np.array([e.offsets[k][0] / rl, e.offsets[k][1] / rl, 0.0])
        d = np.abs(pb[e.system == k] - shift - pa).max()
        assert d < 1e-3 * m.setup.rad.max(), (k, d)
        a.close()
    b.close()


def test_dry_systems_form_no_bridges(ens):
    e = ens
    b = _batched(e, 20)
    _, brg = b.history(256)
    assert brg[e.wet[e.system] == 0].max() == 0
    assert brg[e.wet[e.system] == 1].max() == 1
    b.close()


def test_set_systems_rejects_bad_input(ens):
    e = ens
    eng = Engine(e.combined.setup, precision="mixed")
    bad = e.system.copy()
    bad[3] = len(e.cylinders)
    with pytest.raises(_abi.DemError):
        eng.set_systems(bad, e.cylinders, e.wet)
    eng.set_systems(e.system, e.cylinders, e.wet)
    with pytest.raises(_abi.DemError):
        eng.set_systems(e.system, e.cylinders, e.wet)  # only once
    eng.close()
    f = Engine(e.combined.setup, precision="fp64")
    with pytest.raises(_abi.DemError):
        f.set_systems(e.system, e.cylinders, e.wet)
    f.close()


def test_autotune_picks_a_working_configuration(cuda):
    w = _workloads.small_wet()
    pos, vel, _ = _workloads.stirred(w, vscale=0.05, wscale=0.1)
    setup, opts, rep = autotune(w.inp, w.dia, pos, vel, skins=(1.0, 2.0), cells=(1.0, 1.5), blocks=(64, 128),
                                warmup=5, trial=30)
    assert len(rep["trials"]) == 8 and all(t["particle_steps_per_s"] > 0 for t in rep["trials"])
    best = max(rep["trials"], key=lambda t: t["particle_steps_per_s"])
    assert (best["skin_scale"], best["cell_scale"], best["block_size"]) == (
        rep["skin_scale"], rep["cell_scale"], rep["block_size"])
    eng = Engine(setup, precision="mixed", block_size=opts["block_size"])
    eng.set_state(pos, vel)
    eng.step(50)
    eng.sync()
    assert np.isfinite(eng.get_state()["pos"]).all()
    eng.close()


def test_block_size_and_cell_size_do_not_change_the_physics(cuda):
    """same bed, block size 64 vs 128 and cells 1x vs 1.5x: identical results
    (the neighbour order within a particle's list follows the cell walk, so the
    cell size may reorder a list: forces then agree to FP32 summation order)"""
    import copy

    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w, vscale=0.05, wscale=0.1)
    runs = {}
    for name, bs, cell in (("a", 128, 1.0), ("b", 64, 1.0), ("c", 128, 1.5)):
        st = copy.deepcopy(w.setup)
        st.scale_cells(cell)
        eng = Engine(st, precision="mixed", block_size=bs)
        eng.set_state(pos, vel, ang)
        eng.step(1)
        runs[name] = eng.get_state()["force"]
        eng.close()
    np.testing.assert_array_equal(runs["a"], runs["b"])
    assert np.abs(runs["a"] - runs["c"]).max() <= 1e-5 * np.abs(runs["a"]).max()
