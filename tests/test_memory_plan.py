"""The memory plan (dem_memory_estimate, dem_fit_memory): CPU arithmetic, and
on the GPU the estimate against what dem_create really takes."""
import copy
import ctypes as C

import numpy as np
import pytest

import _workloads
from gpucode_gb300 import _abi
from gpucode_gb300.engine import Engine


def test_estimate_adds_up():
    w = _workloads.small_wet()
    s = w.setup.s
    m = w.setup.memory("mixed")
    assert m["slots"] == s.n_pp_slots
    assert m["per_slot"] == 138 and m["per_particle"] == 756 + 144
    assert m["per_cell"] == 12  # cell start, end and offset
    low = m["per_particle"] * s.np + m["per_slot"] * s.n_pp_slots + m["per_cell"] * s.sys_ncells
    assert low < m["total"] < low + 200 * 2 ** 20
    assert w.setup.memory("fp64")["per_particle"] == 756


def test_fit_memory_scales_slots_to_the_budget():
    w = _workloads.small_wet()
    setup = copy.deepcopy(w.setup)
    orig = list(setup.s.level_nnebors)[: setup.s.n_levels]
    full = setup.memory()["total"]
    budget = full - 0.5 * setup.memory()["per_slot"] * setup.s.n_pp_slots  # half the slot bytes
    f = setup.fit_memory(budget, min_slots=8)
    assert 0.0 < f < 1.0
    new = list(setup.s.level_nnebors)[: setup.s.n_levels]
    assert all(8 <= b <= a for a, b in zip(orig, new))
    assert setup.s.n_pp_slots == sum(b * p for b, p in zip(new, list(setup.s.level_npars)[: setup.s.n_levels]))
    assert setup.memory()["total"] <= budget
    # an impossible budget is an error, and leaves the set-up alone
    tiny = copy.deepcopy(w.setup)
    with pytest.raises(_abi.DemError) as e:
        tiny.fit_memory(1e6, min_slots=8)
    assert e.value.code == _abi.DEM_ERR_NOMEM
    assert list(tiny.s.level_nnebors)[: tiny.s.n_levels] == orig
    # a budget that fits leaves the slots alone
    same = copy.deepcopy(w.setup)
    assert same.fit_memory(10 * full) == 1.0
    assert list(same.s.level_nnebors)[: same.s.n_levels] == orig


@pytest.mark.gpu
def test_estimate_matches_the_device(cuda):
    import torch

    w = _workloads.small_wet()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    eng = Engine(w.setup, precision="mixed")
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    used = free0 - free1
    est = w.setup.memory("mixed")["total"]
    assert used <= est, (used, est)
    eng.close()


@pytest.mark.gpu
def test_fitted_slots_give_the_same_run(cuda):
    """a bed stepped on fitted (fewer) slots evolves bit for bit as on the full
    slots while no level outgrows them (overflow itself: test_gpu_engine)"""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w, vscale=0.05, wscale=0.1)
    fitted = copy.deepcopy(w.setup)
    m = fitted.memory()
    f = fitted.fit_memory(m["total"] - 0.6 * m["per_slot"] * fitted.s.n_pp_slots, 12)
    assert f < 0.5
    a, b = Engine(w.setup, precision="mixed"), Engine(fitted, precision="mixed")
    for e in (a, b):
        e.set_state(pos, vel, ang)
        e.step(50)
        e.sync()
    np.testing.assert_array_equal(a.get_state()["pos"], b.get_state()["pos"])
    for e in (a, b):
        e.close()


@pytest.mark.gpu
def test_sixteen_million_spheres_fit_180_gb(cuda):
    """The 16,000,000-sphere wet set-up (R = 150 mm, four levels): at the
    reference's slot counts it needs more than 180 GB; fitted to 180 GB the
    engine is created within the estimate, takes the state and steps without a
    slot overflow, and a lattice of spheres apart from one another comes back
    through the permutation to cell order and back with x and y unchanged
    (nothing pushes sideways) and every sphere a little lower (gravity)."""
    import torch

    from gpucode_gb300 import configs

    w = configs.wet(n=16_000_000, cyl_r=0.15, packing="lattice")
    assert w.setup.memory("mixed")["total"] > 180e9
    f = w.setup.fit_memory(180e9, min_slots=8, precision="mixed")
    est = w.setup.memory("mixed")["total"]
    assert f < 1.0 and est <= 180e9
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    if free0 < est + 2e9:
        pytest.skip(f"{free0 / 1e9:.0f} GB free on the device, {est / 1e9:.0f} GB needed")
    eng = Engine(w.setup, precision="mixed")
    torch.cuda.synchronize()
    used = free0 - torch.cuda.mem_get_info()[0]
    assert used <= est, (used, est)
    pos = w.pos0_reduced
    eng.set_state(pos)
    eng.step(20)
    eng.sync()  # raises on a slot overflow
    st = eng.get_state()
    eng.close()
    np.testing.assert_array_equal(st["pos"][:, :2], pos[:, :2])
    assert not st["vel"][:, :2].any()
    drop = pos[:, 2] - st["pos"][:, 2]
    assert (drop > 0).all() and (drop < 1e-5).all(), (drop.min(), drop.max())
