"""Pin the CPU oracle to the reference itself.

The reference's own kernel.cu (compiled for the CPU, unmodified, through
oracle/ref_shim by oracle/Makefile) and the oracle restatement run the same
seeded simulations step by step (the main.cpp:433-568 sequence, rebuilds and
history carry-over included); every array a step writes must agree bit for
bit.  Skipped where the reference sources are not present -- there the golden
fixtures (test_oracle_golden.py) pin the oracle instead.
"""
import numpy as np
import pytest

import _harness
import _workloads


@pytest.fixture(scope="module")
def have_ref():
    if not _harness.ref_available():
        pytest.skip(f"reference sources not found at {_harness.REF_SRC} (set DEM_REF_DIR): pinned by "
                    "tests/golden instead")


def _run_pair(w, steps, check_every):
    pos, vel, ang = _workloads.stirred(w)
    a = _harness.OracleSim(w.setup, pos, vel, ang)
    b = _harness.OracleSim(w.setup, pos, vel, ang, use_ref_kernels=True)
    rebuilds = 0
    for t in range(steps):
        ra, rb = a.step(), b.step()
        assert ra == rb, f"rebuild decision differs at step {t}"
        rebuilds += ra
        if (t + 1) % check_every == 0 or ra:
            xa, xb = _harness.sim_arrays(a), _harness.sim_arrays(b)
            for k in xa:
                assert np.array_equal(xa[k], xb[k], equal_nan=True), f"{k} differs at step {t}"
    return rebuilds, a


@pytest.mark.parametrize("make,steps", [(_workloads.small_dry, 900), (_workloads.small_wet, 900)])
def test_oracle_equals_reference_kernels(have_ref, make, steps):
    w = make()
    rebuilds, sim = _run_pair(w, steps, check_every=150)
    assert rebuilds >= 2, "the run must rebuild (and carry history) at least once after the first build"
    num, _ = sim.lists()
    assert num.sum() > 0
    h = np.vstack(sim.history())
    assert (h[:, 8] > 0).any() if w.setup.s.force_cap else True  # bridges formed in the wet bed
    assert (h[:, 7] == 2).any() and (np.abs(h[:, :3]).sum(1) > 0).any()  # loading contacts with springs


def test_fcap_equals_reference(have_ref):
    w = _workloads.small_wet()
    k = _harness.consts_of(w.setup)
    import ctypes as C

    rng = np.random.Generator(np.random.PCG64(11))
    for _ in range(200):
        S = float(rng.uniform(0, 0.05))
        V = float(rng.uniform(1e-4, 5e-2))
        R = float(rng.uniform(0.1, 0.5))
        a = _harness.oracle().orc_fcap(S, V, R, C.byref(k))
        b = _harness.ref().ref_fcap(S, V, R, C.byref(k))
        assert a == b
