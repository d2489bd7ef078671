"""The lockstep harness (tests/_lockstep.py) on the CPU: the oracle resumed from
another oracle's snapshot reproduces that oracle's step bit for bit, and a
mistake planted in the snapshot's lists, records or forces is caught.

The GPU parity tests trust this harness to load a GPU implementation's state
into the oracle and to compare every list, record and force after the step;
here both sides are the oracle, so any difference is the harness's own."""
import numpy as np
import pytest

import _harness
import _lockstep
import _workloads


def _snap_of(sim):
    n = sim.n
    num, flat = sim.lists_flat()
    h = sim.history_flat()
    st = sim.state()
    return dict(pos=st["pos"], vel=st["vel"], angvel=st["angvel"], force=st["force"],
                pmove=sim.arr("pMove", np.float64, n).copy(), lqd=sim.arr("lqdCnt", np.int32, n).copy(),
                counts=num, partners=flat, rec=h[:, :8].copy(), brg=h[:, 8].astype(np.int32),
                nwall=sim.arr("nwall", np.int32, n).copy(), wlist=sim.arr("wlist", np.int32, 3 * n).reshape(n, 3),
                wrec=sim.wall_records(), flag=sim.counter("flag"))


EXACT = {"force": 0.0, "pos": 0.0, "vel": 0.0, "hist": 0.0}


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_resumed_oracle_reproduces_the_oracle(make):
    w = make()
    pos, vel, ang = _workloads.stirred(w)
    a = _harness.OracleSim(w.setup, pos, vel, ang)
    b = _harness.OracleSim(w.setup, pos, vel, ang)
    rebuilds = 0
    for t in range(150):
        _lockstep.load_into(b, _snap_of(a), t, first=(t == 0))
        rebuilds += b.step()
        a.step()
        r = _lockstep.compare_step(_snap_of(a), b, w, EXACT, f"step {t}")
        assert r["force_err"] == 0.0 and r["hist_err"] == 0.0
    assert rebuilds >= 1


def test_planted_mistakes_are_caught():
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    a = _harness.OracleSim(w.setup, pos, vel, ang)
    b = _harness.OracleSim(w.setup, pos, vel, ang)
    a.step(3)
    _lockstep.load_into(b, _snap_of(a), 3, first=False)
    a.step()
    b.step()
    good = _snap_of(a)
    _lockstep.compare_step(good, b, w, EXACT, "unchanged")
    i = int(np.flatnonzero(good["counts"] >= 2)[0])
    ii, _ = _lockstep.flat_slots(good["counts"])
    k = int(np.flatnonzero(ii == i)[0])
    cases = []
    s = {**good, "partners": good["partners"].copy()}
    s["partners"][[k, k + 1]] = s["partners"][[k + 1, k]]
    cases.append((s, "list of"))
    s = {**good, "counts": good["counts"].copy()}
    s["counts"][i] -= 1
    cases.append((s, "list lengths"))
    s = {**good, "rec": good["rec"].copy()}
    c = int(np.flatnonzero(good["rec"][:, 3] != 0)[0])
    s["rec"][c, 3] *= 1.0 + 1e-6
    cases.append((s, "history error"))
    # a particle without slip ties: any change of its force beyond 1e-12 is an error
    budget = _lockstep.slip_ties(b, w, good["counts"], b.history_flat())
    q = int(np.flatnonzero((budget == 0) & (np.abs(good["force"]).max(axis=1) > 0))[0])
    s = {**good, "force": good["force"].copy()}
    s["force"][q] *= 1.0 + 1e-6
    cases.append((s, "force error"))
    for snap, what in cases:
        with pytest.raises(AssertionError, match=what):
            _lockstep.compare_step(snap, b, w, {"force": 1e-12, "pos": 0.0, "vel": 0.0, "hist": 1e-12}, what)
