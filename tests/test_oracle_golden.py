"""The oracle against golden fixtures generated from the reference's own kernels
(tests/golden/make_golden.py).  Integer outputs (hashes, sorted order, lists,
wall lists, load stages, bridge flags, bridge counts) must match exactly;
floating-point outputs must match to 1e-12 relative -- exactly on the x86
host that made them, within last-ulp libm differences (pow/exp/log) on other
hosts such as the aarch64 GPU machine."""
import platform
from pathlib import Path

import numpy as np
import pytest

import _harness
from gpucode_gb300._abi import DemSetup
from gpucode_gb300.engine import Setup

GOLDEN = Path(__file__).resolve().parent / "golden"
INT_KEYS = {"lqdCnt", "hash", "index", "Num_Nebor", "nwall", "wlist", "lists"}


def _load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    s = DemSetup.from_buffer_copy(z["setup_bytes"].tobytes())
    setup = Setup(s, z["rad"].copy(), z["plevel"].copy(), z["nidx"].copy())
    return z, setup


SAME_HOST = platform.machine() == "x86_64"


def _tol(t):
    """Exact on the x86_64 host the fixtures were made on.  Elsewhere: 1e-12
    after the first step; later checkpoints of these stirred, colliding beds
    amplify last-ulp libm differences, so 1e-9 there."""
    if SAME_HOST:
        return 0.0
    return 1e-12 if t == 1 else 1e-9


@pytest.mark.parametrize("name", ["pin_dry300", "pin_wet400"])
def test_oracle_matches_golden(name):
    z, setup = _load(name)
    sim = _harness.OracleSim(setup, z["pos0"], z["vel0"], z["ang0"])
    marks = [int(m) for m in z["marks"]]
    for t in range(1, max(marks) + 1):
        sim.step()
        if t not in marks:
            continue
        got = _harness.sim_arrays(sim)
        rtol = _tol(t)
        for key in z.files:
            if not key.startswith(f"s{t}:"):
                continue
            k = key.split(":", 1)[1]
            want = z[key]
            if k in INT_KEYS:
                assert np.array_equal(got[k], want), f"{name} step {t}: {k}"
            elif k == "hist":
                # stage and bridge columns are integers
                assert np.array_equal(got[k][:, 7:], want[:, 7:]), f"{name} step {t}: stages/bridges"
                np.testing.assert_allclose(got[k][:, :7], want[:, :7], rtol=rtol, atol=1e-300,
                                           err_msg=f"{name} step {t}: history")
            else:
                np.testing.assert_allclose(got[k], want, rtol=rtol, atol=1e-300, err_msg=f"{name} step {t}: {k}")
    assert sim.counter("rebuilds") == int(z["rebuilds"])
