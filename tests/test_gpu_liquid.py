"""The per-contact liquid model (dem_set_liquid_model, liquid.cuh) on the GPU
against the oracle's restatement (oracle/dem_oracle.c), in lockstep
(tests/_lockstep.py): bridge volumes per pair, contact angles per particle and
the capillary regression with its contact-angle terms.  FP64 to 1e-12 with
bridge flags bit-exact; mixed precision to the mixed tolerances."""
import math

import numpy as np
import pytest

import _lockstep
import _workloads
from gpucode_gb300 import _abi
from gpucode_gb300.engine import Engine

pytestmark = pytest.mark.gpu

FP64_TOL = {"force": 1e-12, "pos": 1e-14, "vel": 1e-12, "hist": 1e-12}
MIXED_TOL = {"force": 2e-5, "pos": 1e-9, "vel": 1e-5, "angvel": 2e-5, "hist": 1e-5}
MODEL = dict(vol_min=0.005, vol_max=0.02, theta_max=math.radians(30), seed=11)


def _engine(w, precision, pairs="auto", model=MODEL):
    e = Engine(w.setup, precision=precision, pairs=pairs, use_graph=(precision == "mixed"))
    e.set_liquid_model("per_contact", **model)
    return e


def test_fp64_engine_per_contact_liquid_lockstep(cuda):
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    eng = _engine(w, "fp64")
    worst = _lockstep.run(eng, w, pos, vel, ang, steps=250, tol=FP64_TOL, liquid=dict(mode=1, **MODEL))
    assert worst["rebuilds"] >= 2, worst
    assert eng.stats()["bridges"] > 0
    eng.close()


@pytest.mark.parametrize("pairs", ["warp", "thread"])
def test_mixed_engine_per_contact_liquid_lockstep(cuda, pairs):
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    eng = _engine(w, "mixed", pairs)
    worst = _lockstep.run(eng, w, pos, vel, ang, steps=250, tol=MIXED_TOL, mismatch_budget=0.01,
                          liquid=dict(mode=1, **MODEL))
    assert worst["rebuilds"] >= 2, worst
    eng.close()


def test_per_contact_model_changes_the_bridges_only(cuda):
    """the same bed in both models: identical contacts and lists, different
    capillary forces; with vol_min = vol_max and theta_max = 0 every pair's
    bridge holds the same fraction of its smaller sphere"""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    out = {}
    for name in ("reference", "per_contact"):
        e = Engine(w.setup, precision="fp64", use_graph=False)
        if name == "per_contact":
            e.set_liquid_model("per_contact", **MODEL)
        e.set_state(pos, vel, ang)
        e.step(1)
        out[name] = (e.get_state()["force"], e.neighbors(_lockstep.max_per(w)))
        e.close()
    (fa, (na, pa)), (fb, (nb, pb)) = out["reference"], out["per_contact"]
    assert np.array_equal(na, nb) and np.array_equal(pa, pb)
    assert np.abs(fa - fb).max() > 1e-3 * np.abs(fa).max()


def test_liquid_model_arguments_are_checked(cuda):
    w = _workloads.small_wet()
    e = Engine(w.setup, precision="mixed")
    for bad in (dict(vol_min=0.0), dict(vol_min=0.02, vol_max=0.01), dict(theta_max=2.0), dict(vol_max=1.5)):
        with pytest.raises(_abi.DemError):
            e.set_liquid_model("per_contact", **{**MODEL, **bad})
    e.set_liquid_model("per_contact", **MODEL)
    pos, vel, ang = _workloads.stirred(w)
    e.set_state(pos, vel, ang)
    e.step(2)
    with pytest.raises(_abi.DemError, match="before the first dem_step"):
        e.set_liquid_model("reference")
    e.close()
