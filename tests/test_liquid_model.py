"""The per-contact liquid model in the oracle (CPU): per-pair bridge volumes, per-
particle contact angles and the capillary regression with its contact-angle
terms (Willett et al. 2000), of which the reference's fCap (kernel.cu:65-81) is
the zero-angle case.  The GPU paths are checked against this oracle in
tests/test_gpu_liquid.py."""
import ctypes as C
import math

import numpy as np

import _harness
import _workloads


def _lib():
    return _harness.oracle()


def _consts(vmin=0.005, vmax=0.02, theta_max=math.radians(30), seed=7):
    k = _harness.OConsts()
    k.lqd.gapmn = 2.5e-3
    k.lqd.stension = 1.0
    k.lqd_mode, k.lqd_vol_min, k.lqd_vol_max, k.lqd_theta_max, k.lqd_seed = 1, vmin, vmax, theta_max, seed
    return k


def test_zero_angle_is_the_reference_regression():
    """at theta = 0 the fit's coefficients are fCap's: the same force to rounding"""
    lib = _lib()
    k = _harness.OConsts()
    k.lqd.gapmn, k.lqd.stension = 2.5e-3, 0.7
    rng = np.random.Generator(np.random.PCG64(3))
    for _ in range(2000):
        S = 10 ** rng.uniform(-4, -0.3)
        V8 = 10 ** rng.uniform(-4.5, -1.2)
        effR = rng.uniform(0.2, 1.0)
        ref = lib.orc_fcap(S, V8, effR, C.byref(k))
        got = 2 * 3.1415926 * effR * 0.7 * lib.orc_willett(max(2.5e-3, S), V8, 0.0)
        assert abs(got - ref) <= 1e-13 * abs(ref), (S, V8, got, ref)


def test_contact_angle_weakens_the_bridge_like_cos_theta():
    """F* falls with the contact angle over [0, 30 deg] while the separation is
    below half the bridge's length scale sqrt(V*) (nearer rupture the fit is
    flat in the angle); at small separation and volume F*(theta) / F*(0) is
    within 3 % of cos(theta), the limit of the toroidal bridge theory that the
    fit reproduces"""
    lib = _lib()
    for V8 in (1e-4, 1e-3, 6.5e-3, 3e-2):
        for S in (1e-3, 3e-3, 1e-2, 3e-2, 0.1):
            if S > 0.5 * math.sqrt(V8):
                continue
            prev = None
            for deg in range(0, 31, 5):
                f = lib.orc_willett(S, V8, math.radians(deg))
                assert 0.0 < f < 1.0
                if prev is not None:
                    assert f < prev, (V8, S, deg)
                prev = f
    f0 = lib.orc_willett(1e-3, 1e-4, 0.0)
    for deg in (10, 20, 30):
        ratio = lib.orc_willett(1e-3, 1e-4, math.radians(deg)) / f0
        assert abs(ratio - math.cos(math.radians(deg))) < 0.03 * math.cos(math.radians(deg)), (deg, ratio)


def test_rupture_distance_grows_with_the_angle():
    lib = _lib()
    for V in (1e-4, 1e-3, 1e-2):
        r0 = lib.orc_rupture(V, 0.0)
        assert r0 == 0.99 * V ** 0.33
        assert abs(lib.orc_rupture(V, 0.4) - 1.2 * r0) <= 1e-15 * r0


def test_pair_volumes_and_angles():
    """bridge volumes: the same for both directions of a pair, a fraction in
    [vol_min, vol_max) of the smaller sphere's volume, spread uniformly;
    contact angles uniform in [0, theta_max)"""
    lib = _lib()
    k = _consts()
    rng = np.random.Generator(np.random.PCG64(5))
    fr = []
    for _ in range(4000):
        a, b = (int(x) for x in rng.integers(0, 10_000_000, 2))
        rmin = rng.uniform(0.1, 0.5)
        v = lib.orc_pair_volume(C.byref(k), a, b, rmin)
        assert v == lib.orc_pair_volume(C.byref(k), b, a, rmin)
        fr.append(v / (3.1415926 / 6.0 * (2 * rmin) ** 3))
    fr = np.array(fr)
    assert fr.min() >= 0.005 and fr.max() < 0.02
    hist, _ = np.histogram(fr, bins=10, range=(0.005, 0.02))
    assert hist.min() > 300 and hist.max() < 500
    th = np.array([lib.orc_theta(i, 7, math.radians(30)) for i in range(4000)])
    assert th.min() >= 0.0 and th.max() < math.radians(30)
    assert abs(th.mean() - math.radians(15)) < 0.01
    assert lib.orc_pair_volume(C.byref(_consts(seed=8)), 1, 2, 0.3) != lib.orc_pair_volume(C.byref(k), 1, 2, 0.3)


def test_oracle_steps_a_wet_bed_with_per_contact_bridges():
    """the per-contact model changes the bridge forces of a wet bed and nothing
    else: the same contacts and lists, different capillary forces"""
    w = _workloads.small_wet()
    pos, vel, ang = _workloads.stirred(w)
    a = _harness.OracleSim(w.setup, pos, vel, ang)
    b = _harness.OracleSim(w.setup, pos, vel, ang)
    b.set_liquid_model(1, 0.005, 0.02, math.radians(30), 11)
    a.step(2)
    b.step(2)
    na, la = a.lists_flat()
    nb, lb = b.lists_flat()
    assert np.array_equal(na, nb) and np.array_equal(la, lb)
    fa, fb = a.state()["force"], b.state()["force"]
    assert np.abs(fa - fb).max() > 1e-3 * np.abs(fa).max()
    assert b.arr("lqdCnt", np.int32, w.setup.n).sum() > 0
    a.close()
    b.close()
