"""ParticleFeedDevice: the reference's particle feed (ParticleFeed.cpp:8-72) on
the device arrays.  Checked: its placement rules (inside the cylinder less the
particle's radius, inside the feed band, a clearance of r_i + r_j + 0.002 from
every particle already there and from each other), reproducibility (the same
seed, the same positions), the 60000-per-call limit, the stop at the first
particle without room (the kept particles are a prefix, nothing is written
past it, a capacity below it is filled), and agreement of the position
distribution with the host ParticleFeed."""
import ctypes as C
import time

import numpy as np
import pytest

from gpucode_gb300 import _abi

pytestmark = pytest.mark.gpu

CLEAR = 0.002


def _feed(pos, rad, n0, NP, fz, cyl, seed):
    import torch

    lib = _abi.load()
    f = lib.ParticleFeedDevice
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_ulonglong]
    dpos = torch.tensor(pos, dtype=torch.float64, device="cuda").contiguous()
    drad = torch.tensor(rad, dtype=torch.float64, device="cuda").contiguous()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    got = f(C.byref(fz), C.byref(cyl), 1.0, dpos.data_ptr(), drad.data_ptr(), n0, NP, seed)
    dt = time.perf_counter() - t0
    assert got >= 0, lib.dem_last_error()
    return got, dpos.cpu().numpy(), dt


def _old_bed(n0, R, zmax, rad, seed):
    """n0 non-overlapping spheres below zmax (a loose lattice, seeded jitter)"""
    rng = np.random.default_rng(seed)
    a = 2.0 * rad.max() + 0.05
    xs = np.arange(-R + a, R - a, a)
    pts = [(x, y, z) for z in np.arange(a, zmax, a) for y in xs for x in xs if np.hypot(x, y) < R - a]
    pts = np.array(pts[:n0]) + rng.uniform(-0.02, 0.02, (n0, 3))
    assert len(pts) == n0
    return pts


def _check_valid(p, rad, n0, got, fz, cyl):
    from scipy.spatial import cKDTree

    new = p[n0:got]
    rn = rad[n0:got]
    assert (np.hypot(new[:, 0] - cyl.cir_x, new[:, 1] - cyl.cir_y) <= cyl.R - rn + 1e-12).all()
    assert ((new[:, 2] >= fz.Lmin) & (new[:, 2] <= fz.Lmax)).all()
    allp, allr = p[:got], rad[:got]
    pairs = cKDTree(allp).query_pairs(2.0 * allr.max() + CLEAR, output_type="ndarray")
    pairs = pairs[(pairs[:, 0] >= n0) | (pairs[:, 1] >= n0)]  # old-old pairs are not the feed's
    d = np.linalg.norm(allp[pairs[:, 0]] - allp[pairs[:, 1]], axis=1)
    assert (d >= allr[pairs[:, 0]] + allr[pairs[:, 1]] + CLEAR - 1e-12).all()


def test_device_feed_places_valid_particles_reproducibly(cuda):
    n0, NP, R = 300, 1300, 6.0
    rng = np.random.default_rng(5)
    rad = rng.uniform(0.3, 0.5, NP)
    pos = np.zeros((NP, 3))
    pos[:n0] = _old_bed(n0, R, 6.0, rad, 1)
    fz = _abi.FeedZone(Lmax=30.0, Lmin=4.0)  # the band reaches into the old bed's top
    cyl = _abi.CylinderBC(cir_x=0.0, cir_y=0.0, R=R, Tw=60.0, Bw=0.0)
    got, p1, _ = _feed(pos, rad, n0, NP, fz, cyl, 7)
    assert got == NP
    _check_valid(p1, rad, n0, got, fz, cyl)
    assert np.array_equal(p1[:n0], pos[:n0])  # old particles untouched
    got2, p2, _ = _feed(pos, rad, n0, NP, fz, cyl, 7)
    assert got2 == got and np.array_equal(p1, p2)
    got3, p3, _ = _feed(pos, rad, n0, NP, fz, cyl, 8)
    assert not np.array_equal(p1[n0:got3], p3[n0:got3])


def test_device_feed_stops_at_the_first_particle_without_room(cuda):
    n0, NP, R = 0, 3000, 3.0
    rad = np.full(NP, 0.5)
    pos = np.zeros((NP, 3))
    fz = _abi.FeedZone(Lmax=4.0, Lmin=1.0)  # room for a few dozen
    cyl = _abi.CylinderBC(cir_x=1.0, cir_y=-2.0, R=R, Tw=60.0, Bw=0.0)
    got, p, _ = _feed(pos, rad, n0, NP, fz, cyl, 11)
    assert 10 < got < NP
    _check_valid(p, rad, n0, got, fz, cyl)
    assert (p[got:] == 0.0).all()  # nothing written past the batch
    # a capacity below what the band holds is filled completely
    k = got // 2
    got_k, pk, _ = _feed(pos, rad, n0, n0 + k, fz, cyl, 11)
    assert got_k == k
    _check_valid(pk, rad, n0, got_k, fz, cyl)


def test_device_feed_places_at_most_60000_per_call(cuda):
    n0, NP, R = 0, 70000, 30.0
    rad = np.full(NP, 0.5)
    pos = np.zeros((NP, 3))
    fz = _abi.FeedZone(Lmax=62.0, Lmin=2.0)
    cyl = _abi.CylinderBC(cir_x=0.0, cir_y=0.0, R=R, Tw=100.0, Bw=0.0)
    got, p, dt = _feed(pos, rad, n0, NP, fz, cyl, 3)
    assert got == 60000, got
    _check_valid(p, rad, n0, got, fz, cyl)
    assert dt < 5.0, dt
    # a second call continues from there
    got2, p2, _ = _feed(p, rad, got, NP, fz, cyl, 4)
    assert got < got2 <= NP
    _check_valid(p2, rad, 0, got2, fz, cyl)


def test_device_feed_draws_like_the_host_feed(cuda):
    """the same draw formulas (angle, triangular radius fold, height): the
    radial and height distributions of a sparse feed agree with the host
    ParticleFeed's"""
    n0, NP, R = 0, 1500, 12.0
    rad = np.full(NP, 0.4)
    fz = _abi.FeedZone(Lmax=40.0, Lmin=2.0)
    cyl = _abi.CylinderBC(cir_x=0.0, cir_y=0.0, R=R, Tw=60.0, Bw=0.0)
    got, pd, _ = _feed(np.zeros((NP, 3)), rad, n0, NP, fz, cyl, 21)
    lib = _abi.load()
    lib.dem_set_feed_seed(21)
    ph = np.zeros((NP, 3))
    lib.ParticleFeed.restype = C.c_int
    goth = lib.ParticleFeed(C.byref(fz), C.byref(cyl), C.c_double(1.0), _abi.ptr(ph), _abi.ptr(rad), 0, NP)
    assert got == goth == NP
    from scipy.stats import ks_2samp

    rd, rh = np.hypot(pd[:, 0], pd[:, 1]), np.hypot(ph[:, 0], ph[:, 1])
    assert ks_2samp(rd, rh).pvalue > 1e-3
    assert ks_2samp(pd[:, 2], ph[:, 2]).pvalue > 1e-3
