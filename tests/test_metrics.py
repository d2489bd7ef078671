"""Packing fraction and coordination number (CPU): dem_packing_metrics against
independent estimates."""
import numpy as np

from gpucode_gb300 import _abi, configs
from gpucode_gb300.engine import Setup, packing_metrics


def _setup_for(rad, R, H):
    """a set-up whose cylinder is (0, 0, R, Bw = 0, Tw = H), radii `rad` (reduced = SI here)"""
    n = len(rad)
    inp = configs.make_input(n, 1, 2 * rad.max(), 0.1, R, H, 2500.0, 1e7, 0.3, 0.3, 0.0, 1e6, 0, dt=1e-6)
    s = Setup.build(inp, 2 * rad)
    s.s.cyl.cir_x = 0.0
    s.s.cyl.cir_y = 0.0
    s.s.cyl.R = R
    s.s.cyl.Bw = 0.0
    s.s.cyl.Tw = H
    s.rad = rad.copy()
    return s


def test_packing_fraction_matches_monte_carlo():
    rng = np.random.Generator(np.random.PCG64(3))
    d = 1.0
    dia = rng.uniform(0.6, 1.0, 3000) * d
    R = 10.0
    pos = configs.deposit(dia, R, 0.0, 0.0, 6, 9)
    s = _setup_for(dia / 2, R, 100.0)
    m = packing_metrics(s, pos)
    # Monte-Carlo volume fraction in the same probe
    dmax = dia.max()
    tops = np.sort(pos[:, 2] + dia / 2)
    surf = tops[int(0.98 * (len(tops) - 1))]
    Rp, z0, z1 = R - 3 * dmax, 3 * dmax, surf - 3 * dmax
    npts = 400_000
    u = rng.uniform(size=(npts, 3))
    r = Rp * np.sqrt(u[:, 0])
    th = 2 * np.pi * u[:, 1]
    pts = np.column_stack([r * np.cos(th), r * np.sin(th), z0 + (z1 - z0) * u[:, 2]])
    from scipy.spatial import cKDTree

    tree = cKDTree(pos)
    inside = np.zeros(npts, bool)
    for k, idx in enumerate(tree.query_ball_point(pts, dmax / 2)):
        if idx:
            dd = np.linalg.norm(pos[idx] - pts[k], axis=1)
            inside[k] = (dd < dia[idx] / 2).any()
    mc = inside.mean()
    err = 3 * np.sqrt(mc * (1 - mc) / npts)
    assert abs(m["phi"] - mc) < max(err, 2e-3), (m, mc)
    assert m["n_probe"] > 100


def test_coordination_of_a_compressed_cubic_lattice_is_six():
    a = 0.999  # spacing just below the diameter: every lattice neighbour overlaps
    g = np.arange(-9, 10) * a
    X, Y, Z = np.meshgrid(g, g, np.arange(0, 30) * a + 0.5, indexing="ij")
    pos = np.column_stack([X.ravel(), Y.ravel(), Z.ravel()])
    pos = pos[np.hypot(pos[:, 0], pos[:, 1]) < 9.5]
    rad = np.full(len(pos), 0.5)
    s = _setup_for(rad, 10.0, 40.0)
    m = packing_metrics(s, pos)
    assert m["n_probe"] > 0
    assert abs(m["z"] - 6.0) < 1e-12
    # simple cubic: pi/6 of the volume (slightly more: spacing 0.999)
    assert abs(m["phi"] - np.pi / 6 / a ** 3) < 0.01
