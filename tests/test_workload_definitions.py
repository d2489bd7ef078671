"""The seeded synthetic workloads (gpucode_gb300/configs.py) against the
configurations they stand for (CPU only).

dry5k: 5,000 spheres of 1 mm, rho 2500, E 1e7, nu 0.3, mu 0.3, yield overlap 1 %
of d, restitution 0.7 through the reference's damping coefficient dmpn
(kernel.cu:164), cylinder R = 8 mm, a jittered hexagonal lattice (+-0.05 mm)
from z = 2 mm, dt 1 us, skin 0.1 d, one size level, no liquid.
wet200k: log-normal diameters (median 1 mm, sigma_ln 0.2) kept in [0.5, 2] mm,
R = 25 mm, REALSIZE 2 mm, four size levels, surface tension 0.072 N/m, dt 0.5 us.
The reference has no yield-overlap or restitution knob: yldp and dmpn are
derived (kernel.cu:104-165, main.cpp:328-348)."""
import math

import numpy as np
import pytest

import _harness
from gpucode_gb300 import configs
from gpucode_gb300.engine import Setup


@pytest.fixture(scope="module")
def dry():
    return configs.dry()


def test_dry_material_cylinder_and_steps(dry):
    inp = dry.inp
    d = 1e-3
    assert dry.setup.n == 5000 and np.all(dry.dia == d)
    rho, E, nu, mu, rfrc, dmpn, yldp = list(inp.mat[0])[:7]
    assert (rho, E, nu, mu, rfrc) == (2500.0, 1.0e7, 0.3, 0.3, 0.0)
    assert list(inp.mat[1])[:7] == list(inp.mat[0])[:7]  # the wall takes the particle material
    assert inp.cyl_r == 8e-3 and inp.n_levels == 1 and inp.force_cap == 0
    assert inp.dt_override == 1e-6 and inp.cut_gap == pytest.approx(0.1) and dry.steps == 20_000
    # yield overlap 1 % of d at R* = d/4: ydsp_t = (PI ystress / (2 E*))^2 = 0.04 (kernel.cu:120,
    # main.cpp:333-334, with the reference's PI = 3.1415926 of heydem.h:15)
    e0 = E / (1 - nu * nu)
    emod = e0 * e0 / (e0 + e0)
    ystress = yldp * yldp / (yldp + yldp)
    assert (configs.PI_REF * ystress / (2 * emod)) ** 2 == pytest.approx(0.04, rel=1e-12)
    # restitution 0.7 at the 0.5 m/s impact the damping was calibrated for
    e = configs.normal_law_restitution(dmpn, 0.5, d, rho, E, nu, yldp)
    assert e == pytest.approx(0.7, abs=2e-3)
    assert configs.normal_law_restitution(0.0, 0.5, d, rho, E, nu, yldp) > 0.7 > 0.0 < dmpn


def test_dry_lattice_geometry(dry):
    p, d = dry.pos0, 1e-3
    r_axis = np.hypot(p[:, 0], p[:, 1])
    assert r_axis.max() + d / 2 <= 8e-3
    # the lowest layer's centres: z0 + d/2 plus the lattice offset and the +-0.05 mm jitter
    assert p[:, 2].min() >= 2e-3 + d / 2 - 1e-12
    layer0 = p[p[:, 2] < 2e-3 + d / 2 + 2 * 0.05e-3 + 1e-12]
    assert len(layer0) > 100
    # layers 1.12 d * sqrt(2/3) apart: the heights cluster within the jitter
    a = 1.12 * d
    dz = a * math.sqrt(2.0 / 3.0)
    k = np.round((p[:, 2] - p[:, 2].min()) / dz)
    off = p[:, 2] - (p[:, 2].min() + k * dz)
    assert np.abs(off).max() <= 2 * 0.05e-3 + 1e-12
    # the fill starts at rest, and the seed makes it: same seed same bed, other seed another
    again = configs.dry()
    other = configs.dry(seed=7)
    assert np.array_equal(again.pos0, p) and not np.array_equal(other.pos0, p)


def test_wet_size_distribution():
    dia = configs.lognormal_diameters(200_000, 1e-3, 0.2, 0.5e-3, 2.0e-3, seed=2)
    assert len(dia) == 200_000 and dia.min() >= 0.5e-3 and dia.max() <= 2.0e-3
    ln = np.log(dia / 1e-3)
    # truncation at ln 2 = 3.47 sigma hardly moves the median or the spread
    assert abs(np.median(ln)) < 0.005
    assert np.std(ln) == pytest.approx(0.2, rel=0.01)
    assert np.array_equal(dia, configs.lognormal_diameters(200_000, 1e-3, 0.2, 0.5e-3, 2.0e-3, seed=2))


def test_wet_set_up():
    w = configs.wet(n=20_000, packing="lattice")
    inp = w.inp
    assert inp.n_levels == 4 and inp.real_size == 2e-3 and inp.cyl_r == 25e-3
    assert inp.force_cap == 1 and inp.lqd[0] == 0.072 and inp.dt_override == 5e-7
    assert list(inp.mat[0])[:5] == [2500.0, 1.0e7, 0.3, 0.3, 0.0]
    assert w.setup.s.n_levels == 4 and w.setup.n == 20_000
    assert w.dia.min() >= 0.5e-3 and w.dia.max() <= 2.0e-3


def test_dry_restitution_under_the_oracle():
    """two of the dry workload's spheres meeting head-on at 0.5 m/s, stepped by
    the oracle (the reference's contact law and integrator, kernel.cu:89-228,
    :563-606) at the workload's 1 us step: they part at 0.7 of the impact speed"""
    d = 1e-3
    yldp = configs.yldp_for_yield_overlap(0.01, configs.E_YOUNG, configs.NU)
    dmpn = configs.calibrate_dmpn(0.7, 0.5, d, configs.RHO, configs.E_YOUNG, configs.NU, yldp)
    inp = configs.make_input(2, 1, d, 0.1, 8e-3, 20e-3, configs.RHO, configs.E_YOUNG, configs.NU, configs.MU,
                             dmpn, yldp, 0, dt=1e-6)
    st = Setup.build(inp, np.full(2, d))
    vunit, lunit = st.s.unit.rvunit, st.s.unit.rlunit
    pos = np.array([[-0.55e-3, 0.0, 5e-3], [0.55e-3, 0.0, 5e-3]])
    vel = np.array([[0.25, 0.0, 0.0], [-0.25, 0.0, 0.0]])
    sim = _harness.OracleSim(st, st.to_reduced(pos), vel / vunit)
    try:
        closing = []
        for _ in range(2000):
            sim.step(1)
            s = sim.state()
            p, v = s["pos"], s["vel"]
            closing.append((v[0, 0] - v[1, 0]) * vunit)
            gap = (p[1, 0] - p[0, 0]) * lunit - d
            if gap > 1e-5 and closing[-1] < 0:
                break
    finally:
        sim.close()
    assert closing[0] == pytest.approx(0.5, rel=1e-6)  # gravity acts on both alike
    assert closing[-1] < 0 and len(closing) < 1000
    assert -closing[-1] / closing[0] == pytest.approx(0.7, abs=5e-3)
