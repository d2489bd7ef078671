"""Host input/output and set-up derivation (CPU).

dem_read_input + dem_build_setup replace ReadData.cpp, UnitReduce.cpp,
DiaInput.cpp and the constant derivation of main.cpp:328-348.  Where the
reference sources are present, its own ReadData/UnitReduce (compiled for the
CPU into oracle/_ref) read the same files and every derived quantity must agree
bit for bit: cell sizes and grid dimensions feed the integer cell hash."""
import ctypes as C
import math
import os

import numpy as np
import pytest

import _harness
import _workloads
from gpucode_gb300 import _abi, configs
from gpucode_gb300.engine import Setup


@pytest.fixture
def in_tmp(tmp_path):
    old = os.getcwd()
    os.chdir(tmp_path)
    yield tmp_path
    os.chdir(old)


def _cases():
    return [_workloads.small_dry(), _workloads.small_wet(), _workloads.small_wet(n=500, seed=9, n_levels=5)]


@pytest.mark.parametrize("k", [0, 1, 2])
def test_files_roundtrip_equals_direct_setup(in_tmp, k):
    w = _cases()[k]
    configs.write_heyi("heyi", w.inp, w.dia)
    s2 = Setup.from_files("heyi")
    # heyi.in carries no time step: the file path takes dt from dtFactor (ReadData.cpp:263)
    inp = _abi.DemInput.from_buffer_copy(bytes(w.inp))
    inp.dt_override = 0.0
    direct = Setup.build(inp, w.dia)
    assert bytes(s2.s) == bytes(direct.s)
    assert np.array_equal(s2.rad, direct.rad)
    assert np.array_equal(s2.plevel, direct.plevel) and np.array_equal(s2.nidx, direct.nidx)


@pytest.mark.parametrize("k", [0, 1, 2])
def test_setup_equals_reference_readdata(in_tmp, k):
    if not _harness.ref_available():
        pytest.skip(f"reference sources not found at {_harness.REF_SRC} (set DEM_REF_DIR)")
    w = _cases()[k]
    configs.write_heyi("heyi", w.inp, w.dia)
    mine = Setup.from_files("heyi")
    ref = _harness.ref()
    n, L = w.setup.n, w.setup.s.n_levels
    lvl = np.zeros(L, np.float64); plevel = np.zeros(n, np.int32); nneb = np.zeros(L, np.int32)
    npars = np.zeros(L, np.int32); nidx = np.zeros(n, np.int32); feed = np.zeros(2)
    cyl = _abi.CylinderBC(); mat = (_abi.MatType * 2)(); lqd = _abi.LIQUID(); prm = _abi.PARAMETER()
    ips = C.c_double(); fcap = C.c_int(); dem = np.zeros(11); st = C.c_int(); tp = C.c_double(); nout = C.c_int()
    rad = np.zeros(n); ncell = np.zeros(L, np.int32); grid = np.zeros((L, 3), np.int32); cs = np.zeros(L)
    unit = np.zeros(7)
    P = _abi.ptr
    ref.ref_read_setup.restype = C.c_int
    rc = ref.ref_read_setup(b"heyi", n, L, P(lvl), P(plevel), P(nneb), P(npars), P(nidx), C.byref(cyl), P(feed),
                            mat, C.byref(lqd), C.byref(prm), C.byref(ips), C.byref(fcap), P(dem), C.byref(st),
                            C.byref(tp), C.byref(nout), P(rad), P(ncell), P(grid), P(cs), P(unit))
    assert rc == 0
    s = mine.s
    assert np.array_equal(lvl, np.array(list(s.level_size)[:L]))
    assert np.array_equal(nneb, np.array(list(s.level_nnebors)[:L]))
    assert np.array_equal(npars, np.array(list(s.level_npars)[:L]))
    assert np.array_equal(plevel, mine.plevel) and np.array_equal(nidx, mine.nidx)
    assert np.array_equal(rad, mine.rad)
    assert np.array_equal(cs, np.array(list(s.cell_size)[:L]))
    assert np.array_equal(grid, np.array([[g.x, g.y, g.z] for g in list(s.grid_size)[:L]]))
    assert np.array_equal(ncell, np.array(list(s.num_cells)[:L]))
    # cir, R, Tw, Bw; the reference leaves topv/btmv uninitialised (malloc,
    # ReadData.cpp:118-129) -- this library sets them to 0
    assert bytes(cyl)[:40] == bytes(s.cyl)[:40]
    assert s.cyl.topv == 0.0 and s.cyl.btmv == 0.0
    assert bytes(mat) == bytes(s.mat)
    assert bytes(lqd) == bytes(s.lqd)
    for f in ("x", "y", "z"):
        assert getattr(prm.Origin, f) == getattr(s.prm.Origin, f)
        assert getattr(prm.EndPoint, f) == getattr(s.prm.EndPoint, f)
    assert prm.SearchGap == s.prm.SearchGap and prm.dt == s.prm.dt and prm.NP == s.prm.NP
    assert dem[0] == s.sim.dt and dem[2] == s.sim.cutGap
    assert unit.tolist() == [s.unit.rlunit, s.unit.rmunit, s.unit.rfunit, s.unit.reunit, s.unit.rsunit,
                             s.unit.rtunit, s.unit.rvunit]
    assert fcap.value == s.force_cap and ips.value == s.init_par_size
    assert feed[0] == s.feed.Lmin and feed[1] == s.feed.Lmax


def test_contact_constants_restate_main_cpp():
    """main.cpp:328-348, restated here independently of the library."""
    s = _workloads.small_wet().setup.s
    PI = 3.1415926
    m0, m1 = s.mat[0], s.mat[1]
    emod = (m0.emod * m0.emod) / (m0.emod + m0.emod)
    ystress = m0.yldp * m0.yldp / (m0.yldp + m0.yldp)
    ydsp = math.pow(PI * ystress / (2.0 * emod), 2.0)
    assert s.cal.emod == emod and s.cal.ystress == ystress and s.cal.ydsp_t == ydsp
    assert s.cal.yforce_t == 4.0 / 3.0 * emod * math.pow(ydsp, 1.5)
    assert s.cal.ystiff_t == PI * ystress
    assert s.cal.pois == 2.0 * (m0.pois * m0.pois) / (m0.pois + m0.pois)
    assert s.pwcal.emod == m0.emod and s.pwcal.ystress == m0.yldp
    assert s.pwcal.sfrc == math.pow(m1.sfrc * m1.sfrc, 0.5)
    # the yield mapping: yield overlap 1% of d at R* = d/4 -> ydsp_t = 0.04
    assert abs(s.cal.ydsp_t - 0.04) < 1e-14


def test_keyword_search_is_a_prefix_match(in_tmp):
    """ReadData.cpp:15-19 compares only strlen(key) characters: a file that
    lists SIZELEVEL_INPUT first makes the SIZELEVEL search land on it."""
    w = _workloads.small_dry()
    configs.write_heyi("heyi", w.inp, w.dia)
    txt = open("heyi.in").read().replace("SIZELEVEL\n1\n", "")
    txt = "SIZELEVEL_INPUT\nNo\n" + txt + "SIZELEVEL\n1\n"
    open("heyi.in", "w").write(txt)
    lib = _abi.load()
    inp = _abi.DemInput()
    rc = lib.dem_read_input(b"heyi", C.byref(inp), None)
    # "SIZELEVEL" matched the SIZELEVEL_INPUT line; the value read after it is not a number
    assert rc == _abi.DEM_ERR_IO


def test_missing_keyword_is_an_io_error(in_tmp):
    w = _workloads.small_dry()
    configs.write_heyi("heyi", w.inp, w.dia)
    txt = open("heyi.in").read().replace("LIQUID\n", "LIQUIDX\n")
    open("heyi.in", "w").write(txt.replace("LIQUIDX", "LQ"))
    lib = _abi.load()
    inp = _abi.DemInput()
    assert lib.dem_read_input(b"heyi", C.byref(inp), None) == _abi.DEM_ERR_IO
    assert b"LIQUID" in lib.dem_last_error()
    assert lib.dem_read_input(b"nonexistent_file", C.byref(inp), None) == _abi.DEM_ERR_IO


def test_diameter_list_tiles_and_ignores_trailing_whitespace(in_tmp):
    w = _workloads.small_dry(n=10)
    configs.write_heyi("heyi", w.inp, w.dia)
    open("heyi_dia.dat", "w").write("PARTICLE DIAMETER\n0.001\n0.0015\n0.002\n\n  \n")
    s = Setup.from_files("heyi")
    want = np.array([0.001, 0.0015, 0.002] * 4)[:10] / 2.0 / s.s.unit.rlunit
    assert np.array_equal(s.rad, want)


def test_wrtec_matches_reference_byte_for_byte(in_tmp):
    if not _harness.ref_available():
        pytest.skip(f"reference sources not found at {_harness.REF_SRC} (set DEM_REF_DIR)")
    lib = _abi.load()
    ref = _harness.ref()
    rng = np.random.Generator(np.random.PCG64(5))
    n = 57
    pos, vel, frc, ang = (rng.standard_normal((n, 3)) for _ in range(4))
    rad = rng.uniform(0.2, 0.5, n)
    sim = _abi.SIMULATION()
    unit = _abi.UNIT()
    unit.rtunit = 0.0123
    P = _abi.ptr
    outs = {}
    for tag, L in (("mine", lib), ("ref", ref)):
        for outs_i in (0, 1):
            sim.Outs = outs_i
            sim.ctime = 1.5 + outs_i
            L.WrtTec(P(pos), P(vel), P(frc), P(ang), C.byref(sim), P(rad), C.byref(unit), n, n)
        outs[tag] = open("particle_info.dat", "rb").read()
    assert outs["mine"] == outs["ref"]


def test_binary_columns_hold_the_tecplot_quantities(in_tmp):
    """WrtBin writes WrtTec's quantities and zones as full-precision columns:
    every value agrees with the Tecplot text to its 5 printed decimals, and
    the time of each zone to its 6"""
    from gpucode_gb300.output import read_columns

    lib = _abi.load()
    rng = np.random.Generator(np.random.PCG64(9))
    n = 1000
    pos, vel, frc, ang = (rng.standard_normal((n, 3)) * 3 for _ in range(4))
    rad = rng.uniform(0.2, 0.5, n)
    sim = _abi.SIMULATION()
    unit = _abi.UNIT()
    unit.rtunit = 0.0123
    P = _abi.ptr
    for outs_i in (0, 1, 2):
        sim.Outs = outs_i
        sim.ctime = 1.5 + outs_i
        lib.WrtTec(P(pos), P(vel), P(frc), P(ang), C.byref(sim), P(rad), C.byref(unit), n, n)
        lib.WrtBin(P(pos), P(vel), P(frc), P(ang), C.byref(sim), P(rad), C.byref(unit), n, n)
    names, zones = read_columns("particle_info.bin")
    assert names == ["X", "Y", "Z", "R", "VX", "VY", "VZ", "W", "F"] and len(zones) == 3
    text = open("particle_info.dat").read().splitlines()
    rows = [ln for ln in text if ln and ln[0] in " -0123456789" and not ln.startswith("ZONE")]
    tec = np.array([[float(x) for x in ln.split()] for ln in rows]).reshape(3, n, 9)
    times = [float(ln.split('"')[1].split()[0]) for ln in text if ln.startswith("ZONE")]
    for k, z in enumerate(zones):
        assert z["n"] == n and abs(z["time"] - times[k]) <= 5e-7
        cols = np.stack([z[c] for c in names], 1)
        np.testing.assert_allclose(cols, tec[k], rtol=0, atol=5.01e-6)
        np.testing.assert_array_equal(z["X"], pos[:, 0])
        np.testing.assert_array_equal(z["W"], np.sqrt((ang * ang).sum(1)))


def test_loadpara_reads_checkpoint_header(in_tmp):
    lib = _abi.load()
    open("heyi_dump.dat", "wb").write(b"SYSTEM Info\n1234 7 1200\n" + b"\x00\x01binary")
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    lib.LoadPara(b"heyi_dump.dat", C.byref(a), C.byref(b), C.byref(c))
    assert (a.value, b.value, c.value) == (1234, 7, 1200)


def test_particle_feed_is_seeded_and_non_overlapping():
    lib = _abi.load()
    n = 400
    rad = np.full(n, 0.5)
    fz = _abi.FeedZone(Lmax=30.0, Lmin=2.0)
    cyl = _abi.CylinderBC(cir_x=0.0, cir_y=0.0, R=6.0, Tw=60.0, Bw=0.0)
    res = []
    for _ in range(2):
        lib.dem_set_feed_seed(42)
        pos = np.zeros((n, 3))
        lib.ParticleFeed.restype = C.c_int
        got = lib.ParticleFeed(C.byref(fz), C.byref(cyl), C.c_double(1.0), _abi.ptr(pos), _abi.ptr(rad), 0, n)
        res.append((got, pos.copy()))
    assert res[0][0] == res[1][0] > 0 and np.array_equal(res[0][1], res[1][1])
    got, pos = res[0]
    p = pos[:got]
    d = np.linalg.norm(p[:, None, :] - p[None, :, :], axis=-1) + np.eye(got) * 1e9
    assert d.min() >= 1.0 + 0.002 - 1e-12
    assert (np.hypot(p[:, 0], p[:, 1]) <= 6.0 - 0.5 + 1e-12).all()
    assert ((p[:, 2] >= 2.0) & (p[:, 2] <= 30.0)).all()
