"""BldNeborListNoAlloc: the neighbour build with its cell-sort scratch in a
fixed device array of the library, against BldNeborList (heydem.h:547) and
against the oracle on the same inputs.  Every output is integer and must match
bit for bit.  Its error word is checked on inputs that set both of its bits,
with guard words around every output buffer.

The file name sorts last so the GPU test also runs after every other test of a
session; it sets up all the state it uses and passes alone as well."""
import ctypes as C

import numpy as np
import pytest

import _harness
import _workloads
from gpucode_gb300 import _abi

STATIC_SCRATCH_BYTES = 16 << 20
SCAN_TILE = 2048


def _declare(lib):
    P = C.c_void_p
    lib.BldNeborList.argtypes = [P, P, P, P, P, _abi.SEARCHCELL, P, P, P, P, C.c_int, P, C.c_int, P, P, P,
                                 C.c_int, P]
    lib.BldNeborList.restype = None
    lib.BldNeborListNoAlloc.argtypes = [P, P, P, P, P, _abi.SEARCHCELL, P, P, P, P, C.c_int, P, C.c_int, P, P,
                                        P, C.c_int, P, P]
    lib.BldNeborListNoAlloc.restype = C.c_int
    lib.IndexOffset.argtypes = [P, P, C.c_int]
    lib.dem_compat_errors.restype = C.c_int


def _scratch_bytes(n, ncells):
    return 4 * (2 * n + -(-ncells // SCAN_TILE) + 64)


def test_sizes_beyond_the_static_scratch_are_rejected_before_any_launch():
    """host-side checks only: every pointer is NULL, nothing reaches the device"""
    lib = _abi.load()
    _declare(lib)
    cell = _abi.SEARCHCELL(0, 0, 0)
    n_max = (STATIC_SCRATCH_BYTES // 4 - 64 - 1) // 2
    assert _scratch_bytes(n_max, 1) <= STATIC_SCRATCH_BYTES < _scratch_bytes(n_max + 1, 1)
    err = C.c_void_p(16)  # never dereferenced: the size check comes first
    for n, ncells in ((n_max + 1, 1), (n_max, 200 * SCAN_TILE), (2_100_000, 10)):
        assert _scratch_bytes(n, ncells) > STATIC_SCRATCH_BYTES
        st = lib.BldNeborListNoAlloc(None, None, None, None, None, cell, None, None, None, None, 1, None, ncells,
                                     None, None, None, n, None, err)
        assert st == _abi.DEM_ERR_ARG
        msg = lib.dem_last_error().decode()
        assert "static scratch holds 16777216" in msg and str(n) in msg, msg
    st = lib.BldNeborListNoAlloc(None, None, None, None, None, cell, None, None, None, None, 1, None, 10, None,
                                 None, None, 10, None, None)
    assert st == _abi.DEM_ERR_ARG and "d_err is NULL" in lib.dem_last_error().decode()
    st = lib.BldNeborListNoAlloc(None, None, None, None, None, cell, None, None, None, None, 1, None, 10, None,
                                 None, None, -1, None, err)
    assert st == _abi.DEM_ERR_ARG and "bad sizes" in lib.dem_last_error().decode()


class _Dev:
    """the set-up's level tables on the device, constants uploaded"""

    def __init__(self, w, lib, torch, nneb=None):
        s = w.setup.s
        self.n, self.S, self.L, self.ncells = w.setup.n, int(s.n_pp_slots), int(s.n_levels), int(s.sys_ncells)
        L, dev = self.L, "cuda"
        k = _harness.consts_of(w.setup)
        lib.setMaterial(C.byref(k.mat))
        lib.setLiquid(C.byref(k.lqd))
        lib.setParameters(C.byref(k.prm))
        lib.setCalpara(C.byref(k.cal), C.byref(k.pwcal))
        self.rad = torch.tensor(w.setup.rad, device=dev)
        self.plevel = torch.tensor(w.setup.plevel, device=dev)
        self.nidx = torch.tensor(w.setup.nidx, device=dev)
        self.level_size = torch.tensor(list(s.level_size)[:L], dtype=torch.float64, device=dev)
        self.nneb = torch.tensor(nneb if nneb is not None else list(s.level_nnebors)[:L], dtype=torch.int32,
                                 device=dev)
        self.npars = torch.tensor(list(s.level_npars)[:L], dtype=torch.int32, device=dev)
        self.cellsize = torch.tensor(list(s.cell_size)[:L], dtype=torch.float64, device=dev)
        self.grid = torch.tensor([[g.x, g.y, g.z] for g in list(s.grid_size)[:L]], dtype=torch.int32, device=dev)
        self.numcells = torch.tensor(list(s.num_cells)[:L], dtype=torch.int32, device=dev)
        self.ncell_idx = torch.zeros(L, dtype=torch.int32, device=dev)
        lib.IndexOffset(_p(self.numcells), _p(self.ncell_idx), L)
        self.cell = _abi.SEARCHCELL(self.numcells.data_ptr(), self.grid.data_ptr(), self.cellsize.data_ptr())

    def no_alloc(self, lib, out, pos, err):
        return lib.BldNeborListNoAlloc(_p(out["hash"]), _p(out["index"]), _p(out["cell_start"]),
                                       _p(out["cell_end"]), _p(self.plevel), self.cell, _p(self.ncell_idx),
                                       _p(self.level_size), _p(self.npars), _p(self.nneb), self.L, _p(pos),
                                       self.ncells, _p(out["nebor"]), _p(self.nidx), _p(out["num_nebor"]), self.n,
                                       _p(self.rad), _p(err))


def _p(x):
    return C.c_void_p(x.data_ptr())


@pytest.mark.gpu
@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_no_alloc_build_matches_bld_nebor_list_twice_in_a_row(make, cuda):
    import torch

    lib = _abi.load()
    _declare(lib)
    w = make()
    s = w.setup.s
    n, S, L, ncells = w.setup.n, int(s.n_pp_slots), int(s.n_levels), int(s.sys_ncells)
    assert _scratch_bytes(n, ncells) <= STATIC_SCRATCH_BYTES
    dev = "cuda"
    k = _harness.consts_of(w.setup)
    lib.setMaterial(C.byref(k.mat))
    lib.setLiquid(C.byref(k.lqd))
    lib.setParameters(C.byref(k.prm))
    lib.setCalpara(C.byref(k.cal), C.byref(k.pwcal))

    rad = torch.tensor(w.setup.rad, device=dev)
    plevel = torch.tensor(w.setup.plevel, device=dev)
    nidx = torch.tensor(w.setup.nidx, device=dev)
    level_size = torch.tensor(list(s.level_size)[:L], dtype=torch.float64, device=dev)
    nneb = torch.tensor(list(s.level_nnebors)[:L], dtype=torch.int32, device=dev)
    npars = torch.tensor(list(s.level_npars)[:L], dtype=torch.int32, device=dev)
    cellsize = torch.tensor(list(s.cell_size)[:L], dtype=torch.float64, device=dev)
    grid = torch.tensor([[g.x, g.y, g.z] for g in list(s.grid_size)[:L]], dtype=torch.int32, device=dev)
    numcells = torch.tensor(list(s.num_cells)[:L], dtype=torch.int32, device=dev)
    ncell_idx = torch.zeros(L, dtype=torch.int32, device=dev)
    p = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    lib.IndexOffset(p(numcells), p(ncell_idx), L)
    cell = _abi.SEARCHCELL(numcells.data_ptr(), grid.data_ptr(), cellsize.data_ptr())

    def outputs():
        return {"hash": torch.full((n,), -7, dtype=torch.int32, device=dev),
                "index": torch.full((n,), -7, dtype=torch.int32, device=dev),
                "cell_start": torch.full((ncells,), -7, dtype=torch.int32, device=dev),
                "cell_end": torch.full((ncells,), -7, dtype=torch.int32, device=dev),
                "nebor": torch.full((S,), -7, dtype=torch.int32, device=dev),
                "num_nebor": torch.full((n,), -7, dtype=torch.int32, device=dev)}

    ref_out, out = outputs(), outputs()
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    lib.dem_compat_errors()  # clears the word an earlier test may have left set

    pos_a, _, _ = _workloads.stirred(w)
    rng = np.random.Generator(np.random.PCG64(11))
    pos_b = pos_a + rng.uniform(-0.15, 0.15, pos_a.shape) * w.setup.rad[:, None]
    previous = None
    for call, host_pos in enumerate((pos_a, pos_b)):
        pos = torch.tensor(host_pos, dtype=torch.float64, device=dev).contiguous()
        for o in (ref_out, out):
            for v in o.values():
                v.fill_(-7)
        lib.BldNeborList(p(ref_out["hash"]), p(ref_out["index"]), p(ref_out["cell_start"]), p(ref_out["cell_end"]),
                         p(plevel), cell, p(ncell_idx), p(level_size), p(npars), p(nneb), L, p(pos), ncells,
                         p(ref_out["nebor"]), p(nidx), p(ref_out["num_nebor"]), n, p(rad))
        st = lib.BldNeborListNoAlloc(p(out["hash"]), p(out["index"]), p(out["cell_start"]), p(out["cell_end"]),
                                     p(plevel), cell, p(ncell_idx), p(level_size), p(npars), p(nneb), L, p(pos),
                                     ncells, p(out["nebor"]), p(nidx), p(out["num_nebor"]), n, p(rad), p(err))
        assert st == _abi.DEM_OK, lib.dem_last_error()
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        assert lib.dem_compat_errors() == 0
        got = {key: v.cpu().numpy() for key, v in out.items()}
        want = {key: v.cpu().numpy() for key, v in ref_out.items()}
        for key in want:
            np.testing.assert_array_equal(got[key], want[key], err_msg=f"call {call + 1}: {key}")
        assert (got["num_nebor"] >= 0).all() and got["num_nebor"].sum() > 0
        if previous is not None:  # the second call saw a different configuration
            assert not np.array_equal(previous, got["nebor"])
        previous = got["nebor"]


@pytest.mark.gpu
def test_no_alloc_build_matches_the_oracle(cuda):
    """the same build straight against the oracle (the reference's calcHashG, stable
    sort, reorderDataAndFindCellStartG and NeighborFindG restated, kernel.cu:617-855)"""
    import torch

    lib = _abi.load()
    _declare(lib)
    w = _workloads.small_wet()
    d = _Dev(w, lib, torch)
    n, S, ncells = d.n, d.S, d.ncells
    pos_h, vel, ang = _workloads.stirred(w)
    out = {k: torch.full((m,), -7, dtype=torch.int32, device="cuda")
           for k, m in (("hash", n), ("index", n), ("cell_start", ncells), ("cell_end", ncells), ("nebor", S),
                        ("num_nebor", n))}
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    pos = torch.tensor(pos_h, dtype=torch.float64, device="cuda").contiguous()
    assert d.no_alloc(lib, out, pos, err) == _abi.DEM_OK, lib.dem_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    sim = _harness.OracleSim(w.setup, pos_h, vel, ang)
    sim.step()  # the first step builds the lists from these positions, then moves them
    got = {k: v.cpu().numpy() for k, v in out.items()}
    np.testing.assert_array_equal(got["hash"], sim.arr("hash", np.int32, n))
    np.testing.assert_array_equal(got["index"], sim.arr("index", np.int32, n))
    np.testing.assert_array_equal(got["cell_start"], sim.arr("cellStart", np.int32, ncells))
    np.testing.assert_array_equal(got["cell_end"], sim.arr("cellEnd", np.int32, ncells))
    num, flat = sim.lists_flat()
    np.testing.assert_array_equal(got["num_nebor"], num)
    _, _, sl = sim.slots_of(num)
    np.testing.assert_array_equal(got["nebor"][sl], flat)
    assert num.sum() > 0
    sim.close()


@pytest.mark.gpu
def test_no_alloc_error_bits_with_guarded_outputs(cuda):
    """A particle of the last size level on the far face of its grid (the
    reference clamps grid coordinates to gridSize, kernel.cu:627-629, and would
    write past CellStart) and a level-0 slot capacity of one: the call succeeds,
    the caller's d_err gets bit 4 and bit 1, every output stays inside its
    buffer (guard words around each are untouched) and holds valid values."""
    import torch

    lib = _abi.load()
    _declare(lib)
    w = _workloads.small_wet()
    s = w.setup.s
    L = int(s.n_levels)
    nneb = list(s.level_nnebors)[:L]
    nneb[0] = 1
    d = _Dev(w, lib, torch, nneb=nneb)
    n, S, ncells = d.n, d.S, d.ncells
    assert (w.setup.plevel == 0).sum() > 10
    pos_h, _, _ = _workloads.stirred(w)
    q = int(np.flatnonzero(w.setup.plevel == L - 1)[0])
    g = s.grid_size[L - 1]
    cs = float(s.cell_size[L - 1])
    o = s.prm.Origin
    pos_h[q] = (o.x + 0.5 * g.x * cs, o.y + 0.5 * g.y * cs, o.z + (g.z + 0.25) * cs)
    G, SENT = 64, -123456789
    bufs, out = {}, {}
    for k, m in (("hash", n), ("index", n), ("cell_start", ncells), ("cell_end", ncells), ("nebor", S),
                 ("num_nebor", n)):
        bufs[k] = torch.full((m + 2 * G,), SENT, dtype=torch.int32, device="cuda")
        out[k] = bufs[k][G:G + m]
        out[k].fill_(-7)
    err_buf = torch.full((2 * G + 1,), SENT, dtype=torch.int32, device="cuda")
    err = err_buf[G:G + 1]
    err.zero_()
    pos = torch.tensor(pos_h, dtype=torch.float64, device="cuda").contiguous()
    for call in range(2):
        st = d.no_alloc(lib, out, pos, err)
        assert st == _abi.DEM_OK, lib.dem_last_error()
        torch.cuda.synchronize()
        assert int(err.item()) & 5 == 5, f"call {call + 1}: error word {int(err.item())}"
        for k, b in bufs.items():
            h = b.cpu().numpy()
            assert (h[:G] == SENT).all() and (h[-G:] == SENT).all(), f"call {call + 1}: guard words of {k}"
        e = err_buf.cpu().numpy()
        assert (e[:G] == SENT).all() and (e[-G:] == SENT).all()
        got = {k: v.cpu().numpy() for k, v in out.items()}
        assert ((got["hash"] >= 0) & (got["hash"] < ncells)).all()
        assert got["hash"][np.argsort(got["index"])[0]] >= 0
        assert np.array_equal(np.sort(got["index"]), np.arange(n))
        assert (np.diff(got["hash"]) >= 0).all()
        caps = np.array(nneb)[w.setup.plevel]
        assert ((got["num_nebor"] >= 0) & (got["num_nebor"] <= caps)).all()
        assert (got["num_nebor"][w.setup.plevel == 0] == 1).any()
    err.zero_()
