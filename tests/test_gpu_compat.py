"""The reference-compatible entry points (heydem.h:366-613) on the GPU, driven in
main.cpp:433-568's order on the reference's own layouts, against the oracle in
lockstep (tests/_lockstep.py).

Integer outputs (sorted hashes and indices, CellStart/CellEnd, neighbour slots,
wall lists, load stages, bridge flags) must be bit-exact.  Floating-point
outputs are FP64 with the reference's formulas on both sides: 1e-12 relative
per step (last-ulp differences of CUDA's and glibc's pow/log/exp), except at
contacts whose spring sits exactly on its slip limit, where those differences
legitimately select the other friction branch."""
import ctypes as C

import numpy as np
import pytest

import _harness
import _lockstep
import _workloads
from gpucode_gb300 import _abi

pytestmark = pytest.mark.gpu


class RefDriver:
    """Device buffers in the reference's layouts and the main.cpp step loop."""

    def __init__(self, w, pos, vel, ang, torch):
        self.t = torch
        self.lib = _abi.load()
        s = w.setup.s
        self.s, self.n, self.S, self.C, self.L = s, w.setup.n, int(s.n_pp_slots), int(s.sys_ncells), s.n_levels
        dev = "cuda"
        z = lambda *shape, dt=torch.float64: torch.zeros(*shape, dtype=dt, device=dev)  # noqa: E731
        zi = lambda *shape: torch.zeros(*shape, dtype=torch.int32, device=dev)  # noqa: E731
        n, S, L = self.n, self.S, self.L
        self.pos = torch.tensor(pos, dtype=torch.float64, device=dev).contiguous()
        self.vel = torch.tensor(vel, dtype=torch.float64, device=dev).contiguous()
        self.ang = torch.tensor(ang, dtype=torch.float64, device=dev).contiguous()
        self.force, self.mom, self.rmom = z(n, 3), z(n, 3), z(n)
        self.rad = torch.tensor(w.setup.rad, device=dev)
        self.plevel = torch.tensor(w.setup.plevel, device=dev)
        self.nidx = torch.tensor(w.setup.nidx, device=dev)
        self.level_size = torch.tensor(list(s.level_size)[:L], dtype=torch.float64, device=dev)
        self.nneb = torch.tensor(list(s.level_nnebors)[:L], dtype=torch.int32, device=dev)
        self.npars = torch.tensor(list(s.level_npars)[:L], dtype=torch.int32, device=dev)
        self.cellsize = torch.tensor(list(s.cell_size)[:L], dtype=torch.float64, device=dev)
        self.grid = torch.tensor([[g.x, g.y, g.z] for g in list(s.grid_size)[:L]], dtype=torch.int32, device=dev)
        self.numcells = torch.tensor(list(s.num_cells)[:L], dtype=torch.int32, device=dev)
        self.ncell_idx = zi(L)
        self.lib.IndexOffset(C.c_void_p(self.numcells.data_ptr()), C.c_void_p(self.ncell_idx.data_ptr()), L)
        cyl = np.frombuffer(bytes(s.cyl), np.float64).copy()
        self.cyl = torch.tensor(cyl, device=dev)
        self.hash, self.index = zi(n), zi(n)
        self.cs, self.ce = zi(self.C), zi(self.C)
        self.neb, self.neb_old, self.num, self.num_old = zi(S), zi(S), zi(n), zi(n)
        self.wl, self.wl_old, self.nw, self.nw_old = zi(n, 3), zi(n, 3), zi(n), zi(n)
        self.lqd, self.lqd_old = zi(n), zi(n)
        self.pmove = z(n)
        self.flag = zi(1)
        self.pp = [self._hist(S) for _ in range(2)]
        self.pw = [self._hist(3 * n) for _ in range(2)]
        self.cell = _abi.SEARCHCELL(self.numcells.data_ptr(), self.grid.data_ptr(), self.cellsize.data_ptr())
        k = _harness.consts_of(w.setup)
        self.lib.setMaterial(C.byref(k.mat))
        self.lib.setLiquid(C.byref(k.lqd))
        self.lib.setParameters(C.byref(k.prm))
        self.lib.setCalpara(C.byref(k.cal), C.byref(k.pwcal))
        self.iter = 0
        self.rebuild_pending = True

    def _hist(self, m):
        t = self.t
        h = {"dispt": t.zeros(m, 3, dtype=t.float64, device="cuda")}
        for f in ("nDsp", "nDsp_mx", "plstRad", "plstDfm"):
            h[f] = t.zeros(m, dtype=t.float64, device="cuda")
        for f in ("stage", "lqdBrg"):
            h[f] = t.zeros(m, dtype=t.int32, device="cuda")
        return h

    @staticmethod
    def _pp(h):
        r = _abi.PPCONTACT_HISTORY()
        for f, v in h.items():
            setattr(r, f, v.data_ptr())
        return r

    @staticmethod
    def _pw(h):
        r = _abi.PWCONTACT_HISTORY()
        for f, v in h.items():
            setattr(r, f, v.data_ptr())
        return r

    def p(self, x):
        return C.c_void_p(x.data_ptr())

    def step(self):
        lib, p, s = self.lib, self.p, self.s
        n = self.n
        flag = int(self.flag.item())  # main.cpp:470
        rebuilt = False
        if flag > 0 or self.rebuild_pending:
            if self.iter != 0:
                self.num_old.copy_(self.num)
                self.neb_old.copy_(self.neb)
                lib.PPCntHstryCopy(self._pp(self.pp[1]), self._pp(self.pp[0]), self.S)
                self.nw_old.copy_(self.nw)
                self.wl_old.copy_(self.wl)
                lib.WallCntHstryCopy(self._pw(self.pw[1]), self._pw(self.pw[0]), 3 * n)
            self.pmove.zero_()
            lib.BldNeborList(p(self.hash), p(self.index), p(self.cs), p(self.ce), p(self.plevel), self.cell,
                             p(self.ncell_idx), p(self.level_size), p(self.npars), p(self.nneb), self.L, p(self.pos),
                             self.C, p(self.neb), p(self.nidx), p(self.num), n, p(self.rad))
            lib.BldCirWall(p(self.pos), p(self.rad), p(self.cyl), p(self.wl), C.c_size_t(12), p(self.nw), n)
            if self.iter != 0:
                lib.HstryCopy(p(self.neb), p(self.neb_old), p(self.plevel), p(self.nneb), p(self.npars), p(self.nidx),
                              self._pp(self.pp[1]), self._pp(self.pp[0]), p(self.num), p(self.num_old), n, n)
                lib.HstryCopyPW(p(self.wl), p(self.wl_old), C.c_size_t(12), C.c_size_t(12), self._pw(self.pw[1]),
                                self._pw(self.pw[0]), p(self.nw), p(self.nw_old), n, n)
            self.rebuild_pending = False
            rebuilt = True
        ptrs = [C.c_void_p(x.data_ptr()) for x in (self.force, self.mom, self.rmom, self.lqd, self.lqd_old)]
        lib.VarInit(*[C.byref(q) for q in ptrs], n)
        lib.PpInterCalc(p(self.pos), p(self.vel), p(self.ang), p(self.rad), p(self.neb), p(self.plevel), p(self.nneb),
                        p(self.npars), p(self.nidx), self._pp(self.pp[0]), p(self.num), p(self.lqd), p(self.lqd_old),
                        p(self.force), p(self.mom), p(self.rmom), n, n, int(s.force_cap), int(s.load_stage))
        lib.CirPWCalc(p(self.pos), p(self.vel), p(self.ang), p(self.force), p(self.mom), p(self.rmom), p(self.rad),
                      p(self.cyl), self._pw(self.pw[0]), p(self.nw), p(self.wl), C.c_size_t(12), n, n,
                      int(s.load_stage))
        self.flag.zero_()
        lib.UpdateSystem(p(self.rad), p(self.pos), p(self.vel), p(self.ang), p(self.force), p(self.mom),
                         p(self.rmom), p(self.flag), p(self.pmove), n)
        self.iter += 1
        return rebuilt


def _declare(lib):
    P = C.c_void_p
    lib.BldNeborList.argtypes = [P, P, P, P, P, _abi.SEARCHCELL, P, P, P, P, C.c_int, P, C.c_int, P, P, P, C.c_int, P]
    lib.PpInterCalc.argtypes = [P] * 9 + [_abi.PPCONTACT_HISTORY] + [P] * 6 + [C.c_int] * 4
    lib.CirPWCalc.argtypes = [P] * 8 + [_abi.PWCONTACT_HISTORY, P, P, C.c_size_t] + [C.c_int] * 3
    lib.HstryCopy.argtypes = [P] * 6 + [_abi.PPCONTACT_HISTORY] * 2 + [P, P, C.c_int, C.c_int]
    lib.HstryCopyPW.argtypes = [P, P, C.c_size_t, C.c_size_t] + [_abi.PWCONTACT_HISTORY] * 2 + [P, P, C.c_int,
                                                                                                C.c_int]
    lib.PPCntHstryCopy.argtypes = [_abi.PPCONTACT_HISTORY] * 2 + [C.c_int]
    lib.WallCntHstryCopy.argtypes = [_abi.PWCONTACT_HISTORY] * 2 + [C.c_int]
    lib.UpdateSystem.argtypes = [P] * 9 + [C.c_int]
    lib.BldCirWall.argtypes = [P, P, P, P, C.c_size_t, P, C.c_int]
    lib.VarInit.argtypes = [C.POINTER(P)] * 5 + [C.c_int]
    lib.IndexOffset.argtypes = [P, P, C.c_int]


FP64_TOL = {"force": 1e-12, "pos": 1e-14, "vel": 1e-12, "hist": 1e-12}


def _snap(drv, sim, w):
    """the driver's device state (reference layouts) in the lockstep comparison's
    terms: lists and contact records as the used slots end to end"""
    g = lambda x: x.detach().cpu().numpy()  # noqa: E731
    n = drv.n
    num = g(drv.num)
    _, _, sl = sim.slots_of(num)
    pp = {k: g(v) for k, v in drv.pp[0].items()}
    rec = np.zeros((len(sl), 8))
    rec[:, 0:3] = pp["dispt"][sl]
    for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
        rec[:, 3 + c] = pp[f][sl]
    rec[:, 7] = pp["stage"][sl]
    pw = {k: g(v) for k, v in drv.pw[0].items()}
    wrec = np.zeros((n, 3, 8))
    for a in range(3):
        rows = a * n + np.arange(n)
        wrec[:, a, 0:3] = pw["dispt"][rows]
        for c, f in enumerate(("nDsp", "nDsp_mx", "plstRad", "plstDfm")):
            wrec[:, a, 3 + c] = pw[f][rows]
        wrec[:, a, 7] = pw["stage"][rows]
    return dict(pos=g(drv.pos), vel=g(drv.vel), angvel=g(drv.ang), force=g(drv.force), pmove=g(drv.pmove),
                lqd=g(drv.lqd), counts=num, partners=g(drv.neb)[sl], rec=rec, brg=pp["lqdBrg"][sl],
                nwall=g(drv.nw), wlist=g(drv.wl), wrec=wrec, flag=int(drv.flag.item()))


def _load_oracle_from(drv, sim):
    """the oracle resumes from the driver's device state (same layouts)"""
    n, S = drv.n, drv.S
    g = lambda x: x.detach().cpu().numpy()  # noqa: E731
    sim.vec("pos")[:] = g(drv.pos)
    sim.vec("vel")[:] = g(drv.vel)
    sim.vec("angvel")[:] = g(drv.ang)
    sim.arr("pMove", np.float64, n)[:] = g(drv.pmove)
    sim.arr("lqdCnt", np.int32, n)[:] = g(drv.lqd)
    sim.arr("Num_Nebor", np.int32, n)[:] = g(drv.num)
    sim.arr("Nebor1", np.int32, S)[:] = g(drv.neb)
    for tag, h, m in (("pp", drv.pp[0], S), ("pw", drv.pw[0], 3 * n)):
        sim.arr(tag + ".dispt", np.float64, 3 * m)[:] = g(h["dispt"]).reshape(-1)
        for f in ("nDsp", "nDsp_mx", "plstRad", "plstDfm"):
            sim.arr(f"{tag}.{f}", np.float64, m)[:] = g(h[f])
        for f in ("stage", "lqdBrg"):
            sim.arr(f"{tag}.{f}", np.int32, m)[:] = g(h[f])
    sim.arr("nwall", np.int32, n)[:] = g(drv.nw)
    sim.arr("wlist", np.int32, 3 * n)[:] = g(drv.wl).reshape(-1)
    sim.lib.orc_sim_set_counter(sim.h, b"flag", int(drv.flag.item()))
    sim.lib.orc_sim_set_counter(sim.h, b"iter", drv.iter)
    sim.lib.orc_sim_set_counter(sim.h, b"need_build", 1 if drv.rebuild_pending else 0)


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_compat_step_loop_matches_oracle(cuda, make):
    """main.cpp's loop through the C ABI, in lockstep with the oracle: each step
    starts both from the driver's state; sorted order, cell ranges, neighbour
    slots, wall lists, stages and bridge flags bit-exact after every step;
    forces, state and histories to 1e-12 relative."""
    import torch

    w = make()
    _declare(_abi.load())
    pos, vel, ang = _workloads.stirred(w)
    drv = RefDriver(w, pos, vel, ang, torch)
    sim = _harness.OracleSim(w.setup, pos, vel, ang)
    n = w.setup.n
    g = lambda x: x.detach().cpu().numpy()  # noqa: E731
    rebuilds = 0
    for t in range(250):
        torch.cuda.synchronize()
        _load_oracle_from(drv, sim)
        rb = sim.step()
        ra = drv.step()
        torch.cuda.synchronize()
        assert ra == bool(rb), f"rebuild decision differs at step {t}"
        rebuilds += rb
        if rb:
            assert np.array_equal(g(drv.hash), sim.arr("hash", np.int32, n)), t
            assert np.array_equal(g(drv.index), sim.arr("index", np.int32, n)), t
            assert np.array_equal(g(drv.cs), sim.arr("cellStart", np.int32, drv.C)), t
            assert np.array_equal(g(drv.ce), sim.arr("cellEnd", np.int32, drv.C)), t
        _lockstep.compare_step(_snap(drv, sim, w), sim, w, FP64_TOL, f"step {t}")
    assert rebuilds >= 2
    assert _abi.load().dem_compat_errors() == 0


def test_first_step_forces_match_oracle_tightly(cuda):
    """One step from the same state: no chaotic growth, so FP64 forces agree to 1e-12."""
    import torch

    w = _workloads.small_wet()
    _declare(_abi.load())
    pos, vel, ang = _workloads.stirred(w)
    drv = RefDriver(w, pos, vel, ang, torch)
    sim = _harness.OracleSim(w.setup, pos, vel, ang)
    drv.step()
    sim.step()
    torch.cuda.synchronize()
    st = sim.state()
    scale = np.abs(st["force"]).max()
    np.testing.assert_allclose(drv.force.cpu().numpy(), st["force"], rtol=1e-12, atol=1e-14 * scale)
    np.testing.assert_allclose(drv.mom.cpu().numpy(), st["mom"], rtol=1e-12, atol=1e-14 * np.abs(st["mom"]).max())
    np.testing.assert_allclose(drv.pos.cpu().numpy(), st["pos"], rtol=1e-15, atol=1e-15)
    assert np.array_equal(drv.lqd.cpu().numpy(), sim.arr("lqdCnt", np.int32, w.setup.n))
