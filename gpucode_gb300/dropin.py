"""The reference driver's step loop (main.cpp:433-568) over this library's
drop-in entry points: device buffers in the reference's layouts (torch
tensors), the calls in main.cpp's order with its per-step read of the move
flag, the history copies around a rebuild and the VarInit memsets.

This is what a user of the reference gets by linking its unchanged main.cpp
against libdem_gb300 (the FP64 kernels behind heydem.h's API).  The tests
drive it step by step against the oracle; the bench times it beside the
reference's own kernels on the same bed."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi


def declare(lib) -> None:
    """argument types of the drop-in entry points (heydem.h:366-613)"""
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
    lib.setMaterial.argtypes = [P]
    lib.setLiquid.argtypes = [P]
    lib.setParameters.argtypes = [P]
    lib.setCalpara.argtypes = [P, P]


class DropInDriver:
    """Device buffers in the reference's layouts and the main.cpp step loop."""

    def __init__(self, w, pos, vel, ang, torch):
        self.t = torch
        self.lib = _abi.load()
        declare(self.lib)
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
        # the model's constants (main.cpp:328-348 derives them; the set-up holds them)
        self.lib.setMaterial(C.cast(C.pointer(s.mat), C.c_void_p))
        self.lib.setLiquid(C.cast(C.pointer(s.lqd), C.c_void_p))
        self.lib.setParameters(C.cast(C.pointer(s.prm), C.c_void_p))
        self.lib.setCalpara(C.cast(C.pointer(s.cal), C.c_void_p), C.cast(C.pointer(s.pwcal), C.c_void_p))
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

    @staticmethod
    def p(x):
        return C.c_void_p(x.data_ptr())

    def step(self) -> bool:
        """one time step in main.cpp's order; True when it rebuilt the lists"""
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
