"""The learned capillary closure (dem_capnet_* of libdem_gb300).

A 4 -> 64 -> 64 -> 2 SiLU network standing in for the reference's capillary
routine (kernel.cu:65-81) and rupture distance (kernel.cu:518).  Samples come
from a running wet bed (`collect_samples`), training runs on the GPU with the
library's own forward/backward/Adam kernels (`CapNet.fit`), and the engine
evaluates the trained network on the tensor cores inside its step kernel
(`Engine(..., capillary="mlp")` + `Engine.set_capnet`).

Device buffers are torch CUDA tensors (plumbing only); every computation is
in the library."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import CapnetFitOpts, CapnetReport, check

N_PARAMS = 4610
N_NORM = 20
FEATURES = ("separation", "volume", "contact_angle", "radius_ratio")
TARGETS = ("force_normalised", "rupture_distance")


def _dev(t) -> C.c_void_p:
    import torch

    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
        raise TypeError("expected a contiguous float32 CUDA tensor")
    return C.c_void_p(t.data_ptr())


class CapNet:
    """One network (dem_capnet)."""

    def __init__(self, seed: int = 0):
        self.lib = _abi.load()
        h = C.c_void_p()
        check(self.lib.dem_capnet_create(int(seed), C.byref(h)), "dem_capnet_create")
        self.h = h

    def close(self) -> None:
        if self.h:
            self.lib.dem_capnet_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- parameters ----
    def get(self) -> tuple[np.ndarray, np.ndarray]:
        p = np.zeros(N_PARAMS, np.float32)
        nz = np.zeros(N_NORM, np.float32)
        check(self.lib.dem_capnet_get(self.h, _abi.ptr(p), _abi.ptr(nz)), "dem_capnet_get")
        return p, nz

    def set(self, params: np.ndarray | None = None, norm: np.ndarray | None = None) -> None:
        p = None if params is None else np.ascontiguousarray(params, np.float32).reshape(N_PARAMS)
        nz = None if norm is None else np.ascontiguousarray(norm, np.float32).reshape(N_NORM)
        check(self.lib.dem_capnet_set(self.h, None if p is None else _abi.ptr(p), None if nz is None else _abi.ptr(nz)),
              "dem_capnet_set")

    def save(self, path: str | os.PathLike) -> None:
        p, nz = self.get()
        np.savez(path, params=p, norm=nz)

    def load(self, path: str | os.PathLike) -> None:
        d = np.load(path)
        self.set(d["params"], d["norm"])

    # ---- training ----
    def fit(self, x, y, epochs: int = 20, batch: int = 8192, lr: float = 1e-3, val_frac: float = 0.1,
            seed: int = 0) -> dict:
        opt = CapnetFitOpts(epochs=epochs, batch=batch, lr=lr, val_frac=val_frac, seed=seed)
        rep = CapnetReport()
        check(self.lib.dem_capnet_fit(self.h, _dev(x), _dev(y), int(x.shape[0]), C.byref(opt), C.byref(rep)),
              "dem_capnet_fit")
        out = {k: getattr(rep, k) for k, _ in CapnetReport._fields_ if k not in ("pad", "train_mse")}
        out["train_mse"] = list(rep.train_mse)[: min(rep.epochs, 64)]
        return out

    def grad(self, x, y) -> tuple[np.ndarray, float]:
        g = np.zeros(N_PARAMS, np.float32)
        loss = C.c_float()
        check(self.lib.dem_capnet_grad(self.h, _dev(x), _dev(y), int(x.shape[0]), _abi.ptr(g), C.byref(loss)),
              "dem_capnet_grad")
        return g, float(loss.value)

    def infer(self, x, tensor_cores: bool | str = True):
        """raw features -> raw outputs: tensor_cores True (or "warp") the BF16
        warp tiles the fused step kernel runs, "tcgen05" 128-row tiles on the
        5th-generation tensor cores, False the FP32 network"""
        import torch

        mode = {True: 1, "warp": 1, "tcgen05": 2, False: 0}[tensor_cores]
        y = torch.empty((x.shape[0], 2), dtype=torch.float32, device=x.device)
        check(self.lib.dem_capnet_infer(self.h, _dev(x), int(x.shape[0]), mode, _dev(y)), "dem_capnet_infer")
        return y


def formula(x, fp64: bool = True, angle: bool = False):
    """the plain closure on raw features (FP64 as the reference evaluates it, or
    the step kernel's FP32 form; angle: the per-contact liquid model's
    regression with the contact angle of feature 2), as a float32 CUDA tensor [n][2]"""
    import torch

    y = torch.empty((x.shape[0], 2), dtype=torch.float32, device=x.device)
    lib = _abi.load()
    mode = (1 if fp64 else 0) | (2 if angle else 0)
    check(lib.dem_capnet_formula(_dev(x), int(x.shape[0]), mode, _dev(y)), "dem_capnet_formula")
    return y


def collect_samples(engine, capacity: int):
    """(x[n][4], y[n][2]) float32 CUDA tensors: every bridged pair of the
    engine's current state with the plain formula's outputs."""
    import torch

    x = torch.empty((capacity, 4), dtype=torch.float32, device="cuda")
    y = torch.empty((capacity, 2), dtype=torch.float32, device="cuda")
    n = C.c_longlong()
    check(engine.lib.dem_capnet_samples(engine.h, _dev(x), _dev(y), int(capacity), C.byref(n)), "dem_capnet_samples")
    return x[: n.value], y[: n.value]
