"""The network oracle (oracle/mlp_oracle.py) on the CPU: its analytic gradient
against central finite differences, its BF16 rounding, its formula against
the FP64 C oracle's capillary routine (a restatement of kernel.cu:65-81)."""
import ctypes as C
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import mlp_oracle as mo  # noqa: E402

import _harness  # noqa: E402


def _batch(rng, n):
    x = np.column_stack([np.exp(rng.uniform(np.log(5e-6), np.log(0.05), n)),
                         np.exp(rng.uniform(np.log(1e-4), np.log(0.05), n)),
                         rng.uniform(0, 0.52, n), rng.uniform(0.25, 1.0, n)])
    y = mo.formula(x)
    norm = np.zeros(20)
    f = np.column_stack([np.log(x[:, 0]), np.log(x[:, 1]), x[:, 2], x[:, 3]])
    norm[0:4], norm[4:8] = f.mean(0), f.std(0)
    norm[8:10], norm[10:12] = y.mean(0), y.std(0)
    return x, y, norm


def test_analytic_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    x, y, norm = _batch(rng, 64)
    p = mo.init_params(1)
    loss, g = mo.loss_and_grad(p, x, y, norm)
    assert abs(loss - mo.loss_only(p, x, y, norm)) < 1e-12
    idx = np.concatenate([rng.choice(256, 8, replace=False), 256 + rng.choice(64, 4, replace=False),
                          320 + rng.choice(4096, 16, replace=False), 4416 + rng.choice(64, 4, replace=False),
                          4480 + rng.choice(128, 8, replace=False), [4608, 4609]])
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        fd = (mo.loss_only(p + e, x, y, norm) - mo.loss_only(p - e, x, y, norm)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.01171875, 1.001953125, 1.005859375, -3.14159], np.float32)
    r = mo.bf16(v)
    # 8 significant bits: steps of 1/128 above 1; ties go to the even significand
    assert list(r[:5]) == [1.0, 1.0, 1.015625, 1.0, 1.0078125]
    assert r[5] == np.float32(-3.140625)
    assert (r.view(np.uint32) & 0xFFFF).max() == 0


def test_formula_matches_the_c_oracle():
    lib = _harness.oracle()
    k = _harness.OConsts()
    k.lqd.stension = 0.7
    k.lqd.gapmn = 5e-6
    rng = np.random.default_rng(2)
    x, y, _ = _batch(rng, 50)
    for i in range(50):
        effR = 0.4
        f = lib.orc_fcap(x[i, 0], x[i, 1], effR, C.c_void_p(C.addressof(k)))
        want = f / (2 * mo.PI_REF * effR * 0.7)
        assert abs(y[i, 0] - want) <= 1e-12 * abs(want), (i, y[i, 0], want)
