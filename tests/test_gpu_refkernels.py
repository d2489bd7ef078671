"""The reference's own kernels (kernel.cu compiled for sm_103a, run by
baseline/refgpu.cu in main.cpp:433-568's order) against this library's
drop-in entry points on the same GPU and the same seeded state.

Both sides evaluate the reference's FP64 formulas; the reference build lets
nvcc contract multiply-adds into FMAs and this library does not, so positions
agree to rounding level after one step and drift apart slowly (chaotically)
after that."""
import numpy as np
import pytest

import _workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("make", [_workloads.small_dry, _workloads.small_wet])
def test_reference_gpu_kernels_agree_with_the_drop_in_path(make, cuda):
    import torch

    from baseline import refgpu
    from test_gpu_compat import RefDriver, _declare

    ok, why = refgpu.available()
    if not ok:
        pytest.skip(why)
    w = make()
    pos, vel, ang = _workloads.stirred(w)
    scale = float(np.abs(pos).max())
    for steps, tol in ((1, 1e-13), (4, 1e-8)):
        stats, ref_pos = refgpu.run(w.setup, pos, vel, ang, 0, steps)
        assert stats["overflow"] == 0
        drv = RefDriver(w, pos, vel, ang, torch)
        _declare(drv.lib)
        for _ in range(steps):
            drv.step()
        ours = drv.pos.cpu().numpy()
        err = np.abs(ours - ref_pos).max() / scale
        assert err < tol, (steps, err)
        # the state moved: the comparison is not of two copies of the input
        assert np.abs(ours - pos).max() / scale > 100 * tol
