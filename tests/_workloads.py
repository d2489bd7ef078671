"""Small seeded states for parity tests: a workload's start positions, compressed
slightly so neighbours overlap from the first step (elastic and plastic
contacts), plus random velocities and spins so lists are rebuilt and histories
carried within a few hundred steps."""
from __future__ import annotations

import numpy as np

from gpucode_gb300 import configs


def stirred(w: configs.Workload, seed: int = 7, squeeze: float = 0.985, vscale: float = 0.6,
            wscale: float = 2.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    pos = w.pos0_reduced.copy()
    bw = w.setup.s.cyl.Bw
    rad = w.setup.rad
    pos[:, 2] = bw + rad + (pos[:, 2] - bw - rad) * squeeze
    rng = np.random.Generator(np.random.PCG64(seed))
    vel = vscale * rng.standard_normal((w.setup.n, 3))
    ang = wscale * rng.standard_normal((w.setup.n, 3))
    return pos, vel, ang


def small_dry(n: int = 300, seed: int = 3) -> configs.Workload:
    """A dense dry bed (deposited, monodisperse) in a narrow cylinder."""
    d = 1e-3
    dia = np.full(n, d)
    R = 3e-3
    pos = configs.deposit(dia, R, 0.0, 0.0, 4, seed)
    yldp = configs.yldp_for_yield_overlap(0.01, configs.E_YOUNG, configs.NU)
    top = float(pos[:, 2].max()) + 4 * d
    inp = configs.make_input(n, 1, d, 0.1, R, top, configs.RHO, configs.E_YOUNG, configs.NU, configs.MU, 6.6e-6,
                             yldp, 0, dt=1e-6, rfrc=0.02)
    return configs.Workload(f"pin_dry{n}", inp, dia, pos, configs.Setup.build(inp, dia), 0)


def small_wet(n: int = 400, seed: int = 4, n_levels: int = 3) -> configs.Workload:
    """A dense wet polydisperse bed with several size levels."""
    dia = configs.lognormal_diameters(n, 1e-3, 0.3, 0.5e-3, 2.0e-3, seed)
    R = 4e-3
    pos = configs.deposit(dia, R, 0.0, 0.0, 4, seed)
    real = 2e-3
    yldp = configs.yldp_for_yield_overlap(0.01, configs.E_YOUNG, configs.NU)
    top = float((pos[:, 2] + dia / 2).max()) + 4 * real
    cut = (1e-4 / real) * dia.max() / dia.min()
    inp = configs.make_input(n, n_levels, real, cut, R, top, configs.RHO, configs.E_YOUNG, configs.NU, configs.MU,
                             6.6e-6, yldp, 1, liquid=(0.072, 0.075, 5e-6), dt=5e-7, rfrc=0.02)
    return configs.Workload(f"pin_wet{n}", inp, dia, pos, configs.Setup.build(inp, dia), 0)
