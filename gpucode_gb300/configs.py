"""Synthetic inputs for the benchmark workloads and the tests.

No sample heyi.in ships with the reference, so these generators build the
inputs the reference reads (keyword-file fields + a diameter list + initial
positions) for the packing workloads:

  dry5k   -- 5,000 monodisperse 1 mm spheres, cylinder R = 8 mm, hexagonal
             lattice from z = 2 mm with seeded +-0.05 mm jitter, dt = 1e-6 s,
             skin 0.1 d, no liquid.
  wet200k -- 200,000 log-normal spheres (median 1 mm, sigma_ln 0.2, resampled
             into [0.5, 2] mm), cylinder R = 25 mm, capillary bridges on,
             dt = 5e-7 s, four size levels.  Start: a seeded sequential
             deposition (each sphere dropped at the lowest of 8 random spots
             onto the floor or the spheres below, touching, no overlaps), i.e.
             a loose bed raining into the cylinder; the 25 ms the workload
             simulates is too short for a dilute lattice to pack.

Parameter mapping onto the reference's knobs (it has no restitution or yield
overlap inputs):
  yield overlap 1% of d at R* = d/4  -> ydsp_t = 0.04 -> yldp = 0.8 E*/pi with
      E* = cal.emod = E/(2(1-nu^2))  (main.cpp:330-336, kernel.cu:120);
  restitution e                      -> dmpn from a two-sphere head-on impact of
      the reference's normal law (Hertz + plastic + unload + damping) at the
      fill's impact speed, by bisection (calibrate_dmpn); the same impact
      stepped by the FP64 oracle at the dry workload's 1 us step parts at
      0.6975 of the impact speed for e = 0.7;
  skin s                             -> CUTGAPFORNEIGHBORLIST = (s/REALSIZE)*Rmax/Rmin
      (ReadData.cpp:363 scales it back);
  bridge volume U[0.5%, 2%] of the smaller sphere -> LIQUID vol = 6 x 1.25%:
      the reference splits one liquid fraction per particle over
      max(12, bridges) (kernel.cu:429-434), which for equal spheres gives
      vol/6 of a sphere per bridge; per-contact volumes and contact angles
      are not representable in its formula (fixed theta = 0 regression);
  gravity: the reference constant 9.8 (heydem.h:16) unless gravity is given.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import DemInput
from .engine import Setup


@dataclass
class Workload:
    name: str
    inp: DemInput
    dia: np.ndarray  # SI diameters
    pos0: np.ndarray  # SI initial positions (N, 3)
    setup: Setup
    steps: int
    pos_reduced: np.ndarray | None = None  # the start in reduced units, when it was stored that way

    @property
    def pos0_reduced(self) -> np.ndarray:
        if self.pos_reduced is not None:
            return self.pos_reduced
        return self.setup.to_reduced(self.pos0)


def load_bed(path, steps: int = 0) -> Workload:
    """A bed stored by tests/golden/make_packed_bed.py: the dem_setup struct's
    bytes, the per-particle radius, size level and level rank, and the start
    positions in reduced units.  Reads the file only: nothing here loads
    libdem_gb300, so the oracle can be run on the bed without the library."""
    import json

    f = np.load(path)
    s = _abi.DemSetup()
    raw = f["setup"].tobytes()
    if len(raw) != C.sizeof(s) or int(f["setup_size"]) != C.sizeof(s):
        raise ValueError(f"{path}: dem_setup of {len(raw)} bytes, this build's is {C.sizeof(s)}")
    C.memmove(C.addressof(s), raw, len(raw))
    setup = Setup(s, np.ascontiguousarray(f["rad"], np.float64), np.ascontiguousarray(f["plevel"], np.int32),
                  np.ascontiguousarray(f["nidx"], np.int32))
    pos = np.ascontiguousarray(f["pos"], np.float64)
    rl = s.unit.rlunit
    recipe = json.loads(str(f["recipe"])) if "recipe" in f else {}
    return Workload(f"bed{setup.n}", None, 2.0 * setup.rad * rl, pos * rl, setup, steps or recipe.get("steps", 0),
                    pos_reduced=pos)


PI_REF = 3.1415926  # the reference's PI (heydem.h:15), used by its constant derivations


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def normal_law_restitution(dmpn: float, v0: float, d: float, rho: float, E: float, nu: float, yldp: float,
                           steps: int = 20000) -> float:
    """Coefficient of restitution of a head-on impact of two equal spheres under
    the reference's normal contact law (kernel.cu:104-165), SI units."""
    m = rho * math.pi * d ** 3 / 6.0
    ms = m / 2.0
    Rs = d / 4.0
    e0 = E / (1 - nu * nu)
    emod = e0 * e0 / (e0 + e0)
    ystress = yldp * yldp / (yldp + yldp)
    ydsp = (math.pi * ystress / (2.0 * emod)) ** 2
    yforce = 4.0 / 3.0 * emod * ydsp ** 1.5
    ystiff = math.pi * ystress
    # contact time scale
    k = 4.0 / 3.0 * emod * math.sqrt(Rs)
    dmax = (15.0 / 16.0 * ms * v0 * v0 / k) ** 0.4
    tc = 3.0 * dmax / v0
    dt = tc / steps
    delta, v = 0.0, v0  # overlap and its rate (closing speed > 0)
    plst_rad, plst_dfm, nmax, nprev = Rs, 0.0, 0.0, 0.0
    for _ in range(steps * 4):
        if delta < plst_dfm or delta <= 0.0:
            fn = 0.0
            if v < 0.0 and delta <= plst_dfm:
                return -v / v0
        elif delta >= nmax:  # loading
            if delta <= ydsp * Rs:
                fn = k * delta ** 1.5
                plst_rad, plst_dfm = Rs, 0.0
            else:
                fn = yforce * Rs * Rs + ystiff * Rs * (delta - ydsp * Rs)
                plst_rad = Rs * (k * delta ** 1.5) / fn
                plst_dfm = delta - (fn / (4.0 / 3.0 * emod * math.sqrt(Rs))) ** (2.0 / 3.0)
            nmax = delta
        else:  # unload / reload
            fn = 4.0 / 3.0 * emod * math.sqrt(plst_rad) * (delta - plst_dfm) ** 1.5
        fd = 2.0 * dmpn * emod * math.sqrt(Rs * max(delta, 0.0)) * v if delta > 0 else 0.0
        a = -(fn + fd) / ms
        v += a * dt
        delta += v * dt
        nprev = delta
    return max(0.0, -v / v0)


def calibrate_dmpn(e_target: float, v0: float, d: float, rho: float, E: float, nu: float, yldp: float) -> float:
    """dmpn [s] giving restitution e_target (0 if plasticity alone dissipates enough)."""
    if normal_law_restitution(0.0, v0, d, rho, E, nu, yldp) <= e_target:
        return 0.0
    lo, hi = 0.0, 1e-3
    while normal_law_restitution(hi, v0, d, rho, E, nu, yldp) > e_target:
        hi *= 2.0
    for _ in range(40):
        mid = 0.5 * (lo + hi)
        if normal_law_restitution(mid, v0, d, rho, E, nu, yldp) > e_target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def yldp_for_yield_overlap(frac: float, E: float, nu: float) -> float:
    """yldp giving a yield overlap of frac*d at R* = d/4 (ydsp_t = 4 frac)."""
    e0 = E / (1 - nu * nu)
    emod = e0 / 2.0
    ydsp = 4.0 * frac
    ystress = math.sqrt(ydsp) * 2.0 * emod / PI_REF
    return 2.0 * ystress


def make_input(np_: int, n_levels: int, real_size: float, cut_gap: float, cyl_r: float, cyl_h: float,
               rho: float, E: float, nu: float, mu: float, dmpn: float, yldp: float, force_cap: int,
               liquid=(0.0, 0.0, 0.0), dt: float = 0.0, expand: float = 2.0, rfrc: float = 0.0,
               gravity: float = 0.0, t_packing: float = 1.0, n_out: int = 1) -> DemInput:
    inp = DemInput()
    inp.np = np_
    inp.n_levels = n_levels
    inp.load_stage = 1
    inp.t_packing = t_packing
    inp.force_cap = force_cap
    inp.real_size = real_size
    inp.cut_gap = cut_gap
    inp.expand_size = expand
    inp.cyl_x = inp.cyl_y = inp.cyl_bw = 0.0
    inp.cyl_r = cyl_r
    inp.cyl_h = cyl_h
    inp.feed_lmin = 0.5 * cyl_h
    inp.feed_lmax = 0.9 * cyl_h
    for m in range(2):
        # density ymod pois sfrc rfrc dmpn yldp; the wall uses the particle material
        vals = [rho, E, nu, mu, rfrc, dmpn, yldp]
        for q in range(7):
            inp.mat[m][q] = vals[q]
    inp.lqd[0], inp.lqd[1], inp.lqd[2] = liquid
    inp.dt_factor = 0.6
    inp.n_out = n_out
    inp.level_input = 0
    inp.dt_override = dt
    inp.gravity = gravity
    return inp


def write_heyi(prefix: str, inp: DemInput, dia) -> None:
    """Write <prefix>.in and <prefix>_dia.dat in the reference's keyword format
    (the reading order of main.cpp:63-84 and ReadData.cpp:75-187; a keyword on
    its line, its values on the next).  SIZELEVEL precedes SIZELEVEL_INPUT
    because the keyword search is a prefix match (ReadData.cpp:15-19).  The
    diameter list has no trailing whitespace (the reference's reader would
    count one extra entry, DiaInput.cpp:22-27)."""
    g = lambda x: repr(float(x))  # noqa: E731  shortest round-trip form
    lines = [
        "NUMPARTICLE", str(inp.np), "SIZELEVEL", str(inp.n_levels), "LOADMODE", str(inp.load_stage),
        "packing_TIME", g(inp.t_packing), "FoceCapillary", "Yes" if inp.force_cap else "No",
        "REALSIZE", g(inp.real_size), "CUTGAPFORNEIGHBORLIST", g(inp.cut_gap), "EXPANDSIZE", g(inp.expand_size),
        "ContainerType", "Cylinder",
        "CylinderBC", " ".join(g(v) for v in (inp.cyl_x, inp.cyl_y, inp.cyl_bw, inp.cyl_r, inp.cyl_h)),
        "FeedZone", f"{g(inp.feed_lmin)} {g(inp.feed_lmax)}",
        "MATERIAL", " ".join(g(v) for v in inp.mat[0]), " ".join(g(v) for v in inp.mat[1]),
        "LIQUID", " ".join(g(v) for v in inp.lqd), "SIMULATION", f"{g(inp.dt_factor)} {inp.n_out}",
        "SIZELEVEL_INPUT", "Yes" if inp.level_input else "No",
    ]
    if inp.level_input:
        lines.append(" ".join(g(inp.level_dia[i]) for i in range(inp.n_levels)))
    with open(f"{prefix}.in", "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(f"{prefix}_dia.dat", "w") as f:
        f.write("PARTICLE DIAMETER\n" + "\n".join(g(d) for d in dia))


def hex_lattice(n: int, d: float, R: float, z0: float, spacing: float, jitter: float, seed: int) -> np.ndarray:
    """n sites of stacked hexagonal layers (ABAB) inside radius R - d/2, from z0 up,
    each jittered uniformly by +-jitter per axis (seeded)."""
    a = spacing
    dz = a * math.sqrt(2.0 / 3.0)
    rmax = R - 0.5 * d - jitter - 1e-9
    m = int(math.ceil(2 * R / a)) + 2
    ii, jj = np.meshgrid(np.arange(-m, m + 1), np.arange(-m, m + 1), indexing="ij")
    base = np.stack([a * (ii + 0.5 * jj), a * (math.sqrt(3) / 2) * jj], -1).reshape(-1, 2)
    layers = []
    k = 0
    total = 0
    while total < n:
        shift = np.array([0.5 * a, a / (2 * math.sqrt(3))]) if k % 2 else np.zeros(2)
        xy = base + shift
        xy = xy[np.hypot(xy[:, 0], xy[:, 1]) <= rmax]
        order = np.lexsort((xy[:, 0], xy[:, 1]))
        xy = xy[order]
        z = np.full((len(xy), 1), z0 + 0.5 * d + jitter + k * dz)
        layers.append(np.hstack([xy, z]))
        total += len(xy)
        k += 1
    pos = np.vstack(layers)[:n]
    rng = _rng(seed)
    return pos + rng.uniform(-jitter, jitter, size=pos.shape)


def deposit(dia: np.ndarray, R: float, z0: float, gap: float, tries: int, seed: int) -> np.ndarray:
    """Seeded sequential deposition (libdem_gb300's dem_pack_deposit)."""
    f = _abi.load().dem_pack_deposit
    d = np.ascontiguousarray(dia, np.float64)
    out = np.zeros((len(d), 3), np.float64)
    _abi.check(f(len(d), _abi.ptr(d), 0.0, 0.0, R, z0, gap, tries, seed, _abi.ptr(out)), "dem_pack_deposit")
    return out


def lognormal_diameters(n: int, median: float, sigma: float, lo: float, hi: float, seed: int) -> np.ndarray:
    rng = _rng(seed)
    out = np.empty(0)
    while len(out) < n:
        x = median * np.exp(sigma * rng.standard_normal(2 * n))
        out = np.concatenate([out, x[(x >= lo) & (x <= hi)]])
    return out[:n].copy()


# material of the packing workloads
RHO, E_YOUNG, NU, MU = 2500.0, 1.0e7, 0.3, 0.3


def dry(n: int = 5000, cyl_r: float = 8e-3, seed: int = 1, steps: int = 20000, d: float = 1e-3,
        dt: float = 1e-6, skin_frac: float = 0.1, gravity: float = 0.0) -> Workload:
    """Dry monodisperse gravity packing from a jittered hexagonal lattice."""
    yldp = yldp_for_yield_overlap(0.01, E_YOUNG, NU)
    dmpn = calibrate_dmpn(0.7, 0.5, d, RHO, E_YOUNG, NU, yldp)
    pos = hex_lattice(n, d, cyl_r, 2e-3, 1.12 * d, 0.05e-3, seed)
    top = float(pos[:, 2].max()) + 5 * d
    inp = make_input(n, 1, d, skin_frac, cyl_r, 2.0 * top, RHO, E_YOUNG, NU, MU, dmpn, yldp, 0, dt=dt,
                     gravity=gravity)
    dia = np.full(n, d)
    return Workload(f"dry{n}", inp, dia, pos, Setup.build(inp, dia), steps)


def wet(n: int = 200_000, cyl_r: float = 25e-3, seed: int = 2, steps: int = 50000, dt: float = 5e-7,
        n_levels: int = 4, skin_d: float = 1e-4, bridge_frac: float = 0.0125, gravity: float = 0.0,
        deposit_tries: int = 8, packing: str = "deposit") -> Workload:
    """Wet polydisperse packing: log-normal sizes, capillary bridges, deposited bed
    (packing="lattice": the spheres on a hexagonal lattice spaced 5 % wider than
    the largest diameter instead, apart from one another; seconds to build at
    any size)."""
    dia = lognormal_diameters(n, 1e-3, 0.2, 0.5e-3, 2.0e-3, seed)
    real = 2.0e-3  # REALSIZE: the largest admissible diameter
    rmin, rmax = dia.min() / 2, dia.max() / 2
    yldp = yldp_for_yield_overlap(0.01, E_YOUNG, NU)
    dmpn = calibrate_dmpn(0.7, 0.5, 1e-3, RHO, E_YOUNG, NU, yldp)
    if packing == "deposit":
        pos = deposit(dia, cyl_r, 0.0, 0.0, deposit_tries, seed)
    elif packing == "lattice":
        pos = hex_lattice(n, real, cyl_r, 0.0, 1.05 * real, 0.0, seed)
    else:
        raise ValueError(f"packing must be 'deposit' or 'lattice', not {packing!r}")
    top = float((pos[:, 2] + dia / 2).max())
    cut_gap = (skin_d / real) * rmax / rmin
    inp = make_input(n, n_levels, real, cut_gap, cyl_r, top + 10 * real, RHO, E_YOUNG, NU, MU, dmpn, yldp, 1,
                     liquid=(0.072, 6.0 * bridge_frac, 5e-6), dt=dt, gravity=gravity)
    return Workload(f"wet{n}", inp, dia, pos, Setup.build(inp, dia), steps)


def small_dry(n: int = 600, seed: int = 3) -> Workload:
    """A few hundred spheres, for parity tests (fills the bottom of a small cylinder)."""
    return dry(n=n, cyl_r=4e-3, seed=seed, steps=200)


def small_wet(n: int = 800, seed: int = 4, n_levels: int = 3) -> Workload:
    """Polydisperse wet bed of a few hundred spheres, for parity tests."""
    return wet(n=n, cyl_r=5e-3, seed=seed, steps=200, n_levels=n_levels)


@dataclass
class Ensemble:
    """Independent packings laid out side by side in one domain (one set-up,
    one engine), plus each packing's own set-up for running it alone."""

    combined: Workload       # all systems: one set-up, concatenated particles
    system: np.ndarray       # system of each particle of `combined` (caller order)
    cylinders: list          # CylinderBC per system, reduced units of `combined`
    wet: np.ndarray          # 1: capillary bridges act in that system
    members: list            # Workload per system, its cylinder on the axis (0, 0)
    offsets: np.ndarray      # SI (x, y) of each system's axis in the combined domain


def ensemble(n_systems: int = 256, n_range: tuple = (1000, 50000), seed: int = 3, dt: float = 5e-7,
             steps: int = 10000, n_levels: int = 4, skin_d: float = 1e-4, bridge_frac: float = 0.0125,
             phi_fill: float = 0.6, gap: float = 6e-3, threads: int | None = None) -> Ensemble:
    """n_systems packings, particle counts uniform in n_range (seeded), the wet
    workload's diameter distribution per system, cylinder radius chosen so the
    fill height is about three radii, every other system wet.  Systems are
    deposited independently (in parallel host threads) and placed on shelves
    with `gap` between cylinder walls, wider than any neighbour search, so no
    pair ever spans two systems."""
    from concurrent.futures import ThreadPoolExecutor

    rng = _rng(seed)
    counts = rng.integers(n_range[0], n_range[1] + 1, n_systems)
    wet = np.array([k % 2 for k in range(n_systems)], np.int32)
    dias = [lognormal_diameters(int(n), 1e-3, 0.2, 0.5e-3, 2.0e-3, seed * 1000 + k) for k, n in enumerate(counts)]
    radii = np.array([(np.sum(np.pi / 6 * d ** 3) / (phi_fill * 3 * np.pi)) ** (1 / 3) for d in dias])
    _abi.load()  # bind the library once, before the worker threads use it
    with ThreadPoolExecutor(threads) as ex:
        pos = list(ex.map(lambda k: deposit(dias[k], float(radii[k]), 0.0, 0.0, 8, seed * 7919 + k),
                          range(n_systems)))
    real = 2.0e-3
    rmin = min(float(d.min()) for d in dias) / 2
    rmax = max(float(d.max()) for d in dias) / 2
    cut_gap = (skin_d / real) * rmax / rmin
    yldp = yldp_for_yield_overlap(0.01, E_YOUNG, NU)
    dmpn = calibrate_dmpn(0.7, 0.5, 1e-3, RHO, E_YOUNG, NU, yldp)
    liquid = (0.072, 6.0 * bridge_frac, 5e-6)
    tops = np.array([float((p[:, 2] + d / 2).max()) + 10 * real for p, d in zip(pos, dias)])
    # shelves, largest first, in a square of about the total footprint
    order = np.argsort(-radii, kind="stable")
    side = math.sqrt(float(np.sum((2 * radii + gap) ** 2))) * 1.05
    centres = np.zeros((n_systems, 2))
    x = y = 0.0
    row_h = 0.0
    width = 0.0
    for k in order:
        d = 2 * radii[k]
        if x > 0 and x + d > side:
            y += row_h + gap
            x, row_h = 0.0, 0.0
        centres[k] = (x + radii[k], y + radii[k])
        x += d + gap
        row_h = max(row_h, d)
        width = max(width, x - gap)
    height = y + row_h
    half = 0.5 * max(width, height)
    centres -= np.array([width / 2, height / 2])
    dia_all = np.concatenate(dias)
    pos_all = np.concatenate([p + np.array([c[0], c[1], 0.0]) for p, c in zip(pos, centres)])
    system = np.concatenate([np.full(len(d), k, np.int32) for k, d in enumerate(dias)])
    inp = make_input(len(dia_all), n_levels, real, cut_gap, half, float(tops.max()), RHO, E_YOUNG, NU, MU, dmpn,
                     yldp, 1, liquid=liquid, dt=dt)
    combined = Workload(f"ensemble{n_systems}", inp, dia_all, pos_all, Setup.build(inp, dia_all), steps)
    rl = combined.setup.s.unit.rlunit
    cylinders = []
    for k in range(n_systems):
        c = _abi.CylinderBC()
        c.cir_x, c.cir_y = centres[k][0] / rl, centres[k][1] / rl
        c.R, c.Tw, c.Bw, c.topv, c.btmv = radii[k] / rl, tops[k] / rl, 0.0, 0.0, 0.0
        cylinders.append(c)
    members = []
    for k in range(n_systems):
        mi = make_input(int(counts[k]), n_levels, real, cut_gap, float(radii[k]), float(tops[k]), RHO, E_YOUNG,
                        NU, MU, dmpn, yldp, int(wet[k]), liquid=liquid if wet[k] else (0.0, 0.0, 0.0), dt=dt)
        members.append(Workload(f"system{k}", mi, dias[k], pos[k], None, steps))
    return Ensemble(combined, system, cylinders, wet, members, centres)


def member_setup(m: Workload) -> Workload:
    """the member's own set-up (built on demand: one per system alone)"""
    if m.setup is None:
        m.setup = Setup.build(m.inp, m.dia)
    return m
