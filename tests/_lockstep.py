"""Lockstep parity: before every step the oracle is loaded with the GPU
implementation's exact state (positions, velocities, spins, path lengths,
bridge counts, neighbour and wall lists, contact histories, rebuild flag);
both then take one step and that step's outputs are compared.  This checks
every step of a long run -- rebuilds and history carry-over included -- while
keeping out the chaotic growth of last-ulp differences (the reference's
stick/slip friction law is discontinuous: a 1-ulp change grows to ~1e-6 in
~50 steps of a colliding bed)."""
from __future__ import annotations

import numpy as np

import _harness


def max_per(w) -> int:
    return int(max(list(w.setup.s.level_nnebors)[: w.setup.s.n_levels]))


def flat_slots(counts: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """(particle, list position) of every used slot, particle-major in list order"""
    counts = np.asarray(counts, np.int64)
    ii = np.repeat(np.arange(len(counts)), counts)
    kk = np.arange(len(ii), dtype=np.int64) - np.repeat(np.cumsum(counts) - counts, counts)
    return ii, kk


def snapshot(eng, mp: int) -> dict:
    """the engine's full state in caller order; lists and contact records as
    the used slots end to end (the order of flat_slots)"""
    st = eng.get_state()
    counts, partners = eng.neighbors(mp)
    ii, kk = flat_slots(counts)
    rec, brg = eng.history(max(1, int(counts.max()) if len(counts) else 1))
    n = eng.n
    import ctypes as C

    from gpucode_gb300._abi import check, ptr

    pm = np.zeros(n)
    lq = np.zeros(n, np.int32)
    nw = np.zeros(n, np.int32)
    wl = np.zeros((n, 3), np.int32)
    wr = np.zeros((n, 3, 8))
    fl = C.c_int()
    check(eng.lib.dem_get_aux(eng.h, ptr(pm), ptr(lq), ptr(nw), ptr(wl), ptr(wr), C.byref(fl)), "dem_get_aux")
    return dict(pos=st["pos"], vel=st["vel"], angvel=st["angvel"], force=st["force"], pmove=pm, lqd=lq,
                counts=counts, partners=partners[ii, kk], rec=rec[ii, kk], brg=brg[ii, kk], nwall=nw, wlist=wl,
                wrec=wr, flag=fl.value)


def load_into(sim, snap: dict, it: int, first: bool) -> None:
    sim.load_state(snap["pos"], snap["vel"], snap["angvel"], snap["pmove"], snap["lqd"], snap["counts"],
                   snap["partners"], snap["rec"], snap["brg"], snap["nwall"], snap["wlist"], snap["wrec"],
                   snap["flag"], it)
    if first:
        sim.lib.orc_sim_set_counter(sim.h, b"need_build", 1)


def slip_ties(sim, w, num, hist, rel: float = 1e-9, contacts: bool = False):
    """Per particle, 2*mu*fN summed over its contacts whose spring sits on its
    slip limit after the step (0 where there is none): the largest change of
    that particle's force a flip of the friction branch can make.  With
    contacts=True, also the per-contact mask of those tie contacts (the used
    slots end to end).

    The reference's friction law branches on |dT| < dsmx (kernel.cu:191): once a
    contact slips, its spring is rescaled to exactly dsmx, so the next step's
    comparison is a near-tie, and last-ulp differences of pow (CUDA vs glibc,
    or FP32 vs FP64) pick either branch; the two branches give friction forces
    along different directions (the spring vs the slip velocity).  dsmx is
    re-derived here from each contact's stored overlap and plastic state."""
    s = w.setup.s
    cal = s.cal
    out = np.zeros(w.setup.n)
    ii, kk, _ = sim.slots_of(num)
    tie = _pair_ties(sim, w, cal, ii, hist, rel, out) if len(ii) else np.zeros(0, bool)
    _wall_ties(sim, w, s, rel, out)
    return (out, tie) if contacts else out


def _pair_ties(sim, w, cal, ii, hist, rel, out) -> np.ndarray:
    _, flat = sim.lists_flat()
    jj = flat.astype(np.int64)
    ri, rj = w.setup.rad[ii], w.setup.rad[jj]
    R = ri * rj / (ri + rj)
    nrm, plst_rad, plst_dfm, stage = hist[:, 3], hist[:, 5], hist[:, 6], hist[:, 7]
    k43 = 4.0 / 3.0 * cal.emod
    with np.errstate(invalid="ignore", divide="ignore"):
        elastic = k43 * np.sqrt(np.abs(R * nrm)) * nrm
        plastic = cal.yforce_t * R * R + cal.ystiff_t * R * (nrm - cal.ydsp_t * R)
        unload = k43 * np.sqrt(np.abs(plst_rad)) * np.abs(nrm - plst_dfm) ** 1.5
        fN = np.where(stage == 2, np.where(nrm <= cal.ydsp_t * R, elastic, plastic),
                      np.where(stage >= 3, unload, 0.0))
        dsmx = 3.0 * cal.sfrc * fN / (16.0 * (1 - cal.pois) * cal.emod / (4.0 - 2.0 * cal.pois) *
                                      np.sqrt(np.abs(R * nrm)))
        dlen = np.linalg.norm(hist[:, 0:3], axis=1)
        tie = (dsmx > 0) & (np.abs(dlen - dsmx) <= rel * dsmx)
    np.add.at(out, ii[tie], 2.0 * cal.sfrc * fN[tie])
    return tie


def _wall_ties(sim, w, s, rel, out) -> None:
    # wall contacts: R* = r_i, the wall constants, the same slip test (kernel.cu:321)
    pw = s.pwcal
    nw = sim.arr("nwall", np.int32, w.setup.n)
    wr = sim.wall_records()
    k43w = 4.0 / 3.0 * pw.emod
    for a in range(3):
        m = nw > a
        if not m.any():
            continue
        rec = wr[m, a]
        Rw = w.setup.rad[m]
        nrm, prad, pdfm, st = rec[:, 3], rec[:, 5], rec[:, 6], rec[:, 7]
        with np.errstate(invalid="ignore", divide="ignore"):
            el = k43w * np.sqrt(np.abs(Rw * nrm)) * nrm
            pl = pw.yforce_t * Rw * Rw + pw.ystiff_t * Rw * (nrm - pw.ydsp_t * Rw)
            un = k43w * np.sqrt(np.abs(prad)) * np.abs(nrm - pdfm) ** 1.5
            fN = np.where(st == 2, np.where(nrm < pw.ydsp_t * Rw, el, pl), np.where(st >= 3, un, 0.0))
            dsmx = 3.0 * pw.sfrc * fN / (16.0 * (1 - pw.pois) * pw.emod / (4.0 - 2.0 * pw.pois) *
                                         np.sqrt(np.abs(Rw * nrm)))
            dlen = np.linalg.norm(rec[:, 0:3], axis=1)
            t = (dsmx > 0) & (np.abs(dlen - dsmx) <= rel * dsmx)
        idx = np.flatnonzero(m)
        np.add.at(out, idx[t], 2.0 * pw.sfrc * fN[t])


def wall_amplification(sim, w, ulps: float = 8.0) -> np.ndarray:
    """Per particle, how far its force can move when its distance to the
    cylinder axis is rounded differently (libm vs CUDA: a few ulps).  The
    reference places a lateral-wall contact point at R (p - c) / |p - c| + c
    (kernel.cu:1009-1013) and takes the overlap r - |p - jp|: an error e of the
    distance moves the overlap by R e, relative R e / overlap (~10^4 ulps for a
    1e-3 overlap at R = 12.5), and the Hertz force ~ overlap^1.5 follows it with
    1.5 times that.  Summed over the particle's lateral-wall contacts."""
    s = w.setup.s
    pw, cyl = s.pwcal, s.cyl
    n = w.setup.n
    nw = sim.arr("nwall", np.int32, n)
    wl = sim.arr("wlist", np.int32, 3 * n).reshape(n, 3)
    wr = sim.wall_records()
    reach = cyl.R + np.hypot(cyl.cir_x, cyl.cir_y)
    out = np.zeros(n)
    k43w = 4.0 / 3.0 * pw.emod
    for a in range(3):
        m = (nw > a) & (wl[:, a] == 2)
        if not m.any():
            continue
        rec = wr[m, a]
        Rw = w.setup.rad[m]
        nrm, prad, pdfm, st = rec[:, 3], rec[:, 5], rec[:, 6], rec[:, 7]
        with np.errstate(invalid="ignore", divide="ignore"):
            el = k43w * np.sqrt(np.abs(Rw * nrm)) * nrm
            pl = pw.yforce_t * Rw * Rw + pw.ystiff_t * Rw * (nrm - pw.ydsp_t * Rw)
            un = k43w * np.sqrt(np.abs(prad)) * np.abs(nrm - pdfm) ** 1.5
            fN = np.where(st == 2, np.where(nrm < pw.ydsp_t * Rw, el, pl), np.where(st >= 3, un, 0.0))
            amp = np.where(nrm > 0, 1.5 * np.abs(fN) * reach * ulps * 2.0 ** -52 / nrm, 0.0)
        np.add.at(out, np.flatnonzero(m), np.nan_to_num(amp))
    return out


def bridge_flips(sim, w, snap, num, hist) -> np.ndarray:
    """Per particle, the capillary forces of its bridges whose flag the GPU set
    differently from the oracle: a bridge forms below a gap threshold and
    ruptures above another (kernel.cu:518-521), so where FP32 and FP64 round a
    gap on either side of one, the whole bridge force (at most 2 pi R_eff
    gamma: the regression's F* stays below 1) appears on one side only.  Only
    where the lists agree (else the list check reports them)."""
    out = np.zeros(w.setup.n)
    if not np.array_equal(snap["counts"], num):
        return out
    _, flat = sim.lists_flat()
    if len(flat) != len(snap["brg"]) or not np.array_equal(snap["partners"], flat):
        return out
    flip = np.asarray(snap["brg"]) != hist[:, 8]
    if not flip.any():
        return out
    ii, _, _ = sim.slots_of(num)
    jj = flat.astype(np.int64)
    ri, rj = w.setup.rad[ii[flip]], w.setup.rad[jj[flip]]
    np.add.at(out, ii[flip], 2.0 * np.pi * (2.0 * ri * rj / (ri + rj)) * w.setup.s.lqd.stension)
    return out


def stage_flips(sim, w, snap, num, hist) -> np.ndarray:
    """Per particle, the normal-force jumps of its contacts whose load stage the
    GPU decided differently from the oracle.  The reference's law switches from
    loading to unloading where the overlap falls below its last value
    (kernel.cu:106-113) and the two branches do not meet there: after plastic
    loading the unloading curve k (plstRad)^1/2 (d - plstDfm)^3/2 starts at
    fN (plstRad / R*)^1/2, not at the loading force fN (kernel.cu:124-129, :136).
    Where FP32 and FP64 round the overlap on either side of that turning
    point, the whole jump (and the friction it scales, mu per direction)
    appears on one side only.  Only where the lists agree."""
    out = np.zeros(w.setup.n)
    if not np.array_equal(snap["counts"], num):
        return out
    _, flat = sim.lists_flat()
    if len(flat) != len(snap["rec"]) or not np.array_equal(snap["partners"], flat):
        return out
    got = np.asarray(snap["rec"])
    flip = got[:, 7] != hist[:, 7]
    if not flip.any():
        return out
    cal = w.setup.s.cal
    ii, _, _ = sim.slots_of(num)
    i, j = ii[flip], flat.astype(np.int64)[flip]
    ri, rj = w.setup.rad[i], w.setup.rad[j]
    R = ri * rj / (ri + rj)
    a, b = hist[flip], got[flip]
    nrm = a[:, 3]
    # the plastic state before the step: kept by whichever side did not load
    keep = np.where(np.isin(a[:, 7], (3, 4))[:, None], a[:, :8], b[:, :8])
    prad, pdfm = keep[:, 5], keep[:, 6]
    k43 = 4.0 / 3.0 * cal.emod
    with np.errstate(invalid="ignore"):
        load = np.where(nrm <= cal.ydsp_t * R, k43 * np.sqrt(np.abs(R * nrm)) * nrm,
                        cal.yforce_t * R * R + cal.ystiff_t * R * (nrm - cal.ydsp_t * R))
        unload = k43 * np.sqrt(np.abs(prad)) * np.abs(nrm - pdfm) ** 1.5
    jump = np.abs(load - unload) + np.where((a[:, 7] == 1) | (b[:, 7] == 1), np.abs(unload), 0.0)
    np.add.at(out, i, (1.0 + 2.0 * cal.sfrc) * np.nan_to_num(jump))
    return out


def compare_step(snap: dict, sim, w, tol: dict, label: str, mismatch_budget: float = 0.0) -> dict:
    """Compare the GPU's post-step snapshot with the oracle's post-step state."""
    ref = sim.state()
    n = w.setup.n
    # how near its slip limit a spring counts as a tie: FP64 on both sides
    # rounds within 1e-9 of it; the mixed path keeps the spring's FP32 copy
    tie_rel = 1e-9 if mismatch_budget == 0 else 1e-5
    fscale = max(np.abs(ref["force"]).max(), 1e-300)
    perr = np.abs(snap["force"] - ref["force"]).max(axis=1) / fscale
    bad = perr > tol["force"]
    ties = 0
    if bad.any():
        num0 = sim.arr("Num_Nebor", np.int32, n).copy()
        # a flipped branch changes one friction force: bounded by 2 mu fN per tie contact;
        # last-ulp differences of the distance to the axis move lateral-wall forces
        hist0 = sim.history_flat()
        budget = slip_ties(sim, w, num0, hist0, rel=tie_rel) + wall_amplification(sim, w)
        if mismatch_budget > 0:
            budget += bridge_flips(sim, w, snap, num0, hist0) + stage_flips(sim, w, snap, num0, hist0)
        aerr = np.abs(snap["force"] - ref["force"]).max(axis=1)
        over = bad & (aerr > budget * (1 + 1e-6) + tol["force"] * fscale)
        assert not over.any(), f"{label}: force error {perr.max():.3e} not explained by slip ties, wall " \
                               f"rounding, bridge or stage flips at {np.flatnonzero(over)[:8]}"
        ties = int(bad.sum())
    ok = ~bad
    ferr = perr[ok].max() if ok.any() else 0.0
    # a velocity or spin may also move by what the force / moment tolerance lets
    # through in one step: tol_force * scale * dt / (m or I); near rest, where the
    # bed's largest speed is small, that dominates (small spheres: I ~ (2r)^5)
    dt = w.setup.s.prm.dt
    two_r = 2.0 * w.setup.rad
    mscale = max(np.abs(ref["mom"]).max(), 1e-300)
    through = {"pos": np.zeros(n), "vel": tol["force"] * fscale * dt / two_r ** 3,
               "angvel": tol["force"] * mscale * dt / (0.1 * two_r ** 5)}
    for k, tk in (("pos", "pos"), ("vel", "vel"), ("angvel", "angvel" if "angvel" in tol else "vel")):
        scale = max(np.abs(ref[k]).max(), 1e-300)
        d = np.abs(snap[k] - ref[k]).max(axis=1)
        over = d > tol[tk] * scale + through[k]
        if ok.any() and (over & ok).any():
            i = int(np.flatnonzero(over & ok)[0])
            raise AssertionError(f"{label}: {k} error {d[i] / scale:.3e} at particle {i}")
    num, flat = sim.lists_flat()
    if not np.array_equal(snap["counts"], num):
        i = int(np.flatnonzero(snap["counts"] != num)[0])
        raise AssertionError(f"{label}: list lengths (first at particle {i}: {snap['counts'][i]} vs {num[i]})")
    if not np.array_equal(snap["partners"], flat):
        ii, _ = flat_slots(num)
        i = int(ii[np.flatnonzero(snap["partners"] != flat)[0]])
        raise AssertionError(f"{label}: list of {i}")
    hist = sim.history_flat() if n else np.zeros((0, 9))
    ii, kk, _ = sim.slots_of(num)
    got = np.column_stack([snap["rec"], snap["brg"]])
    st_mis = np.mean(got[:, 7] != hist[:, 7]) if len(hist) else 0.0
    br_mis = np.mean(got[:, 8] != hist[:, 8]) if len(hist) else 0.0
    assert st_mis <= mismatch_budget and br_mis <= mismatch_budget, \
        f"{label}: stage mismatch {st_mis:.3e}, bridge mismatch {br_mis:.3e}"
    same = (got[:, 7] == hist[:, 7])
    hs = np.maximum(np.abs(hist[:, :7]).max(axis=0), 1e-300) if len(hist) else np.ones(7)
    # plstDfm = overlap - (fN / k)^(2/3) (kernel.cu:128): a difference of two
    # near-equal terms, so its rounding is relative to the overlap's scale
    hs[6] = max(hs[6], hs[3])
    rel = np.abs(got[:, :7] - hist[:, :7]) / hs
    herr = rel[same].max() if same.any() else 0.0
    if herr > tol["hist"]:
        # the spring (columns 0-2) of a tie contact legitimately differs (slip
        # rescale vs stick); nothing else of it, and nothing of other contacts
        _, tie = slip_ties(sim, w, num, hist, rel=tie_rel, contacts=True)
        spring_ok = same & tie
        excused = np.zeros_like(rel, dtype=bool)
        excused[spring_ok, 0:3] = True
        left = rel[same[:, None] & ~excused] if len(rel) else np.zeros(0)
        herr = float(left.max()) if left.size else 0.0
    if herr > tol["hist"]:
        col = int(np.argmax((rel * same[:, None]).max(axis=0)))
        raise AssertionError(f"{label}: history error {herr:.3e} (column {col} of dispt xyz, nDsp, nDsp_mx, "
                             "plstRad, plstDfm)")
    assert np.array_equal(snap["lqd"], sim.arr("lqdCnt", np.int32, n)) or mismatch_budget > 0, f"{label}: lqd"
    nw = sim.arr("nwall", np.int32, n)
    assert np.array_equal(snap["nwall"], nw), f"{label}: wall list lengths"
    wl = sim.arr("wlist", np.int32, 3 * n).reshape(n, 3)
    wr = sim.wall_records()
    # the overlap-like fields of a lateral-wall record (nDsp, nDsp_mx, plstDfm)
    # may move by R times a few ulps of the distance to the axis (wall_amplification)
    slack = (w.setup.s.cyl.R + np.hypot(w.setup.s.cyl.cir_x, w.setup.s.cyl.cir_y)) * 8.0 * 2.0 ** -52
    for a in range(3):
        m = nw > a
        assert np.array_equal(snap["wlist"][m, a], wl[m, a]), f"{label}: wall list"
        if m.any():
            ws = max(np.abs(wr[m, a, :7]).max(), 1e-300)
            dif = np.abs(snap["wrec"][m, a, :7] - wr[m, a, :7])
            lateral = (wl[m, a] == 2)[:, None] & np.isin(np.arange(7), (3, 4, 6))[None, :]
            dif = np.where(lateral, np.maximum(dif - slack, 0.0), dif)
            werr = dif.max() / ws
            assert werr <= tol["hist"] or (mismatch_budget > 0 and werr <= 1e3 * tol["hist"]), \
                f"{label}: wall history error {werr:.3e}"
    return {"force_err": ferr, "hist_err": herr, "stage_mismatch": st_mis, "tie_particles": ties}


def run(eng, w, pos, vel, ang, steps: int, tol: dict, mismatch_budget: float = 0.0, liquid: dict | None = None) -> dict:
    """`steps` steps of engine eng in lockstep with the oracle; liquid: the
    oracle's per-contact liquid model (OracleSim.set_liquid_model arguments),
    to match an engine that was given the same one"""
    sim = _harness.OracleSim(w.setup, pos, vel, ang)
    if liquid:
        sim.set_liquid_model(**liquid)
    mp = max_per(w)
    eng.set_state(pos, vel, ang)
    worst = {"force_err": 0.0, "hist_err": 0.0, "stage_mismatch": 0.0, "tie_particles": 0}
    rebuilds = 0
    for t in range(steps):
        before = snapshot(eng, mp)
        load_into(sim, before, t, first=(t == 0))
        r_sim = sim.step()
        s0 = eng.stats()["rebuilds"]
        eng.step(1)
        r_eng = eng.stats()["rebuilds"] - s0
        assert r_eng == r_sim, f"step {t}: rebuild decision {r_eng} vs {r_sim}"
        rebuilds += r_sim
        res = compare_step(snapshot(eng, mp), sim, w, tol, f"step {t}", mismatch_budget)
        for k in worst:
            worst[k] = max(worst[k], res[k])
    worst["rebuilds"] = rebuilds
    sim.close()
    return worst
