/*
 * step64.cu -- FP64 per-step kernels with the reference's formulas (sm_103a).
 *
 * The validation path: p-p contact + capillary (PPForceCalcG, kernel.cu:413-552),
 * cylinder-wall contact (CirPWInterG, kernel.cu:958-1023) and the integrator
 * (UpdateSystemG, kernel.cu:563-606), on the reference's layouts.  Compiled
 * with -fmad=false so every + and * rounds as the CPU oracle's do; the
 * remaining differences are the last-ulp differences of pow/log/exp.
 *
 * Used by the reference-compatible entry points (PpInterCalc, CirPWCalc,
 * UpdateSystem, VarInit) and by the native engine's DEM_PREC_FP64 mode, which
 * runs them on cell-sorted buffers.  On GB300 these are bound by FP64
 * transcendental issue (about 6 Gpow/s per GPU); the fast path is mixed.cu.
 */
#include <cuda_runtime.h>

#include "dem_device.cuh"

namespace dem {

namespace {

inline int grid_for(long long n, int block) { return n <= 0 ? 1 : (int)((n + block - 1) / block); }

/* VarInit (Allocation.cpp:308-317) in one pass */
__global__ void k_var_init(double3* __restrict__ force, double3* __restrict__ mom, double* __restrict__ rmom,
                           int* __restrict__ lqd, int* __restrict__ lqd_old, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  lqd_old[i] = lqd[i];
  lqd[i] = 0;
  force[i] = make_double3(0.0, 0.0, 0.0);
  mom[i] = make_double3(0.0, 0.0, 0.0);
  rmom[i] = 0.0;
}

template <class H> struct Acc;
template <> struct Acc<HistSoA> { using T = HistSoAAcc; static T make(HistSoA h) { return T{h}; } };
template <> struct Acc<HistAoS> { using T = HistAoSAcc; static T make(HistAoS h) { return T{h.rec, h.brg}; } };

/* counters[0]: neighbour entries visited, [1]: contacts, [2]: wet non-contact
 * bridges, [3]: wall contacts */
template <class HA>
__global__ void __launch_bounds__(128) k_pp_force64(
    const double3* __restrict__ pos, const double3* __restrict__ vel, const double3* __restrict__ angvel,
    const double* __restrict__ rad, const int* __restrict__ nebor, const int* __restrict__ plevel,
    const int* __restrict__ level_npars, const int* __restrict__ level_nnebors,
    const int* __restrict__ nebor_idx, HA h, const int* __restrict__ num_nebor, int* __restrict__ lqd,
    const int* __restrict__ lqd_old, double3* __restrict__ force, double3* __restrict__ mom,
    double* __restrict__ rmom, int n, int force_cap, int stage, DevConsts k,
    unsigned long long* __restrict__ counters, const int* __restrict__ id, LiquidModel lm,
    const double* __restrict__ pvol) {
  /* blocks in reverse: in cell order the largest spheres, with the most
   * pairs, come last (in the reference's order this is only another schedule) */
  const int i = reversed_block_thread();
  if (i >= n) return;
  LawCfg64 cfg;
  cfg.cal = &k.cal;
  cfg.hertz_le = true;
  cfg.rot_eps = 1.0e-7;
  cfg.dsmx_eps = 1.0e-7;
  cfg.damp_on = (stage == 1);
  cfg.dmp = sqrt(k.mat[0].dmpn * k.mat[0].dmpn);

  const double3 ip = pos[i], iv = vel[i], iw = angvel[i];
  const double ir = rad[i];
  const bool ref_liquid = force_cap == 1 && lm.mode == 0;
  const double iVol = ref_liquid ? pvol[i] : 0.0;
  double3 F = force[i];
  double3 M = mom[i];
  double R = rmom[i];
  F.z = F.z - cube(2.0 * ir); /* gravity, m = (2r)^3 */
  int wet = lqd[i];
  const int L = plevel[i];
  const long long stride = level_npars[L];
  const long long base = slot_base(L, level_npars, level_nnebors) + nebor_idx[i];
  const int nn = num_nebor[i];
  int ncontact = 0, nbridge = 0;
  /* The unit normal, the partner's liquid volume and the rupture distance
   * are evaluated only where the reference's formulas use them, by the same
   * operations: a contact or a bridge needs the normal, a bridge's force the
   * volume, and the rupture test can change only a bridge that exists beyond
   * the film distance (a flag at 0 stays 0 whatever the rupture distance).
   * On GB300 this loop is bound by FP64 issue, so the pow and divides skipped
   * for the neighbours that neither touch nor hold a bridge are the saving. */
  for (int a = 0; a < nn; a++) {
    const long long ine = base + a * stride;
    const int j = nebor[ine];
    const double3 jp = pos[j];
    const double jr = rad[j];
    const double3 d = sub3(ip, jp);
    const double dl = len3(d);
    const double gap = dl - ir - jr;
    const bool touch = gap < 0.0;
    double3 u = make_double3(0.0, 0.0, 0.0);
    if (touch) {
      u = div3(d, dl);
      const double3 jv = vel[j], jw = angvel[j];
      const double3 cpv = sub3(sub3(iv, jv), cross3(add3(mul3(iw, ir), mul3(jw, jr)), u));
      const double ijRad = ir * jr / (ir + jr);
      HistRec rec = h.load(ine);
      double3 dF, dM;
      double dR;
      contact_law64(cfg, ijRad, -gap, u, cpv, rec, ir, k.mat[0].rfrc, k.prm.dt, dF, dM, dR);
      h.store(ine, rec);
      F = add3(F, dF);
      M = add3(M, dM);
      R = R + dR;
      ncontact++;
    }
    if (force_cap != 1) continue;
    const int brg0 = h.brg(ine);
    const bool film = gap < 2 * k.lqd.layer * (ir + jr);
    if (!film && brg0 == 0) continue;
    int brg = brg0;
    if (ref_liquid) {
      const double jVol = pvol[j];
      double ijVol = iVol + jVol;
      if (film) brg = 1;
      else if (gap > 0.99 * pow(ijVol, 0.33)) brg = 0;
      if (brg != brg0) h.set_brg(ine, brg);
      if (brg == 1) {
        if (!touch) u = div3(d, dl);
        const double Splus = gap < 0 ? 0.0 : gap;
        const double effR = 2 * ir * jr / (ir + jr);
        ijVol = ijVol * 8.0;
        const double3 fc = smul3(-1.0 * fcap64(Splus, ijVol, effR, k.lqd), u);
        F = add3(F, fc);
        wet = wet + 1;
        if (gap >= 0.0) nbridge++;
      }
    } else {
      /* per-contact volume and contact angle (liquid.cuh) */
      const int idi = id ? id[i] : i, idj = id ? id[j] : j;
      const double th = 0.5 * ((double)cap_theta(idi, lm.seed, lm.theta_max) +
                               (double)cap_theta(idj, lm.seed, lm.theta_max));
      const double V = pair_bridge_volume(lm, idi, idj, ir < jr ? ir : jr);
      if (film) brg = 1;
      else if (gap > rupture64(V, th)) brg = 0;
      if (brg != brg0) h.set_brg(ine, brg);
      if (brg == 1) {
        if (!touch) u = div3(d, dl);
        const double Splus = gap < 0 ? 0.0 : gap;
        const double effR = 2 * ir * jr / (ir + jr);
        const double fcap = 2 * kPiRef * effR * k.lqd.stension * willett64(max(k.lqd.gapmn, Splus), 8.0 * V, th);
        F = add3(F, smul3(-1.0 * fcap, u));
        wet = wet + 1;
        if (gap >= 0.0) nbridge++;
      }
    }
  }
  force[i] = F;
  mom[i] = M;
  rmom[i] = R;
  lqd[i] = wet;
  if (counters) {
    atomicAdd(&counters[0], (unsigned long long)nn);
    if (ncontact) atomicAdd(&counters[1], (unsigned long long)ncontact);
    if (nbridge) atomicAdd(&counters[2], (unsigned long long)nbridge);
  }
}

/* CirPWInterG (kernel.cu:958-1023).  The reference's particle-0 thread moves
 * the top wall while other threads read it; here a one-thread launch moves it
 * first and every particle sees the moved wall. */
/* each sphere's share of liquid, vol (2r)^3 / max(bridges last step, 12)
 * (kernel.cu:429-434, :511-518): a per-sphere value the reference recomputes for
 * every neighbour entry; computed once here by the same operations */
__global__ void k_liquid_share(const double* __restrict__ rad, const int* __restrict__ lqd_old,
                               double* __restrict__ pvol, int n, DevConsts k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int nl = lqd_old[i];
  if (nl < 12) nl = 12;
  pvol[i] = k.lqd.vol * cube(rad[i] * 2) / nl;
}

__global__ void k_move_top_wall(CylinderBC* cyl, double dt) {
  if (blockIdx.x == 0 && threadIdx.x == 0) cyl->Tw = cyl->Tw + cyl->topv * dt;
}

template <class HA>
__global__ void __launch_bounds__(128) k_wall_force64(
    const double3* __restrict__ pos, const double3* __restrict__ vel, const double3* __restrict__ angvel,
    double3* __restrict__ force, double3* __restrict__ mom, double* __restrict__ rmom,
    const double* __restrict__ rad, const CylinderBC* __restrict__ cyl, HA h,
    const int* __restrict__ nwall, const int* __restrict__ wlist, size_t pitch, int n, int NP, int stage,
    DevConsts k, unsigned long long* __restrict__ counters) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  LawCfg64 cfg;
  cfg.cal = &k.pwcal;
  cfg.hertz_le = false;
  cfg.rot_eps = 1.0e-10;
  cfg.dsmx_eps = 1.0e-10;
  cfg.damp_on = (stage == 1 || stage == 7);
  cfg.dmp = sqrt(k.mat[0].dmpn * k.mat[1].dmpn);
  const CylinderBC c = *cyl;
  const double3 ip = pos[i], iv = vel[i], iw = angvel[i];
  const double ir = rad[i];
  double3 jp = make_double3(0.0, 0.0, 0.0);
  double3 jv = make_double3(0.0, 0.0, 0.0); /* persists across walls (kernel.cu:980) */
  const int* row = (const int*)((const char*)wlist + (size_t)i * pitch);
  const int nw = nwall[i];
  double3 F = force[i], M = mom[i];
  double R = rmom[i];
  int nc = 0;
  for (int a = 0; a < nw; a++) {
    const int w = row[a];
    if (w == 0) {
      jp = make_double3(ip.x, ip.y, c.Tw);
      jv = make_double3(0.0, 0.0, c.topv);
    } else if (w == 1) {
      jp = make_double3(ip.x, ip.y, c.Bw);
    } else if (w == 2) {
      /* the reference's pow(pow(dx, 2) + pow(dy, 2), 0.5) (kernel.cu:1009) as the
       * correctly rounded squares and square root it denotes: CUDA's pow has up
       * to 2 ulp of error, and the wall overlap r - |p - jp| amplifies an error
       * of dist by R / overlap (~10^4 here) */
      const double ddx = c.cir.x - ip.x, ddy = c.cir.y - ip.y;
      const double dist = sqrt(ddx * ddx + ddy * ddy);
      const double cs = (ip.x - c.cir.x) / dist;
      const double sn = (ip.y - c.cir.y) / dist;
      jp.x = c.R * cs + c.cir.x;
      jp.y = c.R * sn + c.cir.y;
      jp.z = ip.z;
    } else {
      continue;
    }
    const double3 d = sub3(ip, jp);
    const double3 u = div3(d, len3(d));
    const double gap = len3(d) - ir;
    if (gap < 0.0) {
      const double3 cpv = sub3(sub3(iv, jv), cross3(mul3(iw, ir), u));
      const long long ine = (long long)a * NP + i;
      HistRec rec = h.load(ine);
      double3 dF, dM;
      double dR;
      contact_law64(cfg, ir, -gap, u, cpv, rec, ir, k.mat[0].rfrc, k.prm.dt, dF, dM, dR);
      h.store(ine, rec);
      F = add3(F, dF);
      M = add3(M, dM);
      R = R + dR;
      nc++;
    }
  }
  force[i] = F;
  mom[i] = M;
  rmom[i] = R;
  if (counters && nc) atomicAdd(&counters[3], (unsigned long long)nc);
}

/* UpdateSystemG (kernel.cu:563-606) */
__global__ void k_update64(const double* __restrict__ rad, double3* __restrict__ pos, double3* __restrict__ vel,
                           double3* __restrict__ angvel, const double3* __restrict__ force,
                           const double3* __restrict__ mom, double* __restrict__ rmom, int* __restrict__ flag,
                           double* __restrict__ pmove, int n, double dt, double search_gap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double r = rad[i];
  const double mass = cube(2.0 * r);
  double3 v = vel[i];
  const double3 f = force[i];
  v.x = v.x + f.x * dt / mass;
  v.y = v.y + f.y * dt / mass;
  v.z = v.z + f.z * dt / mass;
  vel[i] = v;
  pos[i] = add3(pos[i], mul3(v, dt));
  const double pm = pmove[i] + len3(v) * dt;
  pmove[i] = pm;
  const double inert = 0.1 * pow5(2.0 * r);
  double3 w = angvel[i];
  const double3 m = mom[i];
  w.x = w.x + m.x * dt / inert;
  w.y = w.y + m.y * dt / inert;
  w.z = w.z + m.z * dt / inert;
  const double rm = rmom[i] * dt / inert;
  rmom[i] = rm;
  const double wl = len3(w);
  if (wl > 1.0e-7) {
    const double s = rm / wl;
    w = mul3(w, (1.0 - (s < 1.0 ? s : 1.0)));
  }
  angvel[i] = w;
  if (pm > (0.3 * search_gap)) atomicAdd(flag, 1);
}

}  // namespace

dem_status var_init(double3* force, double3* mom, double* rmom, int* lqd, int* lqd_old, int n,
                    cudaStream_t stream) {
  if (n <= 0) return DEM_OK;
  k_var_init<<<grid_for(n, 256), 256, 0, stream>>>(force, mom, rmom, lqd, lqd_old, n);
  return cuda_check(cudaGetLastError(), "var_init launch");
}

template <class H>
dem_status pp_force64(const double3* pos, const double3* vel, const double3* angvel, const double* rad,
                      const int* nebor, const int* plevel, const int* level_npars, const int* level_nnebors,
                      const int* nebor_idx, H h, const int* num_nebor, int* lqd, const int* lqd_old,
                      double3* force, double3* mom, double* rmom, int n, int force_cap, int stage,
                      const DevConsts& k, unsigned long long* counters, double* pvol, cudaStream_t stream,
                      const int* id, LiquidModel lm) {
  if (n <= 0) return DEM_OK;
  using HA = typename Acc<H>::T;
  if (force_cap == 1 && lm.mode == 0) {
    if (!pvol) return fail(DEM_ERR_ARG, "pp_force64: the liquid shares need an n-double scratch array");
    k_liquid_share<<<grid_for(n, 256), 256, 0, stream>>>(rad, lqd_old, pvol, n, k);
  }
  k_pp_force64<HA><<<grid_for(n, 128), 128, 0, stream>>>(pos, vel, angvel, rad, nebor, plevel, level_npars,
                                                        level_nnebors, nebor_idx, Acc<H>::make(h), num_nebor, lqd,
                                                        lqd_old, force, mom, rmom, n, force_cap, stage, k,
                                                        counters, id, lm, pvol);
  return cuda_check(cudaGetLastError(), "pp_force64 launch");
}

template <class H>
dem_status wall_force64(const double3* pos, const double3* vel, const double3* angvel, double3* force,
                        double3* mom, double* rmom, const double* rad, CylinderBC* cyl, H h,
                        const int* nwall, const int* wlist, size_t pitch, int n, int NP, int stage,
                        const DevConsts& k, unsigned long long* counters, bool move_wall,
                        cudaStream_t stream) {
  if (n <= 0) return DEM_OK;
  using HA = typename Acc<H>::T;
  if (move_wall) k_move_top_wall<<<1, 32, 0, stream>>>(cyl, k.prm.dt);
  k_wall_force64<HA><<<grid_for(n, 128), 128, 0, stream>>>(pos, vel, angvel, force, mom, rmom, rad, cyl,
                                                          Acc<H>::make(h), nwall, wlist, pitch, n, NP, stage, k,
                                                          counters);
  return cuda_check(cudaGetLastError(), "wall_force64 launch");
}

template dem_status pp_force64<HistSoA>(const double3*, const double3*, const double3*, const double*, const int*,
                                        const int*, const int*, const int*, const int*, HistSoA, const int*, int*,
                                        const int*, double3*, double3*, double*, int, int, int, const DevConsts&,
                                        unsigned long long*, double*, cudaStream_t, const int*, LiquidModel);
template dem_status pp_force64<HistAoS>(const double3*, const double3*, const double3*, const double*, const int*,
                                        const int*, const int*, const int*, const int*, HistAoS, const int*, int*,
                                        const int*, double3*, double3*, double*, int, int, int, const DevConsts&,
                                        unsigned long long*, double*, cudaStream_t, const int*, LiquidModel);
template dem_status wall_force64<HistSoA>(const double3*, const double3*, const double3*, double3*, double3*,
                                          double*, const double*, CylinderBC*, HistSoA, const int*, const int*,
                                          size_t, int, int, int, const DevConsts&, unsigned long long*, bool,
                                          cudaStream_t);
template dem_status wall_force64<HistAoS>(const double3*, const double3*, const double3*, double3*, double3*,
                                          double*, const double*, CylinderBC*, HistAoS, const int*, const int*,
                                          size_t, int, int, int, const DevConsts&, unsigned long long*, bool,
                                          cudaStream_t);

dem_status update64(const double* rad, double3* pos, double3* vel, double3* angvel, const double3* force,
                    const double3* mom, double* rmom, int* flag, double* pmove, int n, const DevConsts& k,
                    cudaStream_t stream) {
  if (n <= 0) return DEM_OK;
  k_update64<<<grid_for(n, 256), 256, 0, stream>>>(rad, pos, vel, angvel, force, mom, rmom, flag, pmove, n,
                                                  k.prm.dt, k.prm.SearchGap);
  return cuda_check(cudaGetLastError(), "update64 launch");
}

}  // namespace dem
