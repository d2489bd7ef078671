/*
 * mixed.cu -- the fused FP32-force / FP64-state step kernel (sm_103a).
 *
 * One launch per time step does, for each particle i (cell order, one thread):
 * gravity, every p-p contact and capillary bridge over i's neighbour slots,
 * the <= 3 cylinder-wall contacts, and the integrator -- the reference's
 * VarInit + PPForceCalcG + CirPWInterG + UpdateSystemG (kernel.cu:413-606,
 * 958-1023) in one pass.
 *
 * Why this shape on GB300: FP64 arithmetic runs at ~0.6 T op/s (1/58 of
 * FP32) and FP64 pow at ~6 G/s, so the reference's all-FP64 pair math is
 * bound by FP64 issue.  Here:
 *  - neighbours are read from FP32 "shadow" copies of last step's state
 *    (double-buffered: step t reads buffer t%2, writes the other), written by
 *    the integrator, so a neighbour costs one 16-byte gather until it is a
 *    contact candidate;
 *  - positions are shadowed as hi + lo float pairs of (x + offset), where the
 *    offset puts every coordinate in the binade [2^k, 2^(k+1)): hi_i - hi_j
 *    is then exact (Sterbenz), and the overlap d - (ri + rj) is computed as
 *    (d^2 - S^2) / (d + S) with d^2 - S^2 accumulated from exact products
 *    (FMA two-products + two-sums), so the overlap keeps ~1e-7 relative
 *    accuracy without FP64 operations even though d and S agree to 1e-4;
 *  - pair forces are FP32, summed per particle with Kahan compensation in
 *    the reference's neighbour order;
 *  - FP64 stays for the state (integrator) and for the tangential spring of
 *    the contact history, which is advanced by FP64 additions of FP32
 *    increments (projection correction, length-preserving rescale written as
 *    a small difference, v_t dt) so its accumulation error is relative to
 *    the increment, not to the spring;
 *  - contact records are 64 bytes (two DRAM sectors) read and written only for
 *    contacts; bridge flags are one byte per slot, coalesced across particles.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "capnet.cuh"
#include "dem_device.cuh"
#include "engine.h"

namespace dem {

struct MixedState {
  float4 *phi[2], *plo[2], *vel[2], *angv[2];
  float4* force;
  double3 off;
  float coarse_tol;
  int bin_exp;    /* FP64 biased exponent of the binade [2^k, 2^(k+1)) */
  float lo_scale; /* 2^(k-52): the weight of the last significand bit */
};

namespace {

inline int grid_for(long long n, int block) { return n <= 0 ? 1 : (int)((n + block - 1) / block); }

constexpr float kPiF = 3.1415926f;

/* contact-law constants in FP32 */
struct Law32 {
  float emod, pois, sfrc, ydsp, yforce, ystiff;
  float rot_eps, dsmx_eps;
  float kt;      /* 16 (1 - pois) emod / (4 - 2 pois): slip-distance denominator */
  float dmp;     /* sqrt(dmpn product) */
  int hertz_le;  /* p-p: <=, wall: < */
  int damp_on;
};

struct MixArgs {
  const float4 *phi_in, *plo_in, *v_in, *w_in;
  float4 *phi_out, *plo_out, *v_out, *w_out;
  double3 *pos, *vel, *angv;
  const double* rad;
  double* pmove;
  const int *nebor, *num_nebor, *plevel, *nidx, *npars, *nneb;
  ContactRec* rec;
  unsigned char* brg;
  const int *wlist, *nwall;
  ContactRec* wrec;
  float4* force_out;
  int *flag, *err;
  unsigned long long* counters;
  const CylinderBC* cyl;
  int n, force_cap;
  double3 off;
  float3 offf;    /* the offset rounded to FP32 */
  float wall_tol; /* bound on the error of the FP32 wall gap from the shadow */
  int bin_exp;
  float lo_scale;
  double dt, move_limit; /* 0.3 * SearchGap */
  float dtf, coarse_tol, rfrc;
  float lqd_vol, lqd_layer, lqd_gapmn, lqd_st;
  Law32 pp, pw;
  /* batched systems (NULL for one system): system of each particle id (its
   * cylinder is cyl[system]) and whether the system is wet */
  const int *sys_of_id, *sys_wet;
  /* learned capillary closure (NET variant only) */
  const int* id;
  const CapNetSmem* capw;
  unsigned long long theta_seed;
  float theta_max;
  /* a step chained on the device: the rebuild request word; when it is set
   * the step does nothing (it runs again after the rebuild).  NULL otherwise */
  const int* gate;
  /* the liquid model in FP32 (liquid.cuh): mode 0 the reference's, 1 per-contact
   * volumes (fraction lq_vmin + lq_vspan u of the smaller sphere) and angles */
  int lq_mode;
  float lq_vmin, lq_vspan, lq_theta_max;
  unsigned long long lq_seed;
};

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 operator*(float s, float3 a) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dotf(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float lenf(float3 a) { return sqrtf(dotf(a, a)); }
__device__ __forceinline__ float3 crossf(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

/* Kahan-compensated running sum */
struct KSum {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};
struct KSum3 {
  KSum x, y, z;
  __device__ __forceinline__ void add(float3 v) { x.add(v.x); y.add(v.y); z.add(v.z); }
};
/* four Kahan sums kept as (sums, compensations) in two float4s of shared memory */
__device__ __forceinline__ void kahan4(float4* acc, float3 v, float w) {
  float4 sm = acc[0], cm = acc[1];
  KSum t;
  t.s = sm.x; t.c = cm.x; t.add(v.x); sm.x = t.s; cm.x = t.c;
  t.s = sm.y; t.c = cm.y; t.add(v.y); sm.y = t.s; cm.y = t.c;
  t.s = sm.z; t.c = cm.z; t.add(v.z); sm.z = t.s; cm.z = t.c;
  t.s = sm.w; t.c = cm.w; t.add(w); sm.w = t.s; cm.w = t.c;
  acc[0] = sm;
  acc[1] = cm;
}

/* error-free transforms (Knuth two-sum, FMA two-product) */
__device__ __forceinline__ float two_sum(float a, float b, float& err) {
  const float s = a + b;
  const float bb = s - a;
  err = (a - (s - bb)) + (b - bb);
  return s;
}

/* The overlap of spheres i and j from their shadows, exactly enough for a
 * contact law: with a = hi_i - hi_j (exact: both in one binade) and
 * b = lo_i - lo_j, d^2 - S^2 is accumulated from error-free pieces (FMA
 * two-products, Knuth two-sums) and the overlap is (d^2 - S^2) / (d + S), so
 * it keeps ~1e-7 relative accuracy although d and S agree to ~1e-4.  Returns
 * the gap (negative: overlap); u is the unit vector from j to i, rj j's radius. */
__device__ __forceinline__ float exact_gap(float4 hi, float4 lo, float4 hj, float4 lj, float ax, float ay, float az,
                                           float3& u, float& rj) {
  rj = hj.w + lj.w;
  const float bx = lo.x - lj.x, by = lo.y - lj.y, bz = lo.z - lj.z;
  const float px = ax * ax, py = ay * ay, pz = az * az;
  const float ex = fmaf(ax, ax, -px), ey = fmaf(ay, ay, -py), ez = fmaf(az, az, -pz);
  float t1, t2, es;
  const float s1 = two_sum(px, py, t1);
  const float s2 = two_sum(s1, pz, t2);
  const float slo = (lo.w + lj.w);
  const float Sh = two_sum(hi.w, hj.w, es);
  const float Sl = es + slo;
  const float qq2 = Sh * Sh, eq = fmaf(Sh, Sh, -qq2);
  const float s3 = s2 - qq2;
  const float small = (t1 + t2) + (ex + ey + ez - eq) + 2.0f * (ax * bx + ay * by + az * bz) -
                      2.0f * Sh * Sl + (bx * bx + by * by + bz * bz) - Sl * Sl;
  const float D = s3 + small;
  const float dx = ax + bx, dy = ay + by, dz = az + bz;
  const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
  const float inv = __frcp_rn(dist);
  u = make_float3(dx * inv, dy * inv, dz * inv);
  return __fdividef(D, dist + (Sh + Sl));
}

/* ---- FP32 <-> FP64 through the integer pipe ----
 * On GB300 FP64 conversions issue on the scarce FP64 pipe; these move the bits
 * with integer operations instead.  d2f truncates the mantissa (error below one
 * FP32 ulp) and flushes results below the FP32 normal range to zero; f2d is
 * exact for normal floats.  Infinities and NaNs stay non-finite. */
__device__ __forceinline__ float d2f(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned sign = (unsigned)(u >> 32) & 0x80000000u;
  const int e = (int)((u >> 52) & 0x7ff);
  const int fe = e - 1023 + 127;
  if (fe <= 0) return __uint_as_float(sign);
  if (fe >= 255) return __uint_as_float(sign | 0x7f800000u | (e == 0x7ff && (u & 0xfffffffffffffull) ? 1u : 0u));
  return __uint_as_float(sign | ((unsigned)fe << 23) | (unsigned)((u >> 29) & 0x7fffffu));
}
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(b & 0x80000000u) << 32;
  if (e == 0) return __longlong_as_double((long long)sign);
  const unsigned long long de = (e == 255) ? 0x7ffull : (unsigned long long)(e - 127 + 1023);
  return __longlong_as_double((long long)(sign | (de << 52) | ((unsigned long long)(b & 0x7fffffu) << 29)));
}

/* the elasto-plastic normal law, damping, tangential spring and rolling
 * resistance of kernel.cu:89-228 / :236-359 in FP32.  The spring is advanced
 * as an FP64 update by a small FP32 increment (three FP64 adds per contact);
 * the maximum overlap stays an FP64 field. */
__device__ __forceinline__ void law32(const Law32& c, float ijRad, float nrm, float3 u, float3 cpv, MixedRec& r,
                                      float iRad, float rfrc, float dt, float3& dF, float3& dM, float& dR) {
  const float plstDfm0 = r.plstDfm, nDsp0 = r.nDsp, nDspMx0 = d2f(r.nDsp_mx);
  float plstRad = r.plstRad, plstDfm = plstDfm0;
  int st;
  if (nrm < plstDfm0) st = 1;
  else if (nrm >= plstDfm0 && nrm < nDsp0) st = 3;
  else if (nrm >= nDsp0 && nrm < nDspMx0) st = 4;
  else st = 2;
  float fN = 0.f;
  const float k43 = 4.0f / 3.0f * c.emod;
  const float sq = sqrtf(ijRad * nrm);
  if (st == 2) {
    const bool elastic = c.hertz_le ? (nrm <= c.ydsp * ijRad) : (nrm < c.ydsp * ijRad);
    if (elastic) {
      fN = k43 * sq * nrm;
      plstRad = ijRad;
      plstDfm = 0.f;
    } else {
      fN = c.yforce * ijRad * ijRad + c.ystiff * ijRad * (nrm - c.ydsp * ijRad);
      plstRad = ijRad * (k43 * sq * nrm) / fN;
      const float t = cbrtf(fN / (k43 * sqrtf(ijRad)));
      plstDfm = nrm - t * t;
    }
    r.nDsp_mx = f2d(nrm);
  } else if (st != 1) {
    const float t = nrm - plstDfm0;
    fN = k43 * sqrtf(plstRad) * (t * sqrtf(t));
  }
  const float vn = dotf(cpv, u);
  const float fD = c.damp_on ? -2.0f * c.dmp * c.emod * sq * vn : 0.f;
  const float3 vt = cpv - vn * u;

  /* spring: d_new = rescale(project(d)) + v_t dt.  With cq = u.d the
   * projection is d - u cq, of length^2 |d|^2 - cq^2, so the rescale factor
   * minus one is cq^2 / ((|d| + |p|) |p|): every term of the increment is
   * small, and its FP32 error is relative to the increment, not the spring. */
  const float3 d = f3(r.fx, r.fy, r.fz);
  const float cq = dotf(u, d);
  const float3 corr = f3(-u.x * cq, -u.y * cq, -u.z * cq);
  const float ld = lenf(d);
  const float lp = lenf(d + corr);
  float3 inc;
  if (lp > c.rot_eps) {
    const float sm1 = __fdividef(cq * cq, (ld + lp) * lp);
    inc = corr * (1.0f + sm1) + d * sm1 + vt * dt;
  } else {
    inc = corr + vt * dt;
  }
  double nx = r.dx + f2d(inc.x), ny = r.dy + f2d(inc.y), nz = r.dz + f2d(inc.z);
  float3 dn = f3(d2f(nx), d2f(ny), d2f(nz));
  const float dsmx = __fdividef(3.0f * c.sfrc * fN, c.kt * sq);
  float ratio = 1.0f;
  float ldn = lenf(dn);
  if (ldn < dsmx) {
    if (dsmx > c.dsmx_eps) {
      /* the approximate quotient may round above 1 just below the slip limit */
      const float t = fmaxf(0.0f, 1.0f - __fdividef(ldn, dsmx));
      ratio = 1.0f - t * sqrtf(t);
    }
  } else {
    const float f = (ldn > c.dsmx_eps) ? __fdividef(dsmx, ldn) : dsmx;
    const double fd = f2d(f);
    nx *= fd;
    ny *= fd;
    nz *= fd;
    dn = f3(d2f(nx), d2f(ny), d2f(nz));
    ldn = lenf(dn);
  }
  r.dx = nx;
  r.dy = ny;
  r.dz = nz;
  r.fx = dn.x;
  r.fy = dn.y;
  r.fz = dn.z;
  float3 fT = f3(0.f, 0.f, 0.f);
  if (ldn < dsmx) {
    if (ldn > 1.0e-10f) fT = dn * __fdividef(-c.sfrc * fN * ratio, ldn);
  } else {
    const float lvt = lenf(vt);
    if (lvt > 1.0e-10f) fT = vt * __fdividef(-c.sfrc * fN * ratio, lvt);
  }
  dF = (fN + fD) * u + fT;
  const float arm = iRad - nrm * 0.5f;
  dM = crossf(u * (-arm), fT);
  dR = 0.5f * (rfrc + rfrc) * fN * iRad;
  r.nDsp = nrm;
  r.plstRad = plstRad;
  r.plstDfm = plstDfm;
  r.stage = st;
}

/* a bridge's force magnitude and rupture distance under the context's liquid
 * model: V the pair's bridge volume (reduced, unscaled), th its contact angle
 * (per-contact model only).  The reference's model is kernel.cu:65-81 and
 * :518 in FP32 (the normalised regression: capnet.cuh) */
__device__ __forceinline__ float bridge_force32(const MixArgs& a, float S, float V, float th, float effR) {
  const float s = fmaxf(a.lqd_gapmn, S);
  const float fs = a.lq_mode ? willett32(s, 8.0f * V, th) : cap_formula32(s, 8.0f * V);
  return 2.0f * kPiF * effR * a.lqd_st * fs;
}
__device__ __forceinline__ float bridge_rupture32(const MixArgs& a, float V, float th) {
  return a.lq_mode ? rupture32(V, th) : 0.99f * exp2f(0.33f * __log2f(V));
}

/* A contact record is read once and written once per step: streaming
 * (evict-first) loads and stores keep it from displacing the partners'
 * shadows, which a warp's neighbours read again, from L1 (114.6 vs 118.5 us
 * on the packed 200k bed, the same bits) */
__device__ __forceinline__ MixedRec load_rec(const ContactRec* p) {
  const float4* q = reinterpret_cast<const float4*>(p);
  MixedRec r;
  float4* o = reinterpret_cast<float4*>(&r);
  o[0] = __ldcs(q + 0);
  o[1] = __ldcs(q + 1);
  o[2] = __ldcs(q + 2);
  o[3] = __ldcs(q + 3);
  return r;
}
__device__ __forceinline__ void store_rec(ContactRec* p, const MixedRec& r) {
  float4* q = reinterpret_cast<float4*>(p);
  const float4* o = reinterpret_cast<const float4*>(&r);
  __stcs(q + 0, o[0]);
  __stcs(q + 1, o[1]);
  __stcs(q + 2, o[2]);
  __stcs(q + 3, o[3]);
}

/* One p-p contact (gap < 0, unit vector u from j to i): relative velocity at
 * the contact point, the law, and the 64-byte history record of slot s read
 * and written back */
__device__ __forceinline__ void pp_contact(const Law32& law, ContactRec* rec, float ri, float rj, float3 iv,
                                           float3 iw, float4 vj4, float4 wj4, float3 u, float gap, float rfrc,
                                           float dt, float3& dF, float3& dM, float& dR) {
  MixedRec rc = load_rec(rec);
  const float3 cpv = f3(iv.x - vj4.x, iv.y - vj4.y, iv.z - vj4.z) -
                     crossf(iw * ri + f3(wj4.x, wj4.y, wj4.z) * rj, u);
  const float ijRad = ri * rj / (ri + rj);
  law32(law, ijRad, -gap, u, cpv, rc, ri, rfrc, dt, dF, dM, dR);
  store_rec(rec, rc);
}

/* hi/lo split of a coordinate already shifted into the binade [2^k, 2^(k+1)):
 * hi keeps the top 24 significand bits (exponent fixed), lo the remaining 29
 * bits as an exact integer times 2^(k-52), rounded to 24 bits.  Integer and
 * conversion units only; a value outside the binade takes the FP64 route. */
__device__ __forceinline__ void split_hi_lo(double xo, int dexp, float lo_scale, float& hi, float& lo) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(xo);
  if ((int)((u >> 52) & 0x7ff) == dexp && !(u >> 63)) {
    hi = __uint_as_float(((unsigned)(dexp - 1023 + 127) << 23) | (unsigned)((u >> 29) & 0x7fffffu));
    lo = __uint2float_rn((unsigned)(u & 0x1fffffffull)) * lo_scale;
  } else {
    hi = (float)xo;
    lo = (float)(xo - (double)hi);
  }
}

/* read-only global loads (inputs of the step: never written by this launch) */
template <class T>
__device__ __forceinline__ T ro(const T* p) {
  return __ldg(p);
}
/* pull a line into L2 ahead of its use (no register is held meanwhile) */
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

__device__ __forceinline__ void warp_add(unsigned long long* ctr, unsigned v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(ctr, (unsigned long long)v);
}

/* One bridge waiting for the learned closure: 40 bytes in a per-warp queue in
 * shared memory.  After the network has run, sep and vol hold its two outputs
 * (normalised force, rupture distance). */
struct CapEntry {
  float sep, vol, theta, ratio; /* raw features */
  float wx, wy, wz;             /* -2 pi R_eff gamma u: the force per unit normalised force */
  float gap;
  unsigned slot;
  int meta; /* bit 0: the bridge forms this step (gap below the liquid layer); bits 8..: 1 + the
               queue index of the same lane's previous entry (0: none) */
};
constexpr int kCapQ = 128; /* entries per warp; flushed before an iteration could overflow it */
#ifndef DEM_NET_BLOCKS
#define DEM_NET_BLOCKS 4
#endif
/* resident blocks per SM the network variant is built for: 4 (no register
 * spills) measured faster than 5 on the 200k wet bed */
constexpr int kNetBlocks = DEM_NET_BLOCKS;
constexpr int kWarps = 4;  /* warps per block of the step kernel */
constexpr size_t kCapSmem = ((sizeof(CapNetSmem) + 15) / 16) * 16 + sizeof(CapEntry) * kCapQ * kWarps;

__device__ __forceinline__ uint32_t cap_pair(const CapNetSmem& w, const CapEntry& e, int t) {
  return cap_pair(w, e.sep, e.vol, e.theta, e.ratio, t);
}

/* Run the queued bridges of this warp through the network in 16-row BF16
 * tensor-core tiles; each entry's sep / vol fields receive the two outputs
 * (normalised force, rupture distance).  All 32 lanes call it. */
__device__ __forceinline__ void cap_run_queue(const CapNetSmem& w, CapEntry* qw, int qn) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  __syncwarp();
  for (int t0 = 0; t0 < qn; t0 += 16) {
    const int r0 = t0 + g, r1 = r0 + 8;
    uint32_t xa = 0u, xb = 0u;
    if (t < 2) {
      if (r0 < qn) xa = cap_pair(w, qw[r0], t);
      if (r1 < qn) xb = cap_pair(w, qw[r1], t);
    }
    float o[4];
    cap_tile16(w, xa, xb, o);
    __syncwarp();
    if (t == 0) {
      if (r0 < qn) {
        qw[r0].sep = o[0] * w.y_std[0] + w.y_mean[0];
        qw[r0].vol = o[1] * w.y_std[1] + w.y_mean[1];
      }
      if (r1 < qn) {
        qw[r1].sep = o[2] * w.y_std[0] + w.y_mean[0];
        qw[r1].vol = o[3] * w.y_std[1] + w.y_mean[1];
      }
    }
    __syncwarp();
  }
}

/* Run the queue through the network, then let every lane fold in its own
 * bridges, walking its chain of entries from the newest: rupture decision,
 * bridge flag, force.  All 32 lanes call it; `last` is the lane's newest
 * entry (-1: none). */
__device__ __forceinline__ void cap_flush(const CapNetSmem& w, CapEntry* qw, int qn, int last, unsigned char* brg,
                                          KSum3& F, int& wet, unsigned& nbr, unsigned& nmlp) {
  cap_run_queue(w, qw, qn);
  for (int e = last; e >= 0;) {
    const CapEntry& en = qw[e];
    e = (en.meta >> 8) - 1;
    const int b = (en.meta & 1) ? 1 : (en.gap > en.vol ? 0 : 1);
    brg[en.slot] = (unsigned char)b;
    nmlp++;
    if (b) {
      F.add(f3(en.wx, en.wy, en.wz) * en.sep);
      wet++;
      if (en.gap >= 0.f) nbr++;
    }
  }
  __syncwarp();
}

/* After the pair loop, per particle: the <= 3 cylinder-wall contacts
 * (CirPWInterG, kernel.cu:958-1023), the integrator (UpdateSystemG,
 * kernel.cu:563-606), the next step's shadows and the counters. */
template <bool NET>
__device__ __forceinline__ void finish_particle(const MixArgs& a, int q, int qq, bool live, int sys, float4 hi,
                                                float4 lo, float4 wi4, float3 iv, float3 iw, float ri, float twor,
                                                float mass_f, KSum3& F, KSum3& M, KSum& R, int wet, unsigned nn,
                                                unsigned ncont, unsigned nbr, unsigned nmlp, unsigned nfall) {
  /* cylinder walls (CirPWInterG), geometry in FP64 */
  unsigned nwc = 0;
  double3 p = a.pos[qq];
  const int nw = live ? a.nwall[qq] : 0;
  if (nw > 0) {
    const double rid = a.rad[qq];
    const CylinderBC cy = a.cyl[sys];
    double3 jvel = make_double3(0.0, 0.0, 0.0);
    for (int w = 0; w < nw; w++) {
      const int kind = a.wlist[3 * qq + w];
      /* the top wall's velocity carries over to the walls after it in the
       * list, as the reference's jVel does (kernel.cu:987-1020) */
      if (kind == 0) jvel = make_double3(0.0, 0.0, cy.topv);
      /* A wall the particle certainly does not touch costs no FP64 work:
       * a coarse gap from the shadow (hi part of x + offset, truncated to
       * the binade) is within wall_tol of the exact one -- 5 binade ulps for
       * the flat walls, 11 for the curved one, bounded by 16 -- so only
       * particles within wall_tol of a wall take the reference's geometry. */
      float gc;
      if (kind == 0 || kind == 1) {
        gc = fabsf(hi.z - (d2f(kind == 0 ? cy.Tw : cy.Bw) + a.offf.z)) - ri;
      } else if (kind == 2) {
        const float cxo = d2f(cy.cir.x) + a.offf.x, cyo = d2f(cy.cir.y) + a.offf.y;
        const float dx = hi.x - cxo, dy = hi.y - cyo;
        gc = fabsf(sqrtf(dx * dx + dy * dy) - d2f(cy.R)) - ri;
      } else {
        continue;
      }
      if (gc > a.wall_tol) continue;
      double3 jp;
      if (kind == 0) {
        jp = make_double3(p.x, p.y, cy.Tw);
      } else if (kind == 1) {
        jp = make_double3(p.x, p.y, cy.Bw);
      } else if (kind == 2) {
        const double ddx = cy.cir.x - p.x, ddy = cy.cir.y - p.y;
        const double dist = sqrt(ddx * ddx + ddy * ddy);
        jp = make_double3(cy.R * ((p.x - cy.cir.x) / dist) + cy.cir.x, cy.R * ((p.y - cy.cir.y) / dist) + cy.cir.y,
                          p.z);
      } else {
        continue;
      }
      const double3 d = make_double3(p.x - jp.x, p.y - jp.y, p.z - jp.z);
      const double len = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
      const float gapw = (float)(len - rid);
      if (gapw < 0.f) {
        const float il = (float)(1.0 / len);
        const float3 u = f3((float)d.x * il, (float)d.y * il, (float)d.z * il);
        const float3 cpv = (iv - f3((float)jvel.x, (float)jvel.y, (float)jvel.z)) - crossf(iw * ri, u);
        ContactRec* rp = a.wrec + (long long)w * a.n + qq;
        MixedRec rc = load_rec(rp);
        float3 dF, dM;
        float dR;
        law32(a.pw, ri, -gapw, u, cpv, rc, ri, a.rfrc, a.dtf, dF, dM, dR);
        store_rec(rp, rc);
        F.add(dF);
        M.add(dM);
        R.add(dR);
        nwc++;
      }
    }
  }

  /* integrator (UpdateSystemG) in FP64 with FP32 increments */
  bool flagged = false;
  if (live) {
    /* 13 FP64 operations per particle: v += dv (3), x += v dt (3), path
     * length (1), spin (3), binade shift of the shadow (3); every conversion
     * goes through the integer pipe */
    const float fx = F.x.s - F.x.c, fy = F.y.s - F.y.c, fz = F.z.s - F.z.c;
    const float inv_m = a.dtf / mass_f;
    double3 v = a.vel[q];
    v.x += f2d(fx * inv_m);
    v.y += f2d(fy * inv_m);
    v.z += f2d(fz * inv_m);
    p.x = fma(v.x, a.dt, p.x);
    p.y = fma(v.y, a.dt, p.y);
    p.z = fma(v.z, a.dt, p.z);
    const float vxf = d2f(v.x), vyf = d2f(v.y), vzf = d2f(v.z);
    const double pm = a.pmove[q] + f2d(sqrtf(vxf * vxf + vyf * vyf + vzf * vzf) * a.dtf);
    const float inert = 0.1f * mass_f * twor * twor;
    const float inv_i = a.dtf / inert;
    double3 w = a.angv[q];
    /* spin: w += M dt / I, then the rolling-resistance damping
     * w *= 1 - min(1, Mr dt / I / |w|), folded into one increment */
    const float dwx = (M.x.s - M.x.c) * inv_i, dwy = (M.y.s - M.y.c) * inv_i, dwz = (M.z.s - M.z.c) * inv_i;
    const float rm = (R.s - R.c) * inv_i;
    const float wx1 = wi4.x + dwx, wy1 = wi4.y + dwy, wz1 = wi4.z + dwz;
    const float wl = sqrtf(wx1 * wx1 + wy1 * wy1 + wz1 * wz1);
    float ix = dwx, iy = dwy, iz = dwz;
    if (wl > 1.0e-7f) {
      const float f = fminf(1.0f, rm / wl);
      ix -= wx1 * f;
      iy -= wy1 * f;
      iz -= wz1 * f;
    }
    w.x += f2d(ix);
    w.y += f2d(iy);
    w.z += f2d(iz);
    a.vel[q] = v;
    a.pos[q] = p;
    a.angv[q] = w;
    a.pmove[q] = pm;
    flagged = pm > a.move_limit;
    if (!(isfinite(fx) && isfinite(fy) && isfinite(fz))) atomicOr(a.err, 2);
    /* next step's shadows */
    float4 ph, pl;
    split_hi_lo(p.x + a.off.x, a.bin_exp, a.lo_scale, ph.x, pl.x);
    split_hi_lo(p.y + a.off.y, a.bin_exp, a.lo_scale, ph.y, pl.y);
    split_hi_lo(p.z + a.off.z, a.bin_exp, a.lo_scale, ph.z, pl.z);
    ph.w = hi.w;
    pl.w = lo.w;
    a.phi_out[q] = ph;
    a.plo_out[q] = pl;
    a.v_out[q] = make_float4(vxf, vyf, vzf, __int_as_float(wet));
    a.w_out[q] = make_float4(d2f(w.x), d2f(w.y), d2f(w.z), 0.f);
    a.force_out[q] = make_float4(fx, fy, fz, 0.f);
  }
  const unsigned fm = __ballot_sync(0xffffffffu, flagged);
  if ((threadIdx.x & 31) == 0 && fm) atomicAdd(a.flag, __popc(fm));
  if (a.counters) {
    warp_add(&a.counters[0], (unsigned)nn);
    warp_add(&a.counters[1], ncont);
    warp_add(&a.counters[2], nbr);
    warp_add(&a.counters[3], nwc);
    if (NET) {
      warp_add(&a.counters[5], nmlp);
      warp_add(&a.counters[6], nfall);
    }
  }
}

/* resident blocks per SM the thread loop is built for: 6 (80 registers, a few
 * bytes of spills; its moment sums live in shared memory) measured 5 % faster
 * on the packed 200k wet bed than 5 (96 registers); 7 spills more and is slower */
#ifndef DEM_MIXED_BLOCKS
#define DEM_MIXED_BLOCKS 6
#endif

template <bool WET, bool NET>
__global__ void __launch_bounds__(128, NET ? kNetBlocks : DEM_MIXED_BLOCKS) k_step_mixed(MixArgs a) {
  if (a.n <= 0 || (a.gate && *a.gate)) return;
  const int q = reversed_block_thread(); /* the heaviest particles first */
  const bool live = q < a.n;
  const int qq = live ? q : a.n - 1;
  extern __shared__ __align__(16) unsigned char dsm[];
  const CapNetSmem* capw = reinterpret_cast<const CapNetSmem*>(dsm);
  CapEntry* qw = reinterpret_cast<CapEntry*>(dsm + ((sizeof(CapNetSmem) + 15) / 16) * 16) +
                 (threadIdx.x >> 5) * kCapQ;
  if (NET) {
    cap_stage(a.capw, reinterpret_cast<CapNetSmem*>(dsm));
    __syncthreads();
  }
  /* the integrator's FP64 state is needed only after the pair loop: start
   * bringing it in now */
  prefetch_l2(a.pos + qq);
  prefetch_l2(a.vel + qq);
  prefetch_l2(a.angv + qq);
  prefetch_l2(a.pmove + qq);
  /* so are the wall count and list, which would otherwise be two dependent
   * DRAM misses at the end of the warp's work */
  prefetch_l2(a.nwall + qq);
  prefetch_l2(a.wlist + 3 * qq);

  const float4 hi = ro(a.phi_in + qq), lo = ro(a.plo_in + qq), vi4 = ro(a.v_in + qq), wi4 = ro(a.w_in + qq);
  const float ri = hi.w + lo.w;
  const float3 iv = f3(vi4.x, vi4.y, vi4.z), iw = f3(wi4.x, wi4.y, wi4.z);
  const float twor = 2.0f * ri;
  const float mass_f = twor * twor * twor;
  KSum3 F;
  F.z.add(-mass_f); /* gravity, m = (2r)^3 */
  /* the moment and rolling-moment Kahan sums (sum, compensation) wait in
   * shared memory while the pairs are evaluated: registers for the pair loop */
  __shared__ float4 mr_acc[2 * 128];
  float4* const mra = mr_acc + 2 * threadIdx.x;
  mra[0] = make_float4(0.f, 0.f, 0.f, 0.f);
  mra[1] = make_float4(0.f, 0.f, 0.f, 0.f);
  int wet = 0;
  float iVol = 0.f;
  /* batched systems: this particle's system (its cylinder, dry or wet) */
  const int sys = a.sys_of_id ? a.sys_of_id[ro(a.id + qq)] : 0;
  const bool wet_i = WET && (!a.sys_wet || a.sys_wet[sys]);
  if (WET) {
    int inl = __float_as_int(vi4.w);
    if (inl < 12) inl = 12;
    iVol = a.lqd_vol * mass_f / (float)inl;
  }
  const int L = ro(a.plevel + qq);
  const long long stride = ro(a.npars + L);
  const long long base = slot_base(L, a.npars, a.nneb) + ro(a.nidx + qq);
  const int nn = live ? ro(a.num_nebor + qq) : 0;
  unsigned ncont = 0, nbr = 0, nmlp = 0, nfall = 0;
  /* learned closure: the warp walks its lanes' slots in lockstep so that
   * bridges can be queued and evaluated 16 at a time on the tensor cores */
  const int lane = threadIdx.x & 31;
  const int nloop = NET ? __reduce_max_sync(0xffffffffu, nn) : nn;
  const int id_i = (NET || (WET && a.lq_mode)) ? ro(a.id + qq) : 0;
  const float th_i = (WET && a.lq_mode) ? cap_theta32(id_i, a.lq_seed, a.lq_theta_max)
                     : NET              ? cap_theta(id_i, a.theta_seed, a.theta_max)
                                        : 0.f;
  int qn = 0;    /* entries in this warp's queue (warp-uniform) */
  int last = -1; /* this lane's newest entry in it */
  /* one slot ahead: the next partner's index and coarse shadow are in flight
   * while the current pair is evaluated */
  int j_next = nn > 0 ? ro(a.nebor + base) : 0;
  float4 hj_next = ro(a.phi_in + j_next);
  for (int k = 0; k < nloop; k++) {
    bool want = false; /* NET: this lane queues `ent` at the end of the iteration */
    CapEntry ent;
    if (!NET || k < nn) { /* the slot body (lanes with a k-th neighbour) */
    const long long s = base + k * stride;
    const int j = j_next;
    const float4 hj = hj_next;
    if (k + 1 < nn) {
      j_next = ro(a.nebor + s + stride);
      hj_next = ro(a.phi_in + j_next);
      /* the next pair's lo parts (and, wet, its velocity record and bridge
       * flag) are read by every candidate: into L2 while this pair runs */
      prefetch_l2(a.plo_in + j_next);
      if (WET) {
        prefetch_l2(a.v_in + j_next);
        prefetch_l2(a.brg + s + stride);
      }
    }
    const float ax = hi.x - hj.x, ay = hi.y - hj.y, az = hi.z - hj.z; /* exact */
    const float shi = hi.w + hj.w;
    const float coarse = sqrtf(ax * ax + ay * ay + az * az) - shi;
    float gap = coarse;
    float3 u = f3(0.f, 0.f, 0.f);
    float rj = hj.w;
    const bool cand = WET || coarse < a.coarse_tol;
    float4 vj4 = make_float4(0.f, 0.f, 0.f, 0.f);
    if (WET) vj4 = ro(a.v_in + j);
    if (cand) {
      gap = exact_gap(hi, lo, hj, ro(a.plo_in + j), ax, ay, az, u, rj);
      if (gap < 0.f) {
        if (!WET) vj4 = ro(a.v_in + j);
        float3 dF, dM;
        float dR;
        pp_contact(a.pp, a.rec + s, ri, rj, iv, iw, vj4, ro(a.w_in + j), u, gap, a.rfrc, a.dtf, dF, dM, dR);
        F.add(dF);
        kahan4(mra, dM, dR);
        ncont++;
      }
    }
    if (WET && wet_i) {
      /* the pair's bridge volume and contact angle: the reference's split of
       * both particles' liquid, or the per-contact model's */
      float ijVol, th = 0.f;
      int id_j = 0;
      if (a.lq_mode == 0) {
        int jnl = __float_as_int(vj4.w);
        if (jnl < 12) jnl = 12;
        const float tj = 2.0f * rj;
        ijVol = iVol + __fdividef(a.lqd_vol * (tj * tj * tj), (float)jnl);
      } else {
        id_j = ro(a.id + j);
        th = 0.5f * (th_i + cap_theta32(id_j, a.lq_seed, a.lq_theta_max));
        ijVol = pair_bridge_volume32(id_i, id_j, a.lq_seed, a.lq_vmin, a.lq_vspan, fminf(ri, rj));
      }
      const int bprev = a.brg[s];
      const bool form = gap < 2.0f * a.lqd_layer * (ri + rj);
      if (NET && (bprev || form)) {
        /* a bridge to evaluate: queue it for the network, or (outside the
         * network's training box) take the plain formula right here */
        const float sep = fmaxf(a.lqd_gapmn, fmaxf(gap, 0.f)), vol = 8.0f * ijVol;
        const float theta =
            a.lq_mode ? th : 0.5f * (th_i + cap_theta(ro(a.id + j), a.theta_seed, a.theta_max));
        const float ratio = __fdividef(fminf(ri, rj), fmaxf(ri, rj));
        const float effR = 2.0f * ri * rj / (ri + rj);
        if (cap_in_hull(*capw, sep, vol, theta, ratio) && s <= 0xffffffffLL) {
          const float3 wv = u * (-2.0f * kPiF * effR * a.lqd_st);
          ent = CapEntry{sep, vol, theta, ratio, wv.x, wv.y, wv.z, gap, (unsigned)s, form ? 1 : 0};
          want = true;
        } else {
          const int b = form ? 1 : (gap > bridge_rupture32(a, ijVol, th) ? 0 : 1);
          a.brg[s] = (unsigned char)b;
          if (b) {
            const float fc = bridge_force32(a, gap < 0.f ? 0.f : gap, ijVol, th, effR);
            F.add(u * (-fc));
            wet++;
            if (gap >= 0.f) nbr++;
          }
          nfall++;
        }
      } else if (!NET) {
        int b = bprev;
        if (form) b = 1;
        else if (gap > bridge_rupture32(a, ijVol, th)) b = 0;
        a.brg[s] = (unsigned char)b;
        if (b) {
          const float effR = 2.0f * ri * rj / (ri + rj);
          const float fc = bridge_force32(a, gap < 0.f ? 0.f : gap, ijVol, th, effR);
          F.add(u * (-fc));
          wet++;
          if (gap >= 0.f) nbr++;
        }
      }
    }
    }
    if (NET) {
      const unsigned m = __ballot_sync(0xffffffffu, want);
      if (want) {
        const int pos = qn + __popc(m & ((1u << lane) - 1u));
        ent.meta |= (last + 1) << 8;
        qw[pos] = ent;
        last = pos;
      }
      qn += __popc(m);
      if (qn > kCapQ - 32) {
        cap_flush(*capw, qw, qn, last, a.brg, F, wet, nbr, nmlp);
        qn = 0;
        last = -1;
      }
    }
  }
  if (NET && qn > 0) cap_flush(*capw, qw, qn, last, a.brg, F, wet, nbr, nmlp);

  KSum3 M;
  KSum R;
  {
    const float4 sm = mra[0], cm = mra[1];
    M.x.s = sm.x; M.x.c = cm.x; M.y.s = sm.y; M.y.c = cm.y; M.z.s = sm.z; M.z.c = cm.z;
    R.s = sm.w; R.c = cm.w;
  }
  finish_particle<NET>(a, q, qq, live, sys, hi, lo, wi4, iv, iw, ri, twor, mass_f, F, M, R, wet, (unsigned)nn, ncont,
                       nbr, nmlp, nfall);
}

/* ---------------- the warp-cooperative pair loop ----------------
 * One thread per particle makes a warp walk max(nn) neighbour slots with most
 * lanes idle (measured: 15 of 32 lanes active on the settled 200k wet bed) and
 * issue the whole slot body -- geometry, contact law, bridge -- once per slot
 * whatever each lane needs.  Here the 32 particles of a warp put their slots
 * end to end (inclusive shuffle scan of the slot counts) and each pass over up
 * to kChunk of them runs in phases, every lane taking the next item whichever
 * particle owns it (binary search of the scan, in shuffles):
 *   A  geometry of every pair (one 16-byte gather per partner, the exact
 *      overlap for candidates); contacts and bridges are ballot-compacted into
 *      two lists in shared memory;
 *   B  the contact law over the compacted contacts only (velocity, spin and
 *      the 64-byte record gathered together);
 *   C  the capillary bridges over the compacted bridge list (formula, or the
 *      learned closure's queue on the tensor cores);
 *   D  every lane folds its own particle's pairs, in neighbour order, into its
 *      Kahan sums.
 * so the contact law issues once per 32 contacts rather than once per 32
 * slots.  Then each lane finishes its particle (walls, integrator) as before. */

struct PairOut {
  float fx, fy, fz, mx, my, mz, rr;
  int flags;
};
enum : int { kPContact = 1, kPWet = 2, kPNbr = 4, kPMlp = 8, kPFall = 16 };

/* phase A's result for one pair */
struct PairGeo {
  float ux, uy, uz, gap;
  int j;
  float rj;
  int meta;
  int pad;
};
enum : int { kGContact = 1, kGBridge = 2, kGForm = 4 };

/* the warp's 32 particles as the pair lanes read them */
struct WarpOwn {
  float4 hi[32], lo[32];
  float4 v[32]; /* velocity, liquid volume */
  float4 w[32]; /* spin, contact angle (learned closure) */
  long long base[32];
  int stride[32];
};
static_assert(sizeof(WarpOwn) % 16 == 0, "WarpOwn keeps 16-byte alignment");

/* a lane's running sums and counts between passes (in shared memory, so
 * that they hold no registers while the pairs are evaluated) */
struct LaneAcc {
  KSum3 F, M;
  KSum R;
  int wet;
  unsigned ncont, nbr, nmlp, nfall, pad;
};
static_assert(sizeof(LaneAcc) == 80, "LaneAcc is 80 bytes");

/* a pass's pair geometry and pair results in shared memory, each pair as two
 * 16-byte halves in two arrays, so that a warp's 32 consecutive pairs are 16
 * bytes apart: one 128-bit access a quarter-warp per wavefront, no bank
 * conflicts (a 32-byte record would take two) */
struct PairBuf {
  float4* gu; /* ux, uy, uz, gap */
  int4* gm;   /* j, rj (bits), meta, pad */
  float4* oa; /* fx, fy, fz, mx */
  float4* ob; /* my, mz, rr, flags (bits) */
  __device__ __forceinline__ void put_geo(int k, const PairGeo& g) const {
    gu[k] = make_float4(g.ux, g.uy, g.uz, g.gap);
    gm[k] = make_int4(g.j, __float_as_int(g.rj), g.meta, g.pad);
  }
  __device__ __forceinline__ PairGeo geo(int k) const {
    const float4 u = gu[k];
    const int4 m = gm[k];
    return PairGeo{u.x, u.y, u.z, u.w, m.x, __int_as_float(m.y), m.z, m.w};
  }
  __device__ __forceinline__ int meta(int k) const { return reinterpret_cast<const int*>(gm + k)[2]; }
  __device__ __forceinline__ void put_out(int k, const PairOut& r) const {
    oa[k] = make_float4(r.fx, r.fy, r.fz, r.mx);
    ob[k] = make_float4(r.my, r.mz, r.rr, __int_as_float(r.flags));
  }
  __device__ __forceinline__ PairOut out(int k) const {
    const float4 x = oa[k], y = ob[k];
    return PairOut{x.x, x.y, x.z, x.w, y.x, y.y, y.z, __float_as_int(y.w)};
  }
};

#ifndef DEM_COOP_CHUNK
#define DEM_COOP_CHUNK 64
#endif

/* pairs per warp per pass (the learned closure's bridge queue holds a pass,
 * so it never has to be flushed inside one) and the per-warp shared memory:
 * own particles, lane sums, pair geometry and results, the two lists, queue */
template <bool NET>
struct Coop {
  static constexpr int kChunk = NET ? 64 : DEM_COOP_CHUNK;
  static constexpr size_t kOffAcc = sizeof(WarpOwn);
  static constexpr size_t kOffGeo = kOffAcc + 32 * sizeof(LaneAcc);
  static constexpr size_t kOffOut = kOffGeo + 32 * kChunk; /* PairBuf: two 16-byte halves per pair */
  static constexpr size_t kOffQ = kOffOut + 32 * kChunk;
  static constexpr size_t kOffList = kOffQ + (NET ? sizeof(CapEntry) * kChunk : 0);
  static constexpr size_t kWarpBytes = kOffList + 2 * kChunk;
  static constexpr size_t smem(int warps) {
    return (NET ? ((sizeof(CapNetSmem) + 15) / 16) * 16 : 0) + warps * kWarpBytes;
  }
  static_assert(kChunk % 32 == 0 && kChunk <= 256, "a pass is whole rounds of 32; list entries are bytes");
  static_assert(kWarpBytes % 16 == 0 && kOffQ % 16 == 0, "per-warp areas keep 16-byte alignment");
};

#ifndef DEM_COOP_BLOCKS
#define DEM_COOP_BLOCKS 6
#endif

/* the particle (lane) owning pair p: the number of lanes whose inclusive slot
 * count is <= p.  Every lane of the warp calls it. */
__device__ __forceinline__ int coop_owner(int incl, int p) {
  int o = 0;
#pragma unroll
  for (int b = 16; b > 0; b >>= 1) {
    const int v = __shfl_sync(0xffffffffu, incl, o + b - 1);
    if (v <= p) o += b;
  }
  return o;
}

/* phase A for one pair (owner o, partner j with coarse shadow hj): the
 * overlap -- coarse from the hi parts, exact (hi + lo, error-free
 * transforms) for candidates -- and what the later phases need */
template <bool WET>
__device__ __forceinline__ PairGeo coop_geo(const MixArgs& a, const WarpOwn& ow, int o, bool wet_o, long long s,
                                            int j, float4 hj) {
  PairGeo g;
  const float4 hi = ow.hi[o], lo = ow.lo[o];
  const float ax = hi.x - hj.x, ay = hi.y - hj.y, az = hi.z - hj.z; /* exact */
  const float coarse = sqrtf(ax * ax + ay * ay + az * az) - (hi.w + hj.w);
  g.gap = coarse;
  g.ux = g.uy = g.uz = 0.f;
  g.rj = hj.w;
  g.j = j;
  g.meta = 0;
  g.pad = 0;
  if (WET || coarse < a.coarse_tol) {
    float3 u;
    g.gap = exact_gap(hi, lo, hj, ro(a.plo_in + j), ax, ay, az, u, g.rj);
    g.ux = u.x;
    g.uy = u.y;
    g.uz = u.z;
    if (g.gap < 0.f) g.meta = kGContact;
  }
  if (WET && wet_o) {
    /* a bridge to evaluate: an existing one, or one forming this step (gap
     * below the liquid layer); the others stay unbridged (flag 0) */
    const float ri = hi.w + lo.w;
    const bool form = g.gap < 2.0f * a.lqd_layer * (ri + g.rj);
    if (form) g.meta |= kGBridge | kGForm;
    else if (a.brg[s]) g.meta |= kGBridge;
  }
  return g;
}

/* phase B for one contact: the elasto-plastic law with its history record */
__device__ __forceinline__ PairOut coop_contact(const MixArgs& a, const WarpOwn& ow, int o, long long s,
                                                const PairGeo& g) {
  const float4 hi = ow.hi[o], lo = ow.lo[o], vi = ow.v[o], wi = ow.w[o];
  float3 dF, dM;
  float dR;
  pp_contact(a.pp, a.rec + s, hi.w + lo.w, g.rj, f3(vi.x, vi.y, vi.z), f3(wi.x, wi.y, wi.z), ro(a.v_in + g.j),
             ro(a.w_in + g.j), f3(g.ux, g.uy, g.uz), g.gap, a.rfrc, a.dtf, dF, dM, dR);
  return PairOut{dF.x, dF.y, dF.z, dM.x, dM.y, dM.z, dR, kPContact};
}

/* phase C for one bridge: rupture decision, bridge flag and force with the
 * plain formula, added into the pair's result (NET: inside the network's
 * training box the bridge is queued in `ent` instead, want = true) */
template <bool NET>
__device__ __forceinline__ void coop_bridge(const MixArgs& a, const WarpOwn& ow, int o, long long s,
                                            const PairGeo& g, PairOut& out, const CapNetSmem* capw, int pidx,
                                            bool& want, CapEntry& ent) {
  const float4 hi = ow.hi[o], lo = ow.lo[o];
  const float ri = hi.w + lo.w, rj = g.rj;
  float ijVol, th = 0.f;
  if (a.lq_mode == 0) {
    int jnl = __float_as_int(ro(a.v_in + g.j).w);
    if (jnl < 12) jnl = 12;
    const float tj = 2.0f * rj;
    ijVol = ow.v[o].w + __fdividef(a.lqd_vol * (tj * tj * tj), (float)jnl);
  } else {
    const int id_j = ro(a.id + g.j);
    th = 0.5f * (ow.w[o].w + cap_theta32(id_j, a.lq_seed, a.lq_theta_max));
    ijVol = pair_bridge_volume32(__float_as_int(ow.v[o].w), id_j, a.lq_seed, a.lq_vmin, a.lq_vspan, fminf(ri, rj));
  }
  const bool form = (g.meta & kGForm) != 0;
  const float effR = 2.0f * ri * rj / (ri + rj);
  const float vol = 8.0f * ijVol;
  if (NET) {
    const float sep = fmaxf(a.lqd_gapmn, fmaxf(g.gap, 0.f));
    const float theta =
        a.lq_mode ? th : 0.5f * (ow.w[o].w + cap_theta(ro(a.id + g.j), a.theta_seed, a.theta_max));
    const float ratio = __fdividef(fminf(ri, rj), fmaxf(ri, rj));
    if (cap_in_hull(*capw, sep, vol, theta, ratio) && s <= 0xffffffffLL) {
      const float sc = -2.0f * kPiF * effR * a.lqd_st;
      ent = CapEntry{sep, vol, theta, ratio, g.ux * sc, g.uy * sc, g.uz * sc, g.gap, (unsigned)s,
                     (form ? 1 : 0) | (pidx << 8)};
      want = true;
      return;
    }
    out.flags |= kPFall;
  }
  const int b = form ? 1 : (g.gap > bridge_rupture32(a, ijVol, th) ? 0 : 1);
  a.brg[s] = (unsigned char)b;
  if (b) {
    const float fc = bridge_force32(a, g.gap < 0.f ? 0.f : g.gap, ijVol, th, effR);
    out.fx -= g.ux * fc;
    out.fy -= g.uy * fc;
    out.fz -= g.uz * fc;
    out.flags |= kPWet | (g.gap >= 0.f ? kPNbr : 0);
  }
}

/* run the pass's bridge queue through the network, then fold each entry into
 * its pair's result: rupture decision, bridge flag, force */
__device__ __forceinline__ void cap_fold_coop(const CapNetSmem& w, CapEntry* qw, int qn, const PairBuf& pb,
                                              unsigned char* brg) {
  cap_run_queue(w, qw, qn);
  for (int e = threadIdx.x & 31; e < qn; e += 32) {
    const CapEntry en = qw[e];
    const int b = (en.meta & 1) ? 1 : (en.gap > en.vol ? 0 : 1);
    brg[en.slot] = (unsigned char)b;
    PairOut r = pb.out(en.meta >> 8);
    int fl = r.flags | kPMlp;
    if (b) {
      r.fx += en.wx * en.sep;
      r.fy += en.wy * en.sep;
      r.fz += en.wz * en.sep;
      fl |= kPWet | (en.gap >= 0.f ? kPNbr : 0);
    }
    r.flags = fl;
    pb.put_out(en.meta >> 8, r);
  }
  __syncwarp();
}

/* the slot of pair p of owner o */
__device__ __forceinline__ long long coop_slot(const WarpOwn& ow, int o, int p, int eo) {
  return ow.base[o] + (long long)(p - eo) * ow.stride[o];
}

template <bool WET, bool NET>
__global__ void __launch_bounds__(128, NET ? kNetBlocks : DEM_COOP_BLOCKS) k_step_coop(MixArgs a) {
  if (a.n <= 0 || (a.gate && *a.gate)) return;
  using CF = Coop<NET>;
  constexpr int CH = CF::kChunk;
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const int q = reversed_block_thread(); /* the heaviest particles first */
  const bool live = q < a.n;
  const int qq = live ? q : a.n - 1;
  extern __shared__ __align__(16) unsigned char dsm[];
  const CapNetSmem* capw = reinterpret_cast<const CapNetSmem*>(dsm);
  unsigned char* wsm = dsm + (NET ? ((sizeof(CapNetSmem) + 15) / 16) * 16 : 0) + (threadIdx.x >> 5) * CF::kWarpBytes;
  WarpOwn& ow = *reinterpret_cast<WarpOwn*>(wsm);
  LaneAcc* acc = reinterpret_cast<LaneAcc*>(wsm + CF::kOffAcc);
  const PairBuf pb{reinterpret_cast<float4*>(wsm + CF::kOffGeo), reinterpret_cast<int4*>(wsm + CF::kOffGeo + 16 * CH),
                   reinterpret_cast<float4*>(wsm + CF::kOffOut), reinterpret_cast<float4*>(wsm + CF::kOffOut + 16 * CH)};
  CapEntry* qw = reinterpret_cast<CapEntry*>(wsm + CF::kOffQ);
  unsigned char* clist = wsm + CF::kOffList;
  unsigned char* blist = clist + CH;
  if (NET) {
    cap_stage(a.capw, reinterpret_cast<CapNetSmem*>(dsm));
    __syncthreads();
  }
  /* the integrator's FP64 state is needed only after the pair loop */
  prefetch_l2(a.pos + qq);
  prefetch_l2(a.vel + qq);
  prefetch_l2(a.angv + qq);
  prefetch_l2(a.pmove + qq);
  /* so are the wall count and list, which would otherwise be two dependent
   * DRAM misses at the end of the warp's work */
  prefetch_l2(a.nwall + qq);
  prefetch_l2(a.wlist + 3 * qq);

  const int sys = a.sys_of_id ? a.sys_of_id[ro(a.id + qq)] : 0;
  const int nn = live ? ro(a.num_nebor + qq) : 0;
  unsigned wetm;
  {
    /* this lane's particle, for the lanes that evaluate its pairs and for
     * the integrator after the loop (read back from shared memory then) */
    const float4 hi = ro(a.phi_in + qq), lo = ro(a.plo_in + qq), vi4 = ro(a.v_in + qq), wi4 = ro(a.w_in + qq);
    const float twor = 2.0f * (hi.w + lo.w);
    const float mass_f = twor * twor * twor;
    const bool wet_i = WET && (!a.sys_wet || a.sys_wet[sys]);
    float iVol = 0.f;
    if (WET) {
      int inl = __float_as_int(vi4.w);
      if (inl < 12) inl = 12;
      iVol = a.lqd_vol * mass_f / (float)inl;
    }
    const int L = ro(a.plevel + qq);
    ow.hi[lane] = hi;
    ow.lo[lane] = lo;
    /* .w of the own velocity: the liquid volume (reference model) or the
     * particle's id (per-contact model); of the own spin: the contact angle */
    const bool lqm = WET && a.lq_mode;
    const int id_i = (NET || lqm) ? ro(a.id + qq) : 0;
    ow.v[lane] = make_float4(vi4.x, vi4.y, vi4.z, lqm ? __int_as_float(id_i) : iVol);
    ow.w[lane] = make_float4(wi4.x, wi4.y, wi4.z,
                             lqm   ? cap_theta32(id_i, a.lq_seed, a.lq_theta_max)
                             : NET ? cap_theta(id_i, a.theta_seed, a.theta_max)
                                   : 0.f);
    ow.base[lane] = slot_base(L, a.npars, a.nneb) + ro(a.nidx + qq);
    ow.stride[lane] = ro(a.npars + L);
    LaneAcc z;
    z.F = KSum3();
    z.M = KSum3();
    z.R = KSum();
    z.F.z.add(-mass_f); /* gravity, m = (2r)^3 */
    z.wet = 0;
    z.ncont = z.nbr = z.nmlp = z.nfall = z.pad = 0;
    acc[lane] = z;
    wetm = __ballot_sync(FULL, wet_i);
  }
  /* the warp's slots end to end */
  int incl = nn;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += t;
  }
  const int excl = incl - nn;
  const int total = __shfl_sync(FULL, incl, 31);
  __syncwarp();

  for (int c0 = 0; c0 < total; c0 += CH) {
    const int cend = min(total, c0 + CH);
    /* ---- A: geometry of every pair; contacts and bridges listed ---- */
    int nc = 0, nb = 0;
    {
      /* pair p of this lane, and one round ahead: its partner index and
       * coarse shadow are in flight while the current pair is evaluated */
      int p = c0 + lane;
      bool act = p < cend;
      int o = coop_owner(incl, p);
      long long s = 0;
      int j = 0;
      float4 hj = make_float4(0.f, 0.f, 0.f, 0.f);
      {
        const int eo = __shfl_sync(FULL, excl, o);
        if (act) {
          s = coop_slot(ow, o, p, eo);
          j = ro(a.nebor + s);
          hj = ro(a.phi_in + j);
        }
      }
      for (int p0 = c0; p0 < cend; p0 += 32) {
        const int pn = p + 32;
        const bool actn = pn < cend;
        const int on = coop_owner(incl, pn);
        const int eon = __shfl_sync(FULL, excl, on);
        long long sn = 0;
        int jn = 0;
        float4 hjn = make_float4(0.f, 0.f, 0.f, 0.f);
        if (actn) {
          sn = coop_slot(ow, on, pn, eon);
          jn = ro(a.nebor + sn);
          hjn = ro(a.phi_in + jn);
          /* its lo parts (read for every candidate) and bridge flag: into L2 now */
          prefetch_l2(a.plo_in + jn);
          if (WET) prefetch_l2(a.brg + sn);
        }
        int meta = 0;
        if (act) {
          const PairGeo g = coop_geo<WET>(a, ow, o, (wetm >> o) & 1u, s, j, hj);
          pb.put_geo(p - c0, g);
          meta = g.meta;
          if (meta & kGContact) { /* phase B will need them: start bringing them in */
            prefetch_l2(a.rec + s);
            prefetch_l2(a.w_in + j);
          }
        }
        const unsigned mc = __ballot_sync(FULL, meta & kGContact);
        const unsigned mb = __ballot_sync(FULL, meta & kGBridge);
        if (meta & kGContact) clist[nc + __popc(mc & lt)] = (unsigned char)(p - c0);
        if (meta & kGBridge) blist[nb + __popc(mb & lt)] = (unsigned char)(p - c0);
        nc += __popc(mc);
        nb += __popc(mb);
        p = pn;
        act = actn;
        o = on;
        s = sn;
        j = jn;
        hj = hjn;
      }
    }
    __syncwarp();
    /* ---- B: the contact law over the compacted contacts ---- */
    for (int k0 = 0; k0 < nc; k0 += 32) {
      const int k = k0 + lane;
      const int pidx = k < nc ? clist[k] : 0;
      const int p = c0 + pidx;
      const int o = coop_owner(incl, p);
      const int eo = __shfl_sync(FULL, excl, o);
      if (k < nc) pb.put_out(pidx, coop_contact(a, ow, o, coop_slot(ow, o, p, eo), pb.geo(pidx)));
    }
    __syncwarp();
    /* ---- C: the bridges over the compacted list ---- */
    if (WET) {
      int qn = 0;
      for (int k0 = 0; k0 < nb; k0 += 32) {
        const int k = k0 + lane;
        const int pidx = k < nb ? blist[k] : 0;
        const int p = c0 + pidx;
        const int o = coop_owner(incl, p);
        const int eo = __shfl_sync(FULL, excl, o);
        bool want = false;
        CapEntry ent;
        if (k < nb) {
          const PairGeo g = pb.geo(pidx);
          PairOut r;
          if (g.meta & kGContact) r = pb.out(pidx);
          else r = PairOut{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0};
          coop_bridge<NET>(a, ow, o, coop_slot(ow, o, p, eo), g, r, capw, pidx, want, ent);
          pb.put_out(pidx, r);
        }
        if (NET) {
          const unsigned m = __ballot_sync(FULL, want);
          if (want) qw[qn + __popc(m & lt)] = ent;
          qn += __popc(m);
        }
      }
      if (NET && qn > 0) cap_fold_coop(*capw, qw, qn, pb, a.brg);
    }
    __syncwarp();
    /* ---- D: this lane's particle, its pairs of the pass in neighbour order ---- */
    const int k0 = max(excl, c0), k1 = min(incl, cend);
    if (k0 < k1) {
      LaneAcc A = acc[lane];
      for (int kk = k0; kk < k1; kk++) {
        if (!(pb.meta(kk - c0) & (kGContact | kGBridge))) continue;
        const PairOut r = pb.out(kk - c0);
        if (r.flags & (kPContact | kPWet)) A.F.add(f3(r.fx, r.fy, r.fz));
        if (r.flags & kPContact) {
          A.M.add(f3(r.mx, r.my, r.mz));
          A.R.add(r.rr);
          A.ncont++;
        }
        if (r.flags & kPWet) A.wet++;
        if (r.flags & kPNbr) A.nbr++;
        if (NET) {
          if (r.flags & kPMlp) A.nmlp++;
          if (r.flags & kPFall) A.nfall++;
        }
      }
      acc[lane] = A;
    }
    __syncwarp();
  }
  LaneAcc A = acc[lane];
  const float4 hi = ow.hi[lane], lo = ow.lo[lane], v = ow.v[lane], w = ow.w[lane];
  const float ri = hi.w + lo.w, twor = 2.0f * ri;
  const float4 wi4 = make_float4(w.x, w.y, w.z, 0.f);
  finish_particle<NET>(a, q, qq, live, sys, hi, lo, wi4, f3(v.x, v.y, v.z), f3(w.x, w.y, w.z), ri, twor,
                       twor * twor * twor, A.F, A.M, A.R, A.wet, (unsigned)nn, A.ncont, A.nbr, A.nmlp, A.nfall);
}

/* CirPWInterG's wall motion (kernel.cu:966-969): every cylinder's top wall
 * moves by topv dt before any particle meets it this step (not in a chained
 * step that waits for a rebuild: it moves them when it runs again) */
__global__ void k_move_walls(CylinderBC* cyl, int n_cyl, double dt, const int* gate) {
  if (gate && *gate) return;
  for (int k = threadIdx.x; k < n_cyl; k += blockDim.x) cyl[k].Tw = cyl[k].Tw + cyl[k].topv * dt;
}

__global__ void k_shadows(int n, const double3* __restrict__ pos, const double3* __restrict__ vel,
                          const double3* __restrict__ angv, const double* __restrict__ rad, const int* __restrict__ lqd,
                          double3 off, int bin_exp, float lo_scale, float4* __restrict__ phi, float4* __restrict__ plo,
                          float4* __restrict__ v4, float4* __restrict__ w4) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double3 p = pos[q];
  float4 ph, pl;
  split_hi_lo(p.x + off.x, bin_exp, lo_scale, ph.x, pl.x);
  split_hi_lo(p.y + off.y, bin_exp, lo_scale, ph.y, pl.y);
  split_hi_lo(p.z + off.z, bin_exp, lo_scale, ph.z, pl.z);
  const double r = rad[q];
  ph.w = (float)r;
  pl.w = (float)(r - (double)ph.w);
  phi[q] = ph;
  plo[q] = pl;
  const double3 v = vel[q], w = angv[q];
  v4[q] = make_float4(d2f(v.x), d2f(v.y), d2f(v.z), __int_as_float(lqd[q]));
  w4[q] = make_float4(d2f(w.x), d2f(w.y), d2f(w.z), 0.f);
}

/* A state import without a rebuild in one pass: the caller-order arrays
 * gathered into cell order (k_import), the bridge counts of the last step
 * taken from the shadow (k_lqd_from_shadow) and the shadow rewritten from the
 * new state (k_shadows) -- the same values as those three launches */
__global__ void k_import_shadows(int n, const int* __restrict__ id, const double3* __restrict__ hp,
                                 const double3* __restrict__ hv, const double3* __restrict__ hw, int has_v, int has_w,
                                 double3* __restrict__ pos, double3* __restrict__ vel, double3* __restrict__ angv,
                                 const double* __restrict__ rad, int* __restrict__ lqd, double3 off, int bin_exp,
                                 float lo_scale, float4* __restrict__ phi, float4* __restrict__ plo,
                                 float4* __restrict__ v4, float4* __restrict__ w4) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = id[q];
  const double3 p = hp[i];
  const double3 v = has_v ? hv[i] : make_double3(0.0, 0.0, 0.0);
  const double3 w = has_w ? hw[i] : make_double3(0.0, 0.0, 0.0);
  pos[q] = p;
  vel[q] = v;
  angv[q] = w;
  const int lq = __float_as_int(v4[q].w);
  lqd[q] = lq;
  float4 ph, pl;
  split_hi_lo(p.x + off.x, bin_exp, lo_scale, ph.x, pl.x);
  split_hi_lo(p.y + off.y, bin_exp, lo_scale, ph.y, pl.y);
  split_hi_lo(p.z + off.z, bin_exp, lo_scale, ph.z, pl.z);
  const double r = rad[q];
  ph.w = (float)r;
  pl.w = (float)(r - (double)ph.w);
  phi[q] = ph;
  plo[q] = pl;
  v4[q] = make_float4(d2f(v.x), d2f(v.y), d2f(v.z), __int_as_float(lq));
  w4[q] = make_float4(d2f(w.x), d2f(w.y), d2f(w.z), 0.f);
}

/* the same import from mapped host arrays read in caller order.  A block
 * walks slices of kImportThreads particles (slice, slice + gridDim.x, ...):
 * the caller's three arrays of a slice are read over the host link into
 * registers, staged in shared memory, and each thread scatters its particle
 * to cell position inv[i] (state, bridge count and shadows) -- while the next
 * slice's reads are already in flight, so the link stays busy during the
 * scatter.  16-byte reads where a slice starts 16-byte aligned (a slice of
 * 256 double3 is 6144 bytes, so all slices share the array's alignment),
 * else 8-byte reads. */
constexpr int kImportThreads = 256;
constexpr int kSliceDoubles = 3 * kImportThreads;
/* resident import blocks per SM: 4 (or 8) read the 14.4 MB state of the
 * packed 200k bed in 79 us, 2 in 84 us; one slice per block (the whole grid
 * in one wave, reads then scatters) took 89 us */
#ifndef DEM_IMPORT_BLOCKS
#define DEM_IMPORT_BLOCKS 4
#endif
constexpr int kImportBlocksPerSM = DEM_IMPORT_BLOCKS;

/* this thread's part of one slice of one array: doubles [2t, 2t+1] and
 * [2(t+256), 2(t+256)+1] (aligned), or t, t+256, t+512 (unaligned) */
struct SliceRegs {
  double2 a, b;
};

__device__ __forceinline__ void slice_fetch(const double3* __restrict__ h, int n, long long slice, bool al,
                                            SliceRegs& r) {
  const long long i0 = slice * kImportThreads;
  const int nd = 3 * (int)min((long long)kImportThreads, n - i0);
  const double* src = reinterpret_cast<const double*>(h + i0);
  const int t = threadIdx.x;
  if (al) {
    const int e0 = 2 * t, e1 = 2 * (t + kImportThreads);
    r.a = e0 + 1 < nd ? *reinterpret_cast<const double2*>(src + e0)
                      : make_double2(e0 < nd ? src[e0] : 0.0, 0.0);
    r.b = e1 + 1 < nd ? *reinterpret_cast<const double2*>(src + e1)
                      : make_double2(e1 < nd ? src[e1] : 0.0, 0.0);
  } else {
    r.a.x = t < nd ? src[t] : 0.0;
    r.a.y = t + kImportThreads < nd ? src[t + kImportThreads] : 0.0;
    r.b.x = t + 2 * kImportThreads < nd ? src[t + 2 * kImportThreads] : 0.0;
    r.b.y = 0.0;
  }
}

__device__ __forceinline__ void slice_put(const SliceRegs& r, bool al, double* sm) {
  const int t = threadIdx.x;
  if (al) {
    const int e0 = 2 * t, e1 = 2 * (t + kImportThreads);
    sm[e0] = r.a.x;
    sm[e0 + 1] = r.a.y;
    if (e1 < kSliceDoubles) {
      sm[e1] = r.b.x;
      sm[e1 + 1] = r.b.y;
    }
  } else {
    sm[t] = r.a.x;
    sm[t + kImportThreads] = r.a.y;
    sm[t + 2 * kImportThreads] = r.b.x;
  }
}

__global__ void __launch_bounds__(kImportThreads) k_import_shadows_mapped(
    int n, const int* __restrict__ inv, const double3* __restrict__ hp, const double3* __restrict__ hv,
    const double3* __restrict__ hw, double3* __restrict__ pos, double3* __restrict__ vel, double3* __restrict__ angv,
    const double* __restrict__ rad, int* __restrict__ lqd, double3 off, int bin_exp, float lo_scale,
    float4* __restrict__ phi, float4* __restrict__ plo, float4* __restrict__ v4, float4* __restrict__ w4) {
  __shared__ double sp[kSliceDoubles], sv[kSliceDoubles], sw[kSliceDoubles];
  const long long nsl = ((long long)n + kImportThreads - 1) / kImportThreads;
  const bool ap = (reinterpret_cast<size_t>(hp) & 15) == 0;
  const bool av = hv && (reinterpret_cast<size_t>(hv) & 15) == 0;
  const bool aw = hw && (reinterpret_cast<size_t>(hw) & 15) == 0;
  SliceRegs rp{}, rv{}, rw{};
  long long slice = blockIdx.x;
  if (slice < nsl) {
    slice_fetch(hp, n, slice, ap, rp);
    if (hv) slice_fetch(hv, n, slice, av, rv);
    if (hw) slice_fetch(hw, n, slice, aw, rw);
  }
  for (; slice < nsl; slice += gridDim.x) {
    slice_put(rp, ap, sp);
    if (hv) slice_put(rv, av, sv);
    if (hw) slice_put(rw, aw, sw);
    __syncthreads();
    const long long next = slice + gridDim.x;
    if (next < nsl) {
      slice_fetch(hp, n, next, ap, rp);
      if (hv) slice_fetch(hv, n, next, av, rv);
      if (hw) slice_fetch(hw, n, next, aw, rw);
    }
    const long long ii = slice * kImportThreads + threadIdx.x;
    if (ii < n) {
      const int i = (int)ii;
      const int t3 = 3 * threadIdx.x;
      const int q = inv[i];
      const double3 p = make_double3(sp[t3], sp[t3 + 1], sp[t3 + 2]);
      const double3 v = hv ? make_double3(sv[t3], sv[t3 + 1], sv[t3 + 2]) : make_double3(0.0, 0.0, 0.0);
      const double3 w = hw ? make_double3(sw[t3], sw[t3 + 1], sw[t3 + 2]) : make_double3(0.0, 0.0, 0.0);
      pos[q] = p;
      vel[q] = v;
      angv[q] = w;
      const int lq = __float_as_int(v4[q].w);
      lqd[q] = lq;
      float4 ph, pl;
      split_hi_lo(p.x + off.x, bin_exp, lo_scale, ph.x, pl.x);
      split_hi_lo(p.y + off.y, bin_exp, lo_scale, ph.y, pl.y);
      split_hi_lo(p.z + off.z, bin_exp, lo_scale, ph.z, pl.z);
      const double r = rad[q];
      ph.w = (float)r;
      pl.w = (float)(r - (double)ph.w);
      phi[q] = ph;
      plo[q] = pl;
      v4[q] = make_float4(d2f(v.x), d2f(v.y), d2f(v.z), __int_as_float(lq));
      w4[q] = make_float4(d2f(w.x), d2f(w.y), d2f(w.z), 0.f);
    }
    __syncthreads();
  }
}

__global__ void k_force_out(int n, const float4* __restrict__ f, double3* __restrict__ force, double3* __restrict__ mom) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float4 v = f[q];
  force[q] = make_double3(v.x, v.y, v.z);
  mom[q] = make_double3(0.0, 0.0, 0.0);
}

__global__ void k_lqd_from_shadow(int n, const float4* __restrict__ v4, int* __restrict__ lqd) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  lqd[q] = __float_as_int(v4[q].w);
}

Law32 make_law(const calParaPP& c, bool pp, double dmp_sq, int stage) {
  Law32 l;
  l.emod = (float)c.emod;
  l.pois = (float)c.pois;
  l.sfrc = (float)c.sfrc;
  l.ydsp = (float)c.ydsp_t;
  l.yforce = (float)c.yforce_t;
  l.ystiff = (float)c.ystiff_t;
  l.rot_eps = pp ? 1.0e-7f : 1.0e-10f;
  l.dsmx_eps = pp ? 1.0e-7f : 1.0e-10f;
  l.kt = (float)(16.0 * (1.0 - c.pois) * c.emod / (4.0 - 2.0 * c.pois));
  l.dmp = (float)std::sqrt(dmp_sq);
  l.hertz_le = pp ? 1 : 0;
  l.damp_on = pp ? (stage == 1) : (stage == 1 || stage == 7);
  return l;
}


/* ---- the reference's entry points in mixed precision ----
 * PpInterCalc and CirPWCalc (kernel.cu:413-552, :958-1023) on the reference's
 * own layouts -- spheres in the caller's order, level/slot-major lists, FP64
 * SoA histories -- with the fused step's FP32 laws: a pair's overlap from the
 * FP64 positions as (d^2 - S^2) / (d + S) with d^2 - S^2 in FP64 (eight FP64
 * operations, no FP64 square root, division or pow), the contact law and
 * the bridge in FP32, the sums in Kahan FP32 added to the FP64 force arrays.
 * The histories keep the spring and the peak overlap in FP64, as the fused
 * step does; the re-derived fields are written back as FP64 copies of FP32
 * values. */
struct RefArrays {
  const double3 *pos, *vel, *angv;
  const double* rad;
  const int *nebor, *plevel, *npars, *nneb, *nidx, *num_nebor, *lqd_old;
  int* lqd;
  HistSoA h;
  double3 *force, *mom;
  double* rmom;
  /* walls */
  const CylinderBC* cyl;
  const int *nwall, *wlist;
  size_t pitch;
  int np;
};

__device__ __forceinline__ float3 d2f3(double3 v) { return f3(d2f(v.x), d2f(v.y), d2f(v.z)); }

__device__ __forceinline__ MixedRec soa_load(const HistSoA& h, long long s) {
  MixedRec r;
  const double3 d = h.dispt[s];
  r.dx = d.x;
  r.dy = d.y;
  r.dz = d.z;
  r.nDsp_mx = h.nDsp_mx[s];
  r.fx = d2f(d.x);
  r.fy = d2f(d.y);
  r.fz = d2f(d.z);
  r.nDsp = d2f(h.nDsp[s]);
  r.plstRad = d2f(h.plstRad[s]);
  r.plstDfm = d2f(h.plstDfm[s]);
  r.stage = h.stage[s];
  r.pad = 0;
  return r;
}
__device__ __forceinline__ void soa_store(const HistSoA& h, long long s, const MixedRec& r) {
  h.dispt[s] = make_double3(r.dx, r.dy, r.dz);
  h.nDsp_mx[s] = r.nDsp_mx;
  h.nDsp[s] = f2d(r.nDsp);
  h.plstRad[s] = f2d(r.plstRad);
  h.plstDfm[s] = f2d(r.plstDfm);
  h.stage[s] = r.stage;
}

/* adds sums to an FP64 triple */
__device__ __forceinline__ double3 add_sum(double3 v, const KSum3& s) {
  return make_double3(v.x + f2d(s.x.s - s.x.c), v.y + f2d(s.y.s - s.y.c), v.z + f2d(s.z.s - s.z.c));
}

/* 6 resident blocks (80 registers, a few bytes of spills) measured 15 % faster
 * on the packed 200k bed than 5 (98 registers, no spills); 8 no better */
#ifndef DEM_REF_MIXED_BLOCKS
#define DEM_REF_MIXED_BLOCKS 6
#endif

__global__ void __launch_bounds__(128, DEM_REF_MIXED_BLOCKS) k_pp_ref_mixed(MixArgs a, RefArrays r) {
  const int i = reversed_block_thread();
  if (i >= a.n) return;
  const double3 ip = r.pos[i];
  const double ird = r.rad[i];
  const float ri = d2f(ird);
  const float3 iv = d2f3(r.vel[i]), iw = d2f3(r.angv[i]);
  const bool wet_i = a.force_cap == 1;
  float iVol = 0.f;
  if (wet_i) {
    const int inl = max(r.lqd_old[i], 12);
    const float ti = 2.0f * ri;
    iVol = __fdividef(a.lqd_vol * (ti * ti * ti), (float)inl);
  }
  KSum3 F, M;
  KSum R;
  int wet = 0;
  const int L = r.plevel[i];
  const long long stride = r.npars[L];
  const long long base = slot_base(L, r.npars, r.nneb) + r.nidx[i];
  const int nn = r.num_nebor[i];
  for (int k = 0; k < nn; k++) {
    const long long s = base + k * stride;
    const int j = r.nebor[s];
    const double3 jp = r.pos[j];
    const double jrd = r.rad[j];
    const double dx = ip.x - jp.x, dy = ip.y - jp.y, dz = ip.z - jp.z;
    const double d2 = dx * dx + dy * dy + dz * dz;
    const double S = ird + jrd;
    const double D = d2 - S * S;
    if (!wet_i && D >= 0.0) continue; /* apart: nothing to do on a dry bed */
    const float dist = sqrtf(d2f(d2));
    const float rj = d2f(jrd);
    const float gap = __fdividef(d2f(D), dist + d2f(S));
    const float inv = __frcp_rn(dist);
    const float3 u = f3(d2f(dx) * inv, d2f(dy) * inv, d2f(dz) * inv);
    if (gap < 0.f) {
      MixedRec rc = soa_load(r.h, s);
      const float3 vj = d2f3(r.vel[j]), wj = d2f3(r.angv[j]);
      const float3 cpv = (iv - vj) - crossf(iw * ri + wj * rj, u);
      float3 dF, dM;
      float dR;
      law32(a.pp, ri * rj / (ri + rj), -gap, u, cpv, rc, ri, a.rfrc, a.dtf, dF, dM, dR);
      soa_store(r.h, s, rc);
      F.add(dF);
      M.add(dM);
      R.add(dR);
    }
    if (!wet_i) continue;
    const int bprev = r.h.lqdBrg[s];
    const bool form = gap < 2.0f * a.lqd_layer * (ri + rj);
    if (!form && bprev == 0) continue;
    const int jnl = max(r.lqd_old[j], 12);
    const float tj = 2.0f * rj;
    const float ijVol = iVol + __fdividef(a.lqd_vol * (tj * tj * tj), (float)jnl);
    int b = bprev;
    if (form) b = 1;
    else if (gap > bridge_rupture32(a, ijVol, 0.f)) b = 0;
    if (b != bprev) r.h.lqdBrg[s] = b;
    if (b == 1) {
      const float fc = bridge_force32(a, gap < 0.f ? 0.f : gap, ijVol, 0.f, 2.0f * ri * rj / (ri + rj));
      F.add(u * (-fc));
      wet++;
    }
  }
  double3 f = add_sum(r.force[i], F);
  const double t = 2.0 * ird;
  f.z = f.z - t * t * t; /* gravity, m = (2r)^3 */
  r.force[i] = f;
  r.mom[i] = add_sum(r.mom[i], M);
  r.rmom[i] = r.rmom[i] + f2d(R.s - R.c);
  if (wet_i) r.lqd[i] = r.lqd[i] + wet;
}

/* CirPWInterG on the reference's wall lists (row i of pitch bytes) and wall
 * histories (slot a * NP + i); the wall point in FP64 as the fused step
 * takes it, the law in FP32.  The top wall has moved before this launch. */
__global__ void __launch_bounds__(128) k_wall_ref_mixed(MixArgs a, RefArrays r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int nw = r.nwall[i];
  if (nw <= 0) return;
  const CylinderBC cy = *r.cyl;
  const double3 p = r.pos[i];
  const double rid = r.rad[i];
  const float ri = d2f(rid);
  const float3 iv = d2f3(r.vel[i]), iw = d2f3(r.angv[i]);
  const int* row = reinterpret_cast<const int*>(reinterpret_cast<const char*>(r.wlist) + (size_t)i * r.pitch);
  KSum3 F, M;
  KSum R;
  float3 jv = f3(0.f, 0.f, 0.f); /* persists across walls (kernel.cu:980) */
  const float pxf = d2f(p.x), pyf = d2f(p.y), pzf = d2f(p.z);
  for (int w = 0; w < nw; w++) {
    const int kind = row[w];
    if (kind == 0) jv = f3(0.f, 0.f, d2f(cy.topv));
    /* A wall the sphere certainly does not touch costs no FP64 work: the gap
     * from FP32 copies of the coordinates is within tol of the exact one (a
     * few FP32 ulps of the largest coordinate involved, taken 8x) */
    float gc, tol;
    if (kind == 0 || kind == 1) {
      const float wz = d2f(kind == 0 ? cy.Tw : cy.Bw);
      gc = fabsf(pzf - wz) - ri;
      tol = 1e-6f * (fabsf(pzf) + fabsf(wz) + ri);
    } else if (kind == 2) {
      const float cx = d2f(cy.cir.x), cyy = d2f(cy.cir.y), R = d2f(cy.R);
      const float dx = pxf - cx, dy = pyf - cyy;
      gc = fabsf(sqrtf(dx * dx + dy * dy) - R) - ri;
      tol = 1e-6f * (fabsf(pxf) + fabsf(pyf) + fabsf(cx) + fabsf(cyy) + R + ri);
    } else {
      continue;
    }
    if (gc > tol) continue;
    double3 jp;
    if (kind == 0) {
      jp = make_double3(p.x, p.y, cy.Tw);
    } else if (kind == 1) {
      jp = make_double3(p.x, p.y, cy.Bw);
    } else if (kind == 2) {
      const double ddx = cy.cir.x - p.x, ddy = cy.cir.y - p.y;
      const double dist = sqrt(ddx * ddx + ddy * ddy);
      jp = make_double3(cy.R * ((p.x - cy.cir.x) / dist) + cy.cir.x, cy.R * ((p.y - cy.cir.y) / dist) + cy.cir.y,
                        p.z);
    } else {
      continue;
    }
    const double3 d = make_double3(p.x - jp.x, p.y - jp.y, p.z - jp.z);
    const double len = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
    const float gapw = d2f(len - rid);
    if (gapw >= 0.f) continue;
    const float il = __frcp_rn(d2f(len));
    const float3 u = f3(d2f(d.x) * il, d2f(d.y) * il, d2f(d.z) * il);
    const float3 cpv = (iv - jv) - crossf(iw * ri, u);
    const long long s = (long long)w * r.np + i;
    MixedRec rc = soa_load(r.h, s);
    float3 dF, dM;
    float dR;
    law32(a.pw, ri, -gapw, u, cpv, rc, ri, a.rfrc, a.dtf, dF, dM, dR);
    soa_store(r.h, s, rc);
    F.add(dF);
    M.add(dM);
    R.add(dR);
  }
  r.force[i] = add_sum(r.force[i], F);
  r.mom[i] = add_sum(r.mom[i], M);
  r.rmom[i] = r.rmom[i] + f2d(R.s - R.c);
}

/* UpdateSystemG (kernel.cu:563-606) for the reference entry points' mixed
 * mode: the increments in FP32, as the fused step's integrator takes them,
 * added to the FP64 state (no FP64 division or square root) */
__global__ void k_update_ref_mixed(const double* __restrict__ rad, double3* __restrict__ pos,
                                   double3* __restrict__ vel, double3* __restrict__ angv,
                                   const double3* __restrict__ force, const double3* __restrict__ mom,
                                   double* __restrict__ rmom, int* __restrict__ flag, double* __restrict__ pmove,
                                   int n, double dt, float dtf, double move_limit) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool flagged = false;
  if (i < n) {
    const float t = 2.0f * d2f(rad[i]);
    const float mass = t * t * t;
    const float inv_m = dtf / mass;
    const double3 f = force[i];
    double3 v = vel[i];
    v.x += f2d(d2f(f.x) * inv_m);
    v.y += f2d(d2f(f.y) * inv_m);
    v.z += f2d(d2f(f.z) * inv_m);
    vel[i] = v;
    double3 p = pos[i];
    p.x = fma(v.x, dt, p.x);
    p.y = fma(v.y, dt, p.y);
    p.z = fma(v.z, dt, p.z);
    pos[i] = p;
    const float vx = d2f(v.x), vy = d2f(v.y), vz = d2f(v.z);
    const double pm = pmove[i] + f2d(sqrtf(vx * vx + vy * vy + vz * vz) * dtf);
    pmove[i] = pm;
    const float inv_i = dtf / (0.1f * mass * t * t);
    const double3 m = mom[i];
    const float dwx = d2f(m.x) * inv_i, dwy = d2f(m.y) * inv_i, dwz = d2f(m.z) * inv_i;
    const float rm = d2f(rmom[i]) * inv_i;
    rmom[i] = f2d(rm);
    double3 w = angv[i];
    const float wx1 = d2f(w.x) + dwx, wy1 = d2f(w.y) + dwy, wz1 = d2f(w.z) + dwz;
    const float wl = sqrtf(wx1 * wx1 + wy1 * wy1 + wz1 * wz1);
    float ix = dwx, iy = dwy, iz = dwz;
    if (wl > 1.0e-7f) {
      const float s = fminf(1.0f, rm / wl);
      ix -= wx1 * s;
      iy -= wy1 * s;
      iz -= wz1 * s;
    }
    w.x += f2d(ix);
    w.y += f2d(iy);
    w.z += f2d(iz);
    angv[i] = w;
    flagged = pm > move_limit;
  }
  const unsigned fm = __ballot_sync(0xffffffffu, flagged);
  if ((threadIdx.x & 31) == 0 && fm) atomicAdd(flag, __popc(fm));
}

MixArgs ref_args(const DevConsts& k, int n, int force_cap, int stage) {
  MixArgs a;
  std::memset(&a, 0, sizeof(a));
  a.n = n;
  a.force_cap = force_cap;
  a.dt = k.prm.dt;
  a.dtf = (float)k.prm.dt;
  a.rfrc = (float)k.mat[0].rfrc;
  a.lqd_vol = (float)k.lqd.vol;
  a.lqd_layer = (float)k.lqd.layer;
  a.lqd_gapmn = (float)k.lqd.gapmn;
  a.lqd_st = (float)k.lqd.stension;
  a.pp = make_law(k.cal, true, k.mat[0].dmpn * k.mat[0].dmpn, stage);
  a.pw = make_law(k.pwcal, false, k.mat[0].dmpn * k.mat[1].dmpn, stage);
  a.lq_mode = 0;
  return a;
}
}  // namespace

#ifndef DEM_COOP_CARVEOUT
#define DEM_COOP_CARVEOUT cudaSharedmemCarveoutMaxShared
#endif

template <class K>
cudaError_t coop_attrs(K kernel, size_t smem) {
  cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess && DEM_COOP_CARVEOUT >= 0)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, DEM_COOP_CARVEOUT);
  return e;
}

dem_status mixed_create(dem_ctx* c) {
  /* the cooperative step kernels: shared memory above the default 48 KB per
   * block, and the largest shared-memory carveout (set before any capture) */
  cudaError_t e = coop_attrs(k_step_coop<true, true>, Coop<true>::smem(kWarps));
  if (e == cudaSuccess) e = coop_attrs(k_step_coop<true, false>, Coop<false>::smem(kWarps));
  if (e == cudaSuccess) e = coop_attrs(k_step_coop<false, false>, Coop<false>::smem(kWarps));
  if (e != cudaSuccess) return cuda_check(e, "mixed_create kernel attributes");
  MixedState* m = new MixedState();
  std::memset(m, 0, sizeof(*m));
  c->mx = m;
  const size_t N = (size_t)c->n;
  float4** bufs[9] = {&m->phi[0], &m->phi[1], &m->plo[0], &m->plo[1], &m->vel[0],
                      &m->vel[1], &m->angv[0], &m->angv[1], &m->force};
  for (float4** b : bufs) {
    void* p = nullptr;
    dem_status st = cuda_alloc(&p, sizeof(float4) * N);
    if (st != DEM_OK) return st;
    cudaMemset(p, 0, sizeof(float4) * N);
    c->allocs.push_back(p);
    *b = (float4*)p;
  }
  /* offset putting every coordinate of the domain in [2^k, 2^(k+1)) */
  const PARAMETER& prm = c->s.prm;
  double ext = std::max(prm.EndPoint.x - prm.Origin.x,
                        std::max(prm.EndPoint.y - prm.Origin.y, prm.EndPoint.z - prm.Origin.z));
  int k2 = (int)std::ceil(std::log2(std::max(ext, 1.0) * 1.0001));
  const double base = std::ldexp(1.0, k2);
  m->off = make_double3(base - prm.Origin.x, base - prm.Origin.y, base - prm.Origin.z);
  /* the hi-part-only overlap estimate is off by at most |lo_i - lo_j| per
   * axis, below two ulps of the binade: four ulps is a safe candidate margin */
  m->coarse_tol = (float)(4.0 * std::ldexp(1.0, k2 - 23));
  m->bin_exp = 1023 + k2;
  m->lo_scale = (float)std::ldexp(1.0, k2 - 52);
  return DEM_OK;
}

void mixed_destroy(dem_ctx* c) {
  delete c->mx;
  c->mx = nullptr;
}

dem_status mixed_shadows(dem_ctx* c, int which, cudaStream_t s) {
  MixedState* m = c->mx;
  EngineBufs& b = c->b;
  k_shadows<<<grid_for(c->n, 256), 256, 0, s>>>(c->n, b.pos, b.vel, b.angv, b.rad, b.lqd, m->off, m->bin_exp,
                                                 m->lo_scale, m->phi[which],
                                                 m->plo[which], m->vel[which], m->angv[which]);
  return cuda_check(cudaGetLastError(), "mixed_shadows launch");
}

dem_status mixed_import(dem_ctx* c, int which, int has_v, int has_w, cudaStream_t s) {
  MixedState* m = c->mx;
  EngineBufs& b = c->b;
  k_import_shadows<<<grid_for(c->n, 256), 256, 0, s>>>(c->n, b.id, b.tmp_pos, b.tmp_vel, b.tmp_angv, has_v, has_w,
                                                        b.pos, b.vel, b.angv, b.rad, b.lqd, m->off, m->bin_exp,
                                                        m->lo_scale, m->phi[which], m->plo[which], m->vel[which],
                                                        m->angv[which]);
  return cuda_check(cudaGetLastError(), "mixed_import launch");
}

dem_status mixed_import_mapped(dem_ctx* c, int which, const int* inv, const double3* hp, const double3* hv,
                               const double3* hw, cudaStream_t s) {
  MixedState* m = c->mx;
  EngineBufs& b = c->b;
  /* a few resident blocks per SM, each walking several slices */
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
  }
  const long long nsl = ((long long)c->n + kImportThreads - 1) / kImportThreads;
  const int grid = (int)std::min<long long>(nsl, (long long)kImportBlocksPerSM * sms);
  k_import_shadows_mapped<<<grid, kImportThreads, 0, s>>>(c->n, inv, hp, hv, hw, b.pos, b.vel, b.angv, b.rad, b.lqd,
                                                         m->off, m->bin_exp, m->lo_scale, m->phi[which],
                                                         m->plo[which], m->vel[which], m->angv[which]);
  return cuda_check(cudaGetLastError(), "mixed_import_mapped launch");
}

Prefilter mixed_prefilter(dem_ctx* c, int which) {
  /* |(hi_i - hi_j) - (x_i - x_j)| <= one binade ulp per axis (the lo parts are
   * below half an ulp each): sqrt(3) ulps, plus FP32 rounding of the distance
   * and of the cut-off (~3e-7 relative, distances < 4 reduced units) */
  return Prefilter{c->mx->phi[which], 0.5f * c->mx->coarse_tol + 2.0e-6f};
}

bool mixed_thread_loop(const dem_ctx* c) { return c->opt.pair_mode != DEM_PAIRS_WARP; }

const char* mixed_step_kernel_name(const dem_ctx* c) {
  const bool net = c->s.force_cap == 1 && c->opt.capillary == DEM_CAP_MLP;
  const bool wet = c->s.force_cap == 1;
  if (mixed_thread_loop(c)) return net ? "k_step_mixed<1,1>" : wet ? "k_step_mixed<1,0>" : "k_step_mixed<0,0>";
  return net ? "k_step_coop<1,1>" : wet ? "k_step_coop<1,0>" : "k_step_coop<0,0>";
}

dem_status mixed_step(dem_ctx* c, int which, cudaStream_t s) {
  MixedState* m = c->mx;
  EngineBufs& b = c->b;
  MixArgs a;
  std::memset(&a, 0, sizeof(a));
  a.phi_in = m->phi[which]; a.plo_in = m->plo[which]; a.v_in = m->vel[which]; a.w_in = m->angv[which];
  a.phi_out = m->phi[1 - which]; a.plo_out = m->plo[1 - which]; a.v_out = m->vel[1 - which];
  a.w_out = m->angv[1 - which];
  a.pos = b.pos; a.vel = b.vel; a.angv = b.angv; a.rad = b.rad; a.pmove = b.pmove;
  a.nebor = b.nebor; a.num_nebor = b.num_nebor; a.plevel = b.plevel; a.nidx = b.nidx; a.npars = b.npars;
  a.nneb = b.nneb; a.rec = b.rec; a.brg = b.brg; a.wlist = b.wlist; a.nwall = b.nwall; a.wrec = b.wrec;
  a.force_out = m->force; a.flag = b.flag; a.err = b.err; a.counters = b.counters; a.cyl = b.cyl;
  a.sys_of_id = b.sys_of_id; a.sys_wet = b.sys_wet;
  a.n = c->n;
  a.force_cap = c->s.force_cap;
  a.off = m->off;
  a.offf = make_float3((float)m->off.x, (float)m->off.y, (float)m->off.z);
  a.wall_tol = 4.0f * m->coarse_tol; /* 16 binade ulps */
  a.bin_exp = m->bin_exp;
  a.lo_scale = m->lo_scale;
  a.dt = c->s.prm.dt;
  a.dtf = (float)c->s.prm.dt;
  a.move_limit = 0.3 * c->s.prm.SearchGap;
  a.coarse_tol = m->coarse_tol;
  a.rfrc = (float)c->s.mat[0].rfrc;
  a.lqd_vol = (float)c->s.lqd.vol;
  a.lqd_layer = (float)c->s.lqd.layer;
  a.lqd_gapmn = (float)c->s.lqd.gapmn;
  a.lqd_st = (float)c->s.lqd.stension;
  a.pp = make_law(c->s.cal, true, c->s.mat[0].dmpn * c->s.mat[0].dmpn, c->s.load_stage);
  calParaPP pw;
  std::memcpy(&pw, &c->s.pwcal, sizeof(pw));
  a.pw = make_law(pw, false, c->s.mat[0].dmpn * c->s.mat[1].dmpn, c->s.load_stage);
  a.id = b.id;
  a.capw = reinterpret_cast<const CapNetSmem*>(c->cap_w);
  a.theta_seed = c->theta_seed;
  a.theta_max = c->theta_max;
  a.gate = c->step_gate;
  a.lq_mode = c->lm.mode;
  a.lq_vmin = (float)c->lm.vol_min;
  a.lq_vspan = (float)(c->lm.vol_max - c->lm.vol_min);
  a.lq_theta_max = c->lm.theta_max;
  a.lq_seed = c->lm.seed;
  const bool net = c->s.force_cap == 1 && c->opt.capillary == DEM_CAP_MLP;
  if (net && !c->cap_w) return fail(DEM_ERR_STATE, "DEM_CAP_MLP: no network installed (dem_set_capnet)");
  const bool thread_loop = mixed_thread_loop(c);
  /* threads per block: the option (a multiple of 32 up to 128), else the
   * fastest measured: one warp for the warp-cooperative loop (a block frees
   * its slot as soon as its only warp is done; 75.0 vs 79.5 us at 128 threads
   * on the deposited 200k bed), four for the thread loop (118.9 vs 121.6 us
   * at 64 and 32 threads on the packed 200k bed) and with the learned
   * closure, whose weights are staged once per block */
  const int ob = c->opt.block_size;
  const int bs = (ob >= 32 && ob <= 32 * kWarps && ob % 32 == 0) ? ob : (net || thread_loop) ? 32 * kWarps : 32;
  const int g = grid_for(c->n, bs);
  if (c->moving_walls) {
    k_move_walls<<<1, 32, 0, s>>>(b.cyl, b.n_sys > 0 ? b.n_sys : 1, c->s.prm.dt, c->step_gate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_check(e, "mixed_step wall motion");
  }
  if (thread_loop) {
    if (net) k_step_mixed<true, true><<<g, bs, kCapSmem, s>>>(a);
    else if (c->s.force_cap == 1) k_step_mixed<true, false><<<g, bs, 0, s>>>(a);
    else k_step_mixed<false, false><<<g, bs, 0, s>>>(a);
  } else {
    if (net) k_step_coop<true, true><<<g, bs, Coop<true>::smem(bs / 32), s>>>(a);
    else if (c->s.force_cap == 1) k_step_coop<true, false><<<g, bs, Coop<false>::smem(bs / 32), s>>>(a);
    else k_step_coop<false, false><<<g, bs, Coop<false>::smem(bs / 32), s>>>(a);
  }
  return cuda_check(cudaGetLastError(), "mixed_step launch");
}

dem_status mixed_pre_rebuild(dem_ctx* c, int which, cudaStream_t s) {
  /* the bridge counts of the last step travel in the shadow the next step
   * reads; bring them to the master array before it is permuted */
  k_lqd_from_shadow<<<grid_for(c->n, 256), 256, 0, s>>>(c->n, c->mx->vel[which], c->b.lqd);
  return cuda_check(cudaGetLastError(), "mixed_pre_rebuild launch");
}

const float4* mixed_force_shadow(const dem_ctx* c) { return c->mx ? c->mx->force : nullptr; }

dem_status mixed_force_to_master(dem_ctx* c, cudaStream_t s) {
  k_force_out<<<grid_for(c->n, 256), 256, 0, s>>>(c->n, c->mx->force, c->b.force, c->b.mom);
  /* the bridge counts of the last step live in the shadow the next step reads */
  k_lqd_from_shadow<<<grid_for(c->n, 256), 256, 0, s>>>(c->n, c->mx->vel[c->parity], c->b.lqd);
  return cuda_check(cudaGetLastError(), "mixed_force_to_master launch");
}

dem_status pp_force_ref_mixed(const double3* pos, const double3* vel, const double3* angvel, const double* rad,
                              const int* nebor, const int* plevel, const int* level_npars, const int* level_nnebors,
                              const int* nebor_idx, HistSoA h, const int* num_nebor, int* lqd, const int* lqd_old,
                              double3* force, double3* mom, double* rmom, int n, int force_cap, int stage,
                              const DevConsts& k, cudaStream_t s) {
  if (n <= 0) return DEM_OK;
  RefArrays r;
  std::memset(&r, 0, sizeof(r));
  r.pos = pos; r.vel = vel; r.angv = angvel; r.rad = rad;
  r.nebor = nebor; r.plevel = plevel; r.npars = level_npars; r.nneb = level_nnebors; r.nidx = nebor_idx;
  r.num_nebor = num_nebor; r.lqd_old = lqd_old; r.lqd = lqd; r.h = h;
  r.force = force; r.mom = mom; r.rmom = rmom;
  k_pp_ref_mixed<<<grid_for(n, 128), 128, 0, s>>>(ref_args(k, n, force_cap, stage), r);
  return cuda_check(cudaGetLastError(), "pp_force_ref_mixed launch");
}

dem_status wall_force_ref_mixed(const double3* pos, const double3* vel, const double3* angvel, double3* force,
                                double3* mom, double* rmom, const double* rad, CylinderBC* cyl, HistSoA h,
                                const int* nwall, const int* wlist, size_t pitch, int n, int NP, int stage,
                                const DevConsts& k, cudaStream_t s) {
  if (n <= 0) return DEM_OK;
  RefArrays r;
  std::memset(&r, 0, sizeof(r));
  r.pos = pos; r.vel = vel; r.angv = angvel; r.rad = rad; r.h = h;
  r.force = force; r.mom = mom; r.rmom = rmom;
  r.cyl = cyl; r.nwall = nwall; r.wlist = wlist; r.pitch = pitch; r.np = NP;
  k_move_walls<<<1, 32, 0, s>>>(cyl, 1, k.prm.dt, nullptr);
  k_wall_ref_mixed<<<grid_for(n, 128), 128, 0, s>>>(ref_args(k, n, 0, stage), r);
  return cuda_check(cudaGetLastError(), "wall_force_ref_mixed launch");
}

dem_status update_ref_mixed(const double* rad, double3* pos, double3* vel, double3* angvel, const double3* force,
                            const double3* mom, double* rmom, int* flag, double* pmove, int n, const DevConsts& k,
                            cudaStream_t s) {
  if (n <= 0) return DEM_OK;
  k_update_ref_mixed<<<grid_for(n, 256), 256, 0, s>>>(rad, pos, vel, angvel, force, mom, rmom, flag, pmove, n,
                                                     k.prm.dt, (float)k.prm.dt, 0.3 * k.prm.SearchGap);
  return cuda_check(cudaGetLastError(), "update_ref_mixed launch");
}

}  // namespace dem
