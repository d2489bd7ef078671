/*
 * dem_device.cuh -- device math of the DEM engine, FP64 reference-formula path.
 *
 * The contact laws here restate the reference's kernel.cu formulas with the
 * same operand order and parenthesisation, so that, compiled with
 * -fmad=false, their results differ from a CPU FP64 evaluation only by the
 * last-ulp differences of pow/log/exp between CUDA and the host libm.
 */
#pragma once

#include <cuda_runtime.h>

#include "dem_internal.h"
#include "liquid.cuh"

namespace dem {

/* heydem.h:15 */
constexpr double kPiRef = 3.1415926;

/* ---- double3 algebra in the reference's evaluation order (double_math.h) ---- */
__device__ __forceinline__ double3 d3(double x, double y, double z) { return make_double3(x, y, z); }
__device__ __forceinline__ double3 add3(double3 a, double3 b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ double3 sub3(double3 a, double3 b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double3 mul3(double3 a, double s) { return d3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double3 smul3(double s, double3 a) { return d3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ double3 div3(double3 a, double s) { return d3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double len3(double3 a) { return sqrt(dot3(a, a)); }
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
  return d3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

/* The reference's pow with the exponents 1.5, 3 and 5 as products of sqrt and
 * x (IEEE sqrt and products, no contraction in the FP64 files): x^1.5 and x^3
 * land within 1.3 ulp of the exact power and x^5 within 2.6 ulp (three
 * roundings), against 2 ulp for CUDA's pow and 0.52 for the CPU oracle's --
 * relative differences of a few 1e-16, far inside the 1e-12 lockstep bound --
 * for a few FP64 instructions instead of some tens: on GB300 the FP64 laws are
 * bound by FP64 issue.  pow5 only scales the integrator's spin increments. */
__device__ __forceinline__ double pow1_5(double x) { return x * sqrt(x); }
__device__ __forceinline__ double cube(double x) { return x * x * x; }
__device__ __forceinline__ double pow5(double x) {
  const double x2 = x * x;
  return x2 * x2 * x;
}

/* This thread's particle with the blocks taken in reverse.  Particles sit in
 * level-major cell order, so the largest spheres -- the most neighbours, the
 * longest loops -- come last; the GPU starts blocks roughly in index order,
 * and in index order their blocks would run in the grid's tail.  Taken first,
 * they overlap the many light blocks instead (each particle's work is its
 * own, so the results are the same bits). */
__device__ __forceinline__ int reversed_block_thread() {
  return (int)((gridDim.x - 1 - blockIdx.x) * blockDim.x + threadIdx.x);
}

/* ---- cell hash (kernel.cu:617-641) ---- */
__device__ __forceinline__ int3 grid_pos(double3 p, int lvl, const LevelView& lv, double3 origin) {
  const double cs = lv.cell_size[lvl];
  const int3 g = lv.grid_size[lvl];
  int3 r;
  r.x = max(0, min((int)floor((p.x - origin.x) / cs), g.x));
  r.y = max(0, min((int)floor((p.y - origin.y) / cs), g.y));
  r.z = max(0, min((int)floor((p.z - origin.z) / cs), g.z));
  return r;
}
__device__ __forceinline__ int grid_hash(int3 g, int lvl, const LevelView& lv) {
  const int3 s = lv.grid_size[lvl];
  return (g.z * s.y * s.x) + (g.y * s.x) + g.x;
}

/* first slot of level L's block in a level/slot-major list: the sum over the
 * lower levels of slots x particles (kernel.cu:443-454); reads levels < L only */
__device__ __forceinline__ long long slot_base(int L, const int* npars, const int* nneb) {
  long long b = 0;
  for (int l = 0; l < L; l++) b += (long long)nneb[l] * npars[l];
  return b;
}

/* ---- history record (the fields of one contact slot) ---- */
struct HistRec {
  double3 dispt;
  double nDsp, nDsp_mx, plstRad, plstDfm;
  int stage;
};

/* history access, reference SoA layout */
struct HistSoAAcc {
  HistSoA h;
  __device__ __forceinline__ HistRec load(long long i) const {
    HistRec r;
    r.dispt = h.dispt[i];
    r.nDsp = h.nDsp[i];
    r.nDsp_mx = h.nDsp_mx[i];
    r.plstRad = h.plstRad[i];
    r.plstDfm = h.plstDfm[i];
    r.stage = h.stage[i];
    return r;
  }
  __device__ __forceinline__ void store(long long i, const HistRec& r) const {
    h.dispt[i] = r.dispt;
    h.nDsp[i] = r.nDsp;
    h.nDsp_mx[i] = r.nDsp_mx;
    h.plstRad[i] = r.plstRad;
    h.plstDfm[i] = r.plstDfm;
    h.stage[i] = r.stage;
  }
  __device__ __forceinline__ int brg(long long i) const { return h.lqdBrg[i]; }
  __device__ __forceinline__ void set_brg(long long i, int v) const { h.lqdBrg[i] = v; }
};

/* history access, the engine's 64-byte records + one bridge byte per slot */
struct HistAoSAcc {
  ContactRec* rec;
  unsigned char* brgf;
  __device__ __forceinline__ HistRec load(long long i) const {
    const double2* p = reinterpret_cast<const double2*>(rec + i);
    const double2 a = p[0], b = p[1], c = p[2];
    const double2 d = p[3];
    HistRec r;
    r.dispt = make_double3(a.x, a.y, b.x);
    r.nDsp = b.y;
    r.nDsp_mx = c.x;
    r.plstRad = c.y;
    r.plstDfm = d.x;
    r.stage = __double_as_longlong(d.y) & 0xffffffff;
    return r;
  }
  __device__ __forceinline__ void store(long long i, const HistRec& r) const {
    double2* p = reinterpret_cast<double2*>(rec + i);
    p[0] = make_double2(r.dispt.x, r.dispt.y);
    p[1] = make_double2(r.dispt.z, r.nDsp);
    p[2] = make_double2(r.nDsp_mx, r.plstRad);
    p[3] = make_double2(r.plstDfm, __longlong_as_double((long long)(unsigned)r.stage));
  }
  __device__ __forceinline__ int brg(long long i) const { return brgf ? brgf[i] : 0; }
  __device__ __forceinline__ void set_brg(long long i, int v) const {
    if (brgf) brgf[i] = (unsigned char)v;
  }
};

/* Differences between the p-p law (ContactForceD, kernel.cu:89-228) and the
 * wall law (PWcontactD, kernel.cu:236-359). */
struct LawCfg64 {
  const calParaPP* cal;
  bool hertz_le;   /* p-p: nrm <= ydsp*R; wall: nrm < ydsp*R */
  double rot_eps;  /* 1e-7 (p-p) / 1e-10 (wall): spring rotation guard */
  double dsmx_eps; /* 1e-7 (p-p) / 1e-10 (wall): slip-ratio and rescale guard */
  bool damp_on;    /* p-p: stage == 1; wall: stage == 1 || 7 */
  double dmp;      /* sqrt of the dmpn product (the reference takes it per contact) */
};

/* elasto-plastic Hertz normal force + damping + tangential spring with slip
 * + rolling resistance, FP64, the reference's operand order.
 *
 * The reference's pow(x, 0.5) and pow(x, 2.0) are taken as sqrt(x) and x * x:
 * the correctly rounded square root and product, which is what a correctly
 * rounded pow returns for these exponents (the CPU oracle's glibc pow, within
 * its 0.52-ulp bound; CUDA's pow carries up to 2 ulp); pow(x, 1.5) as pow1_5.
 * The exponent 2/3 (plastic loading only) stays pow.  On
 * GB300 the law is bound by FP64 issue, where each pow is some tens of FP64
 * instructions. */
__device__ __forceinline__ void contact_law64(const LawCfg64& c, double ijRad, double nrm, double3 u,
                                              double3 cpv, HistRec& h, double iRad, double rfrc,
                                              double dt, double3& dF, double3& dM, double& dR) {
  const calParaPP& cal = *c.cal;
  /* pow(ijRad * nrm, 0.5) (twice in the reference's law) and the damping's
   * sqrt(ijRad * nrm): one value */
  const double sq = sqrt(ijRad * nrm);
  double fN = 0.0;
  int st;
  if (nrm < h.plstDfm) st = 1;
  else if (nrm >= h.plstDfm && nrm < h.nDsp) st = 3;
  else if (nrm >= h.nDsp && nrm < h.nDsp_mx) st = 4;
  else st = 2;
  h.stage = st;
  if (st == 1) {
    fN = 0.0;
  } else if (st == 2) {
    bool elastic = c.hertz_le ? (nrm <= cal.ydsp_t * ijRad) : (nrm < (cal.ydsp_t * ijRad));
    if (elastic) {
      fN = 4.0 / 3.0 * cal.emod * sq * nrm;
      h.plstRad = ijRad;
      h.plstDfm = 0.0;
    } else {
      fN = cal.yforce_t * (ijRad * ijRad) + cal.ystiff_t * ijRad * (nrm - cal.ydsp_t * ijRad);
      h.plstRad = ijRad * (4.0 / 3.0 * cal.emod * sq * nrm) / fN;
      h.plstDfm = nrm - pow((fN / (4.0 / 3.0 * cal.emod * sqrt(ijRad))), 2.0 / 3.0);
    }
    h.nDsp_mx = nrm;
  } else {
    fN = 4.0 / 3.0 * cal.emod * sqrt(h.plstRad) * pow1_5(nrm - h.plstDfm);
  }
  h.nDsp = nrm;

  const double vn = dot3(cpv, u);
  double fD = 0.0;
  if (c.damp_on) fD = -2.0 * c.dmp * cal.emod * sq * vn;

  const double3 vt = sub3(cpv, smul3(vn, u));
  const double3 old = h.dispt;
  double3 dT = cross3(smul3(-1.0, u), cross3(u, old));
  if (len3(dT) > c.rot_eps)
    dT = add3(div3(mul3(dT, len3(old)), len3(dT)), mul3(vt, dt));
  else
    dT = add3(dT, mul3(vt, dt));

  const double dsmx = 3.0 * cal.sfrc * fN /
                      (16.0 * (1 - cal.pois) * cal.emod / (4.0 - 2.0 * cal.pois) * sq);
  double ratio = 1.0;
  if (len3(dT) < dsmx) {
    if (dsmx > c.dsmx_eps) ratio = 1.0 - pow1_5(1.0 - len3(dT) / dsmx);
  } else {
    ratio = 1.0;
    if (len3(dT) > c.dsmx_eps) dT = div3(smul3(dsmx, dT), len3(dT));
    else dT = smul3(dsmx, dT);
  }
  h.dispt = dT;

  double3 fT = d3(0.0, 0.0, 0.0);
  if (len3(dT) < dsmx) {
    if (len3(dT) > 1.0e-10) fT = div3(smul3(-1.0 * cal.sfrc * fN * ratio, dT), len3(dT));
  } else {
    if (len3(vt) > 1.0e-10) fT = div3(smul3(-1.0 * cal.sfrc * fN * ratio, vt), len3(vt));
  }
  dF = add3(smul3(fN + fD, u), fT);
  const double arm = iRad - nrm / 2.0;
  dM = cross3(smul3(-arm, u), fT);
  dR = 0.5 * (rfrc + rfrc) * fN * iRad;
}

/* capillary bridge force, kernel.cu:65-81 (the closed-form fit of Willett et
 * al. 2000 at zero contact angle, the reference's coefficients); pow(x, 0.5),
 * pow(x, 2.0) and pow(x, 3.0) as sqrt(x), x * x and cube(x) (contact_law64) */
__device__ __forceinline__ double fcap64(double Splus, double ijVol, double effectR, const LIQUID& L) {
  Splus = max(L.gapmn, Splus);
  Splus = Splus / sqrt(ijVol);
  const double lv = log(ijVol);
  const double lv2 = lv * lv, lv3 = cube(lv);
  const double f1 = -0.44507 - 0.1119 * lv - 0.012101 * lv2 - 0.0005 * lv3;
  const double f2 = 1.9222 - 0.0668 * lv - 0.0013375 * lv2;
  const double f3 = 1.268 + 0.198 * lv + 0.02232 * lv2 + 0.0008585 * lv3;
  const double f4 = -0.010703 + 0.03345 * lv + 0.0018574 * lv2;
  const double ls = log(Splus);
  return 2 * kPiRef * effectR * L.stension * exp(f1 - f2 * exp(f3 * ls + f4 * (ls * ls)));
}

/* warp-aggregated counter increment */
__device__ __forceinline__ void warp_count(unsigned long long* ctr, bool pred) {
  if (!ctr) return;
  const unsigned act = __activemask();
  const unsigned mask = __ballot_sync(act, pred);
  if ((int)(threadIdx.x & 31) == __ffs(act) - 1 && mask) atomicAdd(ctr, (unsigned long long)__popc(mask));
}

}  // namespace dem
