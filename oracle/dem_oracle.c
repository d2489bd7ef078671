/*
 * dem_oracle.c -- CPU oracle for the per-step DEM path (TEST INFRASTRUCTURE).
 *
 * FP64 restatement of the reference heyDEM step in plain C.  Every arithmetic
 * expression keeps the reference's evaluation order (left-to-right sums, the
 * same parenthesisation, the same libm calls) so that, compiled with
 * -ffp-contract=off, it reproduces the reference's own kernels run on the CPU
 * bit for bit.  Used only by tests, smoke() and the CPU-baseline leg of
 * bench.py; never by the product library.
 */
#include "dem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* heydem.h:15 */
#define ORC_PI 3.1415926

/* ---- double3 helpers in the reference's operation order (double_math.h) ---- */
static inline ov3 v3(double x, double y, double z) { ov3 r = {x, y, z}; return r; }
static inline ov3 vadd(ov3 a, ov3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline ov3 vsub(ov3 a, ov3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline ov3 vmul(ov3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline ov3 smul(double s, ov3 a) { return v3(s * a.x, s * a.y, s * a.z); }
static inline ov3 vdiv(ov3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline double vdot(ov3 a, ov3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vlen(ov3 a) { return sqrt(vdot(a, a)); }
static inline ov3 vcross(ov3 a, ov3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

/* ======================= cell hash: kernel.cu:617-673 ======================= */

/* kernel.cu:617-632: cell coordinate, clamped to [0, gridSize] (not gridSize-1) */
static inline oi3 grid_pos(ov3 p, int lvl, o_searchcell cell, const o_consts* k) {
  oi3 g;
  double cs = cell.Cellsize[lvl];
  g.x = imax(0, imin((int)floor((p.x - k->prm.Origin.x) / cs), cell.gridSize[lvl].x));
  g.y = imax(0, imin((int)floor((p.y - k->prm.Origin.y) / cs), cell.gridSize[lvl].y));
  g.z = imax(0, imin((int)floor((p.z - k->prm.Origin.z) / cs), cell.gridSize[lvl].z));
  return g;
}

/* kernel.cu:638-641: z-major linear cell id within a level */
static inline int grid_hash(oi3 g, int lvl, o_searchcell cell) {
  return (g.z * cell.gridSize[lvl].y * cell.gridSize[lvl].x) + (g.y * cell.gridSize[lvl].x) + g.x;
}

/* kernel.cu:646-673 */
void orc_calc_hash(int* hash, int* index, const int* pLevel, o_searchcell cell,
                   const int* Ncell_Idx, const ov3* pos, int n, const o_consts* k) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    int lvl = pLevel[i];
    int h = grid_hash(grid_pos(pos[i], lvl, cell, k), lvl, cell);
    int pre = (lvl != 0) ? Ncell_Idx[lvl - 1] : 0; /* inclusive scan of numCells */
    hash[i] = h + pre;
    index[i] = i;
  }
}

/* ParticleSystem.cu:61-69: sort (hash, index) by hash.  thrust's radix path is
 * stable, so equal hashes keep ascending index; an LSD byte radix sort over the
 * 32-bit key gives exactly that order. */
void orc_sort_by_key(int* hash, int* index, int n) {
  if (n <= 1) return;
  unsigned* k0 = (unsigned*)malloc(sizeof(unsigned) * (size_t)n);
  unsigned* k1 = (unsigned*)malloc(sizeof(unsigned) * (size_t)n);
  int* v0 = (int*)malloc(sizeof(int) * (size_t)n);
  int* v1 = (int*)malloc(sizeof(int) * (size_t)n);
  /* hashes are non-negative ints; flip the sign bit to order signed values too */
  for (int i = 0; i < n; i++) { k0[i] = (unsigned)hash[i] ^ 0x80000000u; v0[i] = index[i]; }
  for (int pass = 0; pass < 4; pass++) {
    int shift = 8 * pass;
    size_t cnt[257];
    memset(cnt, 0, sizeof(cnt));
    for (int i = 0; i < n; i++) cnt[((k0[i] >> shift) & 255u) + 1]++;
    for (int b = 0; b < 256; b++) cnt[b + 1] += cnt[b];
    for (int i = 0; i < n; i++) {
      size_t d = cnt[(k0[i] >> shift) & 255u]++;
      k1[d] = k0[i];
      v1[d] = v0[i];
    }
    unsigned* tk = k0; k0 = k1; k1 = tk;
    int* tv = v0; v0 = v1; v1 = tv;
  }
  for (int i = 0; i < n; i++) { hash[i] = (int)(k0[i] ^ 0x80000000u); index[i] = v0[i]; }
  free(k0); free(k1); free(v0); free(v1);
}

/* ParticleSystem.cu:92-93 (memset 0xff) + kernel.cu:682-724: for each run of
 * equal sorted hashes, start = first position, end = one past the last. */
void orc_find_cell_start(int* cellStart, int* cellEnd, const int* hash, int n, int numCells) {
  memset(cellStart, 0xff, sizeof(int) * (size_t)numCells);
  memset(cellEnd, 0xff, sizeof(int) * (size_t)numCells);
  for (int i = 0; i < n; i++) {
    int h = hash[i];
    if (i == 0 || h != hash[i - 1]) {
      cellStart[h] = i;
      if (i > 0) cellEnd[hash[i - 1]] = i;
    }
    if (i == n - 1) cellEnd[h] = i + 1;
  }
}

/* ===================== neighbour lists: kernel.cu:729-855 ===================== */

int orc_neighbor_find(const ov3* pos, const int* sortedIndex, const int* cellStart,
                      const int* cellEnd, const int* pLevel, o_searchcell cell,
                      const int* Ncell_Idx, const double* Level_size,
                      const int* level_nPars, const int* level_nNebors, int nLevels,
                      int* Nebor1, const int* Nebor_Idx, int* Num_Nebor, int n,
                      const double* rad, const o_consts* k) {
  int overflow = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : overflow)
  for (int i = 0; i < n; i++) {
    ov3 opos = pos[i];
    int iLevel = pLevel[i];
    long base = 0; /* start of this level's slot block (kernel.cu:743-747) */
    for (int l = 0; l < iLevel; l++) base += (long)level_nNebors[l] * level_nPars[l];
    int cap = level_nNebors[iLevel];
    int count = 0, over = 0;
    for (int iL = 0; iL < nLevels; iL++) {
      oi3 g = grid_pos(opos, iL, cell, k);
      int off = (int)ceil(Level_size[iLevel] / Level_size[iL]);
      int cellSum = (iL != 0) ? Ncell_Idx[iL - 1] : 0;
      int gx = cell.gridSize[iL].x, gy = cell.gridSize[iL].y, gz = cell.gridSize[iL].z;
      for (int z = -off; z <= off; z++) {
        for (int y = -off; y <= off; y++) {
          oi3 s = {g.x - off, g.y + y, g.z + z};
          oi3 e = {g.x + off, g.y + y, g.z + z};
          if (s.x < 0) s.x = 0;
          if (e.x > gx - 1) e.x = gx - 1;
          if (s.y < 0 || s.z < 0 || s.y > gy - 1 || s.z > gz - 1) continue;
          /* trim empty cells off both ends of the x-row (kernel.cu:792-815) */
          while (s.x != e.x) {
            if (cellStart[grid_hash(s, iL, cell) + cellSum] == -1) s.x++;
            else break;
          }
          int first = cellStart[grid_hash(s, iL, cell) + cellSum];
          while (s.x != e.x) {
            if (cellEnd[grid_hash(e, iL, cell) + cellSum] == -1) e.x--;
            else break;
          }
          int last = cellEnd[grid_hash(e, iL, cell) + cellSum];
          if (first == -1 || last == -1) continue;
          for (int q = first; q < last; q++) {
            int j = sortedIndex[q];
            if (j == i) continue;
            ov3 d = vsub(opos, pos[j]);
            if (vlen(d) < rad[j] + rad[i] + k->prm.SearchGap) {
              if (count >= cap) { over = 1; continue; }
              Nebor1[base + (long)count * level_nPars[iLevel] + Nebor_Idx[i]] = j;
              count++;
            }
          }
        }
      }
    }
    Num_Nebor[i] = count;
    overflow += over;
  }
  return overflow;
}

/* ===================== wall list: kernel.cu:1034-1073 ===================== */

void orc_wall_list(const ov3* pos, const double* rad, const o_cylinder* cir, int* wlist,
                   int* nwall, int n, const o_consts* k) {
  double sg = k->prm.SearchGap;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    ov3 p = pos[i];
    double r = rad[i];
    int* row = wlist + 3 * (long)i;
    int c = 0;
    if (p.z >= (cir->Tw - (2.0 * r + sg))) row[c++] = 0; /* top */
    if (p.z <= ((2.0 * r + sg) + cir->Bw)) row[c++] = 1; /* bottom */
    double dist = pow(pow((cir->cir_x - p.x), 2.0) + pow((cir->cir_y - p.y), 2.0), 0.5);
    if (dist >= cir->R - (2.0 * r + sg)) row[c++] = 2; /* lateral */
    nwall[i] = c;
  }
}

/* ============ history carry-over: ParticleSystem.cu:336-375, kernel.cu:869-950 ============ */

void orc_history_rotate(o_history old_h, o_history cur_h, long count) {
  memcpy(old_h.dispt, cur_h.dispt, sizeof(ov3) * (size_t)count);
  memcpy(old_h.nDsp, cur_h.nDsp, sizeof(double) * (size_t)count);
  memcpy(old_h.nDsp_mx, cur_h.nDsp_mx, sizeof(double) * (size_t)count);
  memcpy(old_h.plstRad, cur_h.plstRad, sizeof(double) * (size_t)count);
  memcpy(old_h.plstDfm, cur_h.plstDfm, sizeof(double) * (size_t)count);
  memcpy(old_h.stage, cur_h.stage, sizeof(int) * (size_t)count);
  memcpy(old_h.lqdBrg, cur_h.lqdBrg, sizeof(int) * (size_t)count);
  memset(cur_h.dispt, 0, sizeof(ov3) * (size_t)count);
  memset(cur_h.nDsp, 0, sizeof(double) * (size_t)count);
  memset(cur_h.nDsp_mx, 0, sizeof(double) * (size_t)count);
  memset(cur_h.plstRad, 0, sizeof(double) * (size_t)count);
  memset(cur_h.plstDfm, 0, sizeof(double) * (size_t)count);
  memset(cur_h.stage, 0, sizeof(int) * (size_t)count);
  memset(cur_h.lqdBrg, 0, sizeof(int) * (size_t)count);
}

static inline void copy_record(o_history dst, long d, o_history src, long s) {
  dst.dispt[d] = src.dispt[s];
  dst.nDsp[d] = src.nDsp[s];
  dst.nDsp_mx[d] = src.nDsp_mx[s];
  dst.plstRad[d] = src.plstRad[s];
  dst.plstDfm[d] = src.plstDfm[s];
  dst.stage[d] = src.stage[s];
  dst.lqdBrg[d] = src.lqdBrg[s];
}

/* kernel.cu:869-911: a new slot inherits the record of the old slot with the
 * same partner; unmatched slots keep the zeros written by the rotate step. */
void orc_history_carry_pp(const int* Nebor1, const int* Nebor1_Old, const int* pLevel,
                          const int* level_nNebors, const int* level_nPars,
                          const int* Nebor_Idx, o_history old_h, o_history cur_h,
                          const int* Num_Nebor, const int* Num_Nebor_Old, int n) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; i++) {
    int lvl = pLevel[i];
    long base = 0;
    for (int l = 0; l < lvl; l++) base += (long)level_nNebors[l] * level_nPars[l];
    long stride = level_nPars[lvl];
    for (int a = 0; a < Num_Nebor[i]; a++) {
      long ine = base + a * stride + Nebor_Idx[i];
      int partner = Nebor1[ine];
      for (int b = 0; b < Num_Nebor_Old[i]; b++) {
        long jne = base + b * stride + Nebor_Idx[i];
        if (Nebor1_Old[jne] == partner) copy_record(cur_h, ine, old_h, jne);
      }
    }
  }
}

/* kernel.cu:918-950 (wall history slot k of particle i lives at k*NP + i) */
void orc_history_carry_pw(const int* wlist, const int* wlist_old, o_history old_h,
                          o_history cur_h, const int* nwall, const int* nwall_old, int n,
                          int NP) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    for (int a = 0; a < nwall[i]; a++) {
      int w = wlist[3 * (long)i + a];
      for (int b = 0; b < nwall_old[i]; b++) {
        if (wlist_old[3 * (long)i + b] == w)
          copy_record(cur_h, (long)a * NP + i, old_h, (long)b * NP + i);
      }
    }
  }
}

/* Allocation.cpp:308-317 */
void orc_var_init(ov3* force, ov3* mom, double* rmom, int* lqdCnt, int* lqdCnt_Old, int NP) {
  memcpy(lqdCnt_Old, lqdCnt, sizeof(int) * (size_t)NP);
  memset(lqdCnt, 0, sizeof(int) * (size_t)NP);
  memset(force, 0, sizeof(ov3) * (size_t)NP);
  memset(mom, 0, sizeof(ov3) * (size_t)NP);
  memset(rmom, 0, sizeof(double) * (size_t)NP);
}

/* ===================== contact laws ===================== */

/* kernel.cu:65-81: capillary bridge force; the closed-form regression in
 * ln V and ln S+ of Willett, Adams, Johnson and Seville (2000, Langmuir
 * 16:9396) at zero contact angle, with the reference's coefficients. */
double orc_fcap(double Splus, double ijVol, double effectR, const o_consts* k) {
  Splus = k->lqd.gapmn > Splus ? k->lqd.gapmn : Splus; /* max(gapmn, S+) */
  Splus = Splus / pow(ijVol, 0.5);
  double L = log(ijVol);
  double f1 = -0.44507 - 0.1119 * L - 0.012101 * pow(L, 2.0) - 0.0005 * pow(L, 3.0);
  double f2 = 1.9222 - 0.0668 * L - 0.0013375 * pow(L, 2.0);
  double f3 = 1.268 + 0.198 * L + 0.02232 * pow(L, 2.0) + 0.0008585 * pow(L, 3.0);
  double f4 = -0.010703 + 0.03345 * L + 0.0018574 * pow(L, 2.0);
  return 2 * ORC_PI * effectR * k->lqd.stension *
         exp(f1 - f2 * exp(f3 * log(Splus) + f4 * pow(log(Splus), 2.0)));
}

/* ---- the per-contact liquid model (no counterpart in the reference) ----
 * Restates the library's definition: contact angle per particle uniform in
 * [0, theta_max] from a splitmix64 hash of its id and the seed; a pair's
 * bridge volume a fraction uniform in [vol_min, vol_max] (a hash of the two
 * ids, order-free) of the smaller sphere's volume pi/6 (2 r_min)^3 with the
 * reference's pi; the force the same Willett et al. (2000) fit with its
 * contact-angle terms (theta in radians); rupture at (1 + theta/2) 0.99 V^0.33
 * (Lian, Thornton and Adams 1993, on the reference's kernel.cu:518). */
static unsigned long long orc_mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

float orc_theta(int id, unsigned long long seed, float theta_max) {
  const unsigned long long z = orc_mix64(seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(id + 1));
  return theta_max * (float)((double)(z >> 11) * (1.0 / 9007199254740992.0));
}

double orc_pair_volume(const o_consts* k, int ida, int idb, double r_min) {
  const unsigned long long lo = (unsigned long long)(ida < idb ? ida : idb);
  const unsigned long long hi = (unsigned long long)(ida < idb ? idb : ida);
  const unsigned long long z =
      orc_mix64(orc_mix64(k->lqd_seed ^ (0xD1B54A32D192ED03ull * (lo + 1))) + 0x9E3779B97F4A7C15ull * (hi + 1));
  const double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  const double f = k->lqd_vol_min + (k->lqd_vol_max - k->lqd_vol_min) * u;
  const double d = 2.0 * r_min;
  return f * (3.1415926 / 6.0) * (d * d * d);
}

double orc_willett(double s, double v, double t) {
  const double t2 = t * t;
  const double L = log(v), L2 = L * L, L3 = L2 * L;
  const double f1 = (-0.44507 + 0.050832 * t - 1.1466 * t2) + (-0.1119 - 0.000411 * t - 0.1490 * t2) * L +
                    (-0.012101 - 0.0036456 * t - 0.01255 * t2) * L2 +
                    (-0.0005 - 0.0003505 * t - 0.00029076 * t2) * L3;
  const double f2 = (1.9222 - 0.57473 * t - 1.2918 * t2) + (-0.0668 - 0.1201 * t - 0.22574 * t2) * L +
                    (-0.0013375 - 0.0068988 * t - 0.01137 * t2) * L2;
  const double f3 = (1.268 - 0.01396 * t - 0.23566 * t2) + (0.198 + 0.092 * t - 0.06418 * t2) * L +
                    (0.02232 + 0.02238 * t - 0.009853 * t2) * L2 + (0.0008585 + 0.001318 * t - 0.00053 * t2) * L3;
  const double f4 = (-0.010703 + 0.073776 * t - 0.34742 * t2) + (0.03345 + 0.04543 * t - 0.09056 * t2) * L +
                    (0.0018574 + 0.004456 * t - 0.006257 * t2) * L2;
  const double ls = log(s / sqrt(v));
  return exp(f1 - f2 * exp(f3 * ls + f4 * ls * ls));
}

double orc_rupture(double V, double t) { return (1.0 + 0.5 * t) * (0.99 * pow(V, 0.33)); }

/* Shared normal/tangential law of ContactForceD (kernel.cu:89-228) and
 * PWcontactD (kernel.cu:236-359).  The two differ only in: the effective radius,
 * the constant set, "<=" vs "<" on the Hertz/plastic switch, the 1e-7 vs 1e-10
 * threshold in the spring rotation and the slip guard, the damping gate and
 * coefficient, and the contact-velocity expression, all passed in. */
typedef struct {
  const o_calpara* cal;
  int hertz_le;       /* 1: nrm <= ydsp*R (p-p); 0: nrm < ydsp*R (wall) */
  double rot_eps;     /* 1e-7 (p-p) or 1e-10 (wall) */
  double dsmx_eps;    /* 1e-7 (p-p) or 1e-10 (wall) */
  int damp_on;
  double dmp_sq;      /* the argument of the sqrt in the damping coefficient */
} law_cfg;

static void contact_law(const law_cfg* c, double ijRad, double nrm, ov3 unitVec, ov3 ijCPVel,
                        o_history h, long ine, double iRad, double rfrc, double dt,
                        ov3* dF, ov3* dM, double* dR) {
  const o_calpara* cal = c->cal;
  double fN = 0.0;
  /* load / unload / reload stage */
  int st;
  if (nrm < h.plstDfm[ine]) st = 1;
  else if (nrm >= h.plstDfm[ine] && nrm < h.nDsp[ine]) st = 3;
  else if (nrm >= h.nDsp[ine] && nrm < h.nDsp_mx[ine]) st = 4;
  else st = 2;
  h.stage[ine] = st;
  if (st == 1) {
    fN = 0.0;
  } else if (st == 2) {
    int elastic = c->hertz_le ? (nrm <= cal->ydsp_t * ijRad) : (nrm < (cal->ydsp_t * ijRad));
    if (elastic) {
      fN = 4.0 / 3.0 * cal->emod * pow(ijRad * nrm, 0.5) * nrm;
      h.plstRad[ine] = ijRad;
      h.plstDfm[ine] = 0.0;
    } else {
      if (c->hertz_le)
        fN = cal->yforce_t * pow(ijRad, 2.0) + cal->ystiff_t * ijRad * (nrm - cal->ydsp_t * ijRad);
      else
        fN = (cal->yforce_t * pow(ijRad, 2.0)) + (cal->ystiff_t * ijRad) * (nrm - (cal->ydsp_t * ijRad));
      h.plstRad[ine] = ijRad * (4.0 / 3.0 * cal->emod * pow(ijRad * nrm, 0.5) * nrm) / fN;
      h.plstDfm[ine] = nrm - pow((fN / (4.0 / 3.0 * cal->emod * pow(ijRad, 0.5))), 2.0 / 3.0);
    }
    h.nDsp_mx[ine] = nrm;
  } else {
    fN = 4.0 / 3.0 * cal->emod * pow(h.plstRad[ine], 0.5) * pow((nrm - h.plstDfm[ine]), 1.5);
  }
  h.nDsp[ine] = nrm;

  /* normal damping */
  double vn = vdot(ijCPVel, unitVec);
  double fD = 0.0;
  if (c->damp_on) fD = -2.0 * sqrt(c->dmp_sq) * cal->emod * sqrt(ijRad * nrm) * vn;

  /* tangential spring: rotate into the new tangent plane keeping its length,
   * then add v_t dt */
  ov3 vt = vsub(ijCPVel, smul(vn, unitVec));
  ov3 old = h.dispt[ine];
  ov3 dT = vcross(smul(-1.0, unitVec), vcross(unitVec, old));
  if (vlen(dT) > c->rot_eps)
    dT = vadd(vdiv(vmul(dT, vlen(old)), vlen(dT)), vmul(vt, dt));
  else
    dT = vadd(dT, vmul(vt, dt));

  double dsmx = 3.0 * cal->sfrc * fN /
                (16.0 * (1 - cal->pois) * cal->emod / (4.0 - 2.0 * cal->pois) * pow(ijRad * nrm, 0.5));
  double ratio = 1.0;
  if (vlen(dT) < dsmx) {
    if (dsmx > c->dsmx_eps) ratio = 1.0 - pow((1.0 - vlen(dT) / dsmx), 1.5);
  } else {
    ratio = 1.0;
    if (vlen(dT) > c->dsmx_eps) dT = vdiv(smul(dsmx, dT), vlen(dT));
    else dT = smul(dsmx, dT);
  }
  h.dispt[ine] = dT;

  ov3 fT = v3(0.0, 0.0, 0.0);
  if (vlen(dT) < dsmx) {
    if (vlen(dT) > 1.0e-10) fT = vdiv(smul(-1.0 * cal->sfrc * fN * ratio, dT), vlen(dT));
  } else {
    if (vlen(vt) > 1.0e-10) fT = vdiv(smul(-1.0 * cal->sfrc * fN * ratio, vt), vlen(vt));
  }

  *dF = vadd(smul(fN + fD, unitVec), fT);
  double arm = iRad - nrm / 2.0;
  *dM = vcross(smul(-arm, unitVec), fT);
  *dR = 0.5 * (rfrc + rfrc) * fN * iRad;
}

/* ===================== p-p forces: kernel.cu:413-552 ===================== */

void orc_pp_force(const ov3* pos, const ov3* vel, const ov3* angvel, const double* rad,
                  const int* Nebor1, const int* pLevel, const int* level_nNebors,
                  const int* level_nPars, const int* Nebor_Idx, o_history h,
                  const int* Num_Nebor, int* lqdCnt, const int* lqdCnt_Old, ov3* force,
                  ov3* mom, double* rmom, int n, int NP, int ForceCap, int stage,
                  const o_consts* k) {
  (void)NP;
  law_cfg cfg;
  cfg.cal = &k->cal;
  cfg.hertz_le = 1;
  cfg.rot_eps = 1.0e-7;
  cfg.dsmx_eps = 1.0e-7;
  cfg.damp_on = (stage == 1);
  cfg.dmp_sq = k->mat[0].dmpn * k->mat[0].dmpn;
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; i++) {
    ov3 ip = pos[i], iv = vel[i], iw = angvel[i];
    double ir = rad[i];
    int inl = lqdCnt_Old[i];
    if (inl < 12) inl = 12;
    double iVol = k->lqd.vol * pow((rad[i] * 2), 3.0) / inl;
    force[i].z = force[i].z - pow(2.0 * rad[i], 3.0); /* gravity, m = (2r)^3 */
    int lvl = pLevel[i];
    long base = 0;
    for (int l = 0; l < lvl; l++) base += (long)level_nNebors[l] * level_nPars[l];
    for (int a = 0; a < Num_Nebor[i]; a++) {
      long ine = base + (long)a * level_nPars[lvl] + Nebor_Idx[i];
      int j = Nebor1[ine];
      ov3 jp = pos[j];
      double jr = rad[j];
      ov3 d = vsub(ip, jp);
      ov3 u = vdiv(d, vlen(d));
      double gap = vlen(d) - ir - jr;
      if (gap < 0.0) {
        ov3 jv = vel[j], jw = angvel[j];
        ov3 cpv = vsub(vsub(iv, jv), vcross(vadd(vmul(iw, ir), vmul(jw, jr)), u));
        double ijRad = ir * jr / (ir + jr);
        ov3 dF, dM;
        double dR;
        contact_law(&cfg, ijRad, -gap, u, cpv, h, ine, ir, k->mat[0].rfrc, k->prm.dt, &dF, &dM, &dR);
        force[i] = vadd(force[i], dF);
        mom[i] = vadd(mom[i], dM);
        rmom[i] = rmom[i] + dR;
      }
      if (ForceCap == 1 && k->lqd_mode == 1) {
        /* the per-contact liquid model (particle index = caller id here) */
        double th = 0.5 * ((double)orc_theta(i, k->lqd_seed, k->lqd_theta_max) +
                           (double)orc_theta(j, k->lqd_seed, k->lqd_theta_max));
        double V = orc_pair_volume(k, i, j, ir < jr ? ir : jr);
        if (gap < 2 * k->lqd.layer * (ir + jr)) h.lqdBrg[ine] = 1;
        else if (gap > orc_rupture(V, th)) h.lqdBrg[ine] = 0;
        if (h.lqdBrg[ine] == 1) {
          double Splus = (gap < 0) ? 0.0 : gap;
          double effR = 2 * ir * jr / (ir + jr);
          double fcap = 2 * ORC_PI * effR * k->lqd.stension *
                        orc_willett(k->lqd.gapmn > Splus ? k->lqd.gapmn : Splus, 8.0 * V, th);
          force[i] = vadd(force[i], smul(-1.0 * fcap, u));
          lqdCnt[i] = lqdCnt[i] + 1;
        }
      } else if (ForceCap == 1) {
        int jnl = lqdCnt_Old[j];
        if (jnl < 12) jnl = 12;
        double jVol = k->lqd.vol * pow((jr * 2), 3.0) / jnl;
        double ijVol = iVol + jVol;
        double rupture = 0.99 * pow(ijVol, 0.33);
        if (gap < 2 * k->lqd.layer * (ir + jr)) h.lqdBrg[ine] = 1;
        else if (gap > rupture) h.lqdBrg[ine] = 0;
        double Splus = (gap < 0) ? 0.0 : gap;
        if (h.lqdBrg[ine] == 1) {
          double effR = 2 * ir * jr / (ir + jr);
          ijVol = ijVol * 8.0;
          ov3 fc = smul(-1.0 * orc_fcap(Splus, ijVol, effR, k), u);
          force[i] = vadd(force[i], fc);
          lqdCnt[i] = lqdCnt[i] + 1;
        }
      }
    }
  }
}

/* ===================== wall forces: kernel.cu:958-1023 ===================== */

void orc_wall_force(const ov3* pos, const ov3* vel, const ov3* angvel, ov3* force, ov3* mom,
                    double* rmom, const double* rad, o_cylinder* cir, o_history h,
                    const int* nwall, const int* wlist, int n, int NP, int stage,
                    const o_consts* k) {
  /* kernel.cu:966-969: particle 0's thread moves the top wall.  Done once,
   * before any particle reads Tw (the reference races here; with topv = 0 the
   * two orders agree). */
  if (n > 0) cir->Tw = cir->Tw + cir->topv * k->prm.dt;
  law_cfg cfg;
  cfg.cal = &k->pwcal;
  cfg.hertz_le = 0;
  cfg.rot_eps = 1.0e-10;
  cfg.dsmx_eps = 1.0e-10;
  cfg.damp_on = (stage == 1 || stage == 7);
  cfg.dmp_sq = k->mat[0].dmpn * k->mat[1].dmpn;
  const o_cylinder c = *cir;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    ov3 ip = pos[i], iv = vel[i], iw = angvel[i];
    double ir = rad[i];
    ov3 jp = v3(0.0, 0.0, 0.0);
    ov3 jv = v3(0.0, 0.0, 0.0); /* persists across walls, as in kernel.cu:980 */
    for (int a = 0; a < nwall[i]; a++) {
      int w = wlist[3 * (long)i + a];
      if (w == 0) {
        jp = v3(ip.x, ip.y, c.Tw);
        jv = v3(0.0, 0.0, c.topv);
      } else if (w == 1) {
        jp = v3(ip.x, ip.y, c.Bw);
      } else if (w == 2) {
        double dist = pow(pow((c.cir_x - ip.x), 2.0) + pow((c.cir_y - ip.y), 2.0), 0.5);
        double cs = (ip.x - c.cir_x) / dist;
        double sn = (ip.y - c.cir_y) / dist;
        jp.x = c.R * cs + c.cir_x;
        jp.y = c.R * sn + c.cir_y;
        jp.z = ip.z;
      } else {
        continue;
      }
      /* kernel.cu:370-403 MultiPWForceD */
      ov3 d = vsub(ip, jp);
      ov3 u = vdiv(d, vlen(d));
      double gap = vlen(d) - ir;
      if (gap < 0.0) {
        ov3 cpv = vsub(vsub(iv, jv), vcross(vmul(iw, ir), u));
        ov3 dF, dM;
        double dR;
        contact_law(&cfg, ir, -gap, u, cpv, h, (long)a * NP + i, ir, k->mat[0].rfrc, k->prm.dt,
                    &dF, &dM, &dR);
        force[i] = vadd(force[i], dF);
        mom[i] = vadd(mom[i], dM);
        rmom[i] = rmom[i] + dR;
      }
    }
  }
}

/* ===================== integrator: kernel.cu:563-606 ===================== */

int orc_update(const double* rad, ov3* pos, ov3* vel, ov3* angvel, const ov3* force,
               const ov3* mom, double* rmom, double* pMove, int n, const o_consts* k) {
  int flagged = 0;
  double dt = k->prm.dt;
#pragma omp parallel for schedule(static) reduction(+ : flagged)
  for (int i = 0; i < n; i++) {
    double mass = pow(2.0 * rad[i], 3.0);
    vel[i].x = vel[i].x + force[i].x * dt / mass;
    vel[i].y = vel[i].y + force[i].y * dt / mass;
    vel[i].z = vel[i].z + force[i].z * dt / mass;
    pos[i] = vadd(pos[i], vmul(vel[i], dt));
    pMove[i] = pMove[i] + vlen(vel[i]) * k->prm.dt;
    double inert = 0.1 * pow(2.0 * rad[i], 5.0);
    angvel[i].x = angvel[i].x + mom[i].x * dt / inert;
    angvel[i].y = angvel[i].y + mom[i].y * dt / inert;
    angvel[i].z = angvel[i].z + mom[i].z * dt / inert;
    rmom[i] = rmom[i] * dt / inert;
    double wl = vlen(angvel[i]);
    if (wl > 1.0e-7) {
      double s = rmom[i] / wl;
      angvel[i] = vmul(angvel[i], (1.0 - ((s < 1.0) ? s : 1.0))); /* std::min(1.0, s) */
    }
    if (pMove[i] > (0.3 * k->prm.SearchGap)) flagged += 1;
  }
  return flagged;
}

/* ===================== whole simulation: main.cpp:433-568 ===================== */

struct orc_sim {
  int NP, nLevels, Sys_nCells;
  long nPPCnt;
  int ForceCap, stage;
  long iter, rebuilds;
  int need_build, flag, last_overflow;
  orc_kernels kern;
  o_consts k;
  o_cylinder cir;
  ov3 *pos, *vel, *angvel, *force, *mom;
  double *rmom, *rad, *pMove;
  int *lqdCnt, *lqdCnt_Old, *pLevel, *Nebor_Idx;
  double* Level_size;
  int *level_nNebors, *level_nPars, *Ncell_Idx, *numCells;
  oi3* gridSize;
  double* Cellsize;
  int *hash, *index, *cellStart, *cellEnd;
  int *Nebor1, *Nebor1_Old, *Num_Nebor, *Num_Nebor_Old;
  int *wlist, *wlist_old, *nwall, *nwall_old;
  o_history pp, pp_old, pw, pw_old;
};

static void* zalloc(size_t n) { return calloc(n ? n : 1, 1); }

static void history_alloc(o_history* h, long n) {
  h->dispt = (ov3*)zalloc(sizeof(ov3) * (size_t)n);
  h->nDsp = (double*)zalloc(sizeof(double) * (size_t)n);
  h->nDsp_mx = (double*)zalloc(sizeof(double) * (size_t)n);
  h->plstRad = (double*)zalloc(sizeof(double) * (size_t)n);
  h->plstDfm = (double*)zalloc(sizeof(double) * (size_t)n);
  h->stage = (int*)zalloc(sizeof(int) * (size_t)n);
  h->lqdBrg = (int*)zalloc(sizeof(int) * (size_t)n);
}
static void history_free(o_history* h) {
  free(h->dispt); free(h->nDsp); free(h->nDsp_mx); free(h->plstRad); free(h->plstDfm);
  free(h->stage); free(h->lqdBrg);
}

static const orc_kernels g_default_kernels = {
    orc_calc_hash, orc_find_cell_start, orc_neighbor_find, orc_wall_list,
    orc_history_carry_pp, orc_history_carry_pw, orc_pp_force, orc_wall_force, orc_update};

const orc_kernels* orc_default_kernels(void) { return &g_default_kernels; }

orc_sim* orc_sim_new(int NP, int nLevels, int Sys_nCells, long nPPCnt) {
  orc_sim* s = (orc_sim*)zalloc(sizeof(orc_sim));
  s->NP = NP; s->nLevels = nLevels; s->Sys_nCells = Sys_nCells; s->nPPCnt = nPPCnt;
  s->stage = 1;
  s->need_build = 1;
  s->kern = g_default_kernels;
  size_t N = (size_t)NP, L = (size_t)nLevels;
  s->pos = (ov3*)zalloc(sizeof(ov3) * N); s->vel = (ov3*)zalloc(sizeof(ov3) * N);
  s->angvel = (ov3*)zalloc(sizeof(ov3) * N); s->force = (ov3*)zalloc(sizeof(ov3) * N);
  s->mom = (ov3*)zalloc(sizeof(ov3) * N);
  s->rmom = (double*)zalloc(sizeof(double) * N); s->rad = (double*)zalloc(sizeof(double) * N);
  s->pMove = (double*)zalloc(sizeof(double) * N);
  s->lqdCnt = (int*)zalloc(sizeof(int) * N); s->lqdCnt_Old = (int*)zalloc(sizeof(int) * N);
  s->pLevel = (int*)zalloc(sizeof(int) * N); s->Nebor_Idx = (int*)zalloc(sizeof(int) * N);
  s->Level_size = (double*)zalloc(sizeof(double) * L);
  s->level_nNebors = (int*)zalloc(sizeof(int) * L); s->level_nPars = (int*)zalloc(sizeof(int) * L);
  s->Ncell_Idx = (int*)zalloc(sizeof(int) * L); s->numCells = (int*)zalloc(sizeof(int) * L);
  s->gridSize = (oi3*)zalloc(sizeof(oi3) * L); s->Cellsize = (double*)zalloc(sizeof(double) * L);
  s->hash = (int*)zalloc(sizeof(int) * N); s->index = (int*)zalloc(sizeof(int) * N);
  s->cellStart = (int*)zalloc(sizeof(int) * (size_t)Sys_nCells);
  s->cellEnd = (int*)zalloc(sizeof(int) * (size_t)Sys_nCells);
  s->Nebor1 = (int*)zalloc(sizeof(int) * (size_t)nPPCnt);
  s->Nebor1_Old = (int*)zalloc(sizeof(int) * (size_t)nPPCnt);
  s->Num_Nebor = (int*)zalloc(sizeof(int) * N); s->Num_Nebor_Old = (int*)zalloc(sizeof(int) * N);
  s->wlist = (int*)zalloc(sizeof(int) * 3 * N); s->wlist_old = (int*)zalloc(sizeof(int) * 3 * N);
  s->nwall = (int*)zalloc(sizeof(int) * N); s->nwall_old = (int*)zalloc(sizeof(int) * N);
  history_alloc(&s->pp, nPPCnt); history_alloc(&s->pp_old, nPPCnt);
  history_alloc(&s->pw, 3 * (long)NP); history_alloc(&s->pw_old, 3 * (long)NP);
  return s;
}

void orc_sim_free(orc_sim* s) {
  if (!s) return;
  free(s->pos); free(s->vel); free(s->angvel); free(s->force); free(s->mom);
  free(s->rmom); free(s->rad); free(s->pMove); free(s->lqdCnt); free(s->lqdCnt_Old);
  free(s->pLevel); free(s->Nebor_Idx); free(s->Level_size); free(s->level_nNebors);
  free(s->level_nPars); free(s->Ncell_Idx); free(s->numCells); free(s->gridSize);
  free(s->Cellsize); free(s->hash); free(s->index); free(s->cellStart); free(s->cellEnd);
  free(s->Nebor1); free(s->Nebor1_Old); free(s->Num_Nebor); free(s->Num_Nebor_Old);
  free(s->wlist); free(s->wlist_old); free(s->nwall); free(s->nwall_old);
  history_free(&s->pp); history_free(&s->pp_old); history_free(&s->pw); history_free(&s->pw_old);
  free(s);
}

static void* history_field(o_history* h, const char* f) {
  if (!strcmp(f, "dispt")) return h->dispt;
  if (!strcmp(f, "nDsp")) return h->nDsp;
  if (!strcmp(f, "nDsp_mx")) return h->nDsp_mx;
  if (!strcmp(f, "plstRad")) return h->plstRad;
  if (!strcmp(f, "plstDfm")) return h->plstDfm;
  if (!strcmp(f, "stage")) return h->stage;
  if (!strcmp(f, "lqdBrg")) return h->lqdBrg;
  return NULL;
}

void* orc_sim_ptr(orc_sim* s, const char* name) {
#define NAMED(f) if (!strcmp(name, #f)) return (void*)s->f
  NAMED(pos); NAMED(vel); NAMED(angvel); NAMED(force); NAMED(mom); NAMED(rmom); NAMED(rad);
  NAMED(pMove); NAMED(lqdCnt); NAMED(lqdCnt_Old); NAMED(pLevel); NAMED(Nebor_Idx);
  NAMED(Level_size); NAMED(level_nNebors); NAMED(level_nPars); NAMED(Ncell_Idx);
  NAMED(numCells); NAMED(gridSize); NAMED(Cellsize); NAMED(hash); NAMED(index);
  NAMED(cellStart); NAMED(cellEnd); NAMED(Nebor1); NAMED(Nebor1_Old); NAMED(Num_Nebor);
  NAMED(Num_Nebor_Old); NAMED(wlist); NAMED(wlist_old); NAMED(nwall); NAMED(nwall_old);
#undef NAMED
  if (!strcmp(name, "consts")) return &s->k;
  if (!strcmp(name, "cylinder")) return &s->cir;
  if (!strncmp(name, "pp.", 3)) return history_field(&s->pp, name + 3);
  if (!strncmp(name, "pp_old.", 7)) return history_field(&s->pp_old, name + 7);
  if (!strncmp(name, "pw.", 3)) return history_field(&s->pw, name + 3);
  if (!strncmp(name, "pw_old.", 7)) return history_field(&s->pw_old, name + 7);
  return NULL;
}

void orc_sim_set_mode(orc_sim* s, int ForceCap, int stage) { s->ForceCap = ForceCap; s->stage = stage; }
void orc_sim_set_kernels(orc_sim* s, const orc_kernels* t) { s->kern = *t; }
void orc_sim_request_rebuild(orc_sim* s) { s->need_build = 1; }

void orc_sim_set_counter(orc_sim* s, const char* name, long v) {
  if (!strcmp(name, "iter")) s->iter = v;
  else if (!strcmp(name, "flag")) s->flag = (int)v;
  else if (!strcmp(name, "need_build")) s->need_build = (int)v;
}

long orc_sim_counter(orc_sim* s, const char* name) {
  if (!strcmp(name, "iter")) return s->iter;
  if (!strcmp(name, "rebuilds")) return s->rebuilds;
  if (!strcmp(name, "flag")) return s->flag;
  if (!strcmp(name, "overflow")) return s->last_overflow;
  return -1;
}

static o_searchcell sim_cell(orc_sim* s) {
  o_searchcell c;
  c.numCells = s->numCells; c.gridSize = s->gridSize; c.Cellsize = s->Cellsize;
  return c;
}

int orc_sim_step(orc_sim* s) {
  int n = s->NP, rebuilt = 0;
  const o_consts* k = &s->k;
  /* main.cpp:470-527: rebuild when the previous integration flagged it (or on
   * the first step / an explicit request) */
  if (s->flag > 0 || s->need_build) {
    int carry = (s->iter != 0); /* main.cpp:476, :507 */
    if (carry) {
      memcpy(s->Num_Nebor_Old, s->Num_Nebor, sizeof(int) * (size_t)n);
      memcpy(s->Nebor1_Old, s->Nebor1, sizeof(int) * (size_t)s->nPPCnt);
      orc_history_rotate(s->pp_old, s->pp, s->nPPCnt);
      memcpy(s->nwall_old, s->nwall, sizeof(int) * (size_t)n);
      memcpy(s->wlist_old, s->wlist, sizeof(int) * 3 * (size_t)n);
      orc_history_rotate(s->pw_old, s->pw, 3 * (long)n);
    }
    memset(s->pMove, 0, sizeof(double) * (size_t)n);
    o_searchcell c = sim_cell(s);
    s->kern.calc_hash(s->hash, s->index, s->pLevel, c, s->Ncell_Idx, s->pos, n, k);
    orc_sort_by_key(s->hash, s->index, n);
    s->kern.find_cell_start(s->cellStart, s->cellEnd, s->hash, n, s->Sys_nCells);
    s->last_overflow = s->kern.neighbor_find(s->pos, s->index, s->cellStart, s->cellEnd,
                                             s->pLevel, c, s->Ncell_Idx, s->Level_size,
                                             s->level_nPars, s->level_nNebors, s->nLevels,
                                             s->Nebor1, s->Nebor_Idx, s->Num_Nebor, n, s->rad, k);
    s->kern.wall_list(s->pos, s->rad, &s->cir, s->wlist, s->nwall, n, k);
    if (carry) {
      s->kern.carry_pp(s->Nebor1, s->Nebor1_Old, s->pLevel, s->level_nNebors, s->level_nPars,
                       s->Nebor_Idx, s->pp_old, s->pp, s->Num_Nebor, s->Num_Nebor_Old, n);
      s->kern.carry_pw(s->wlist, s->wlist_old, s->pw_old, s->pw, s->nwall, s->nwall_old, n, n);
    }
    s->need_build = 0;
    s->rebuilds++;
    rebuilt = 1;
  }
  /* main.cpp:536-558 */
  orc_var_init(s->force, s->mom, s->rmom, s->lqdCnt, s->lqdCnt_Old, n);
  s->kern.pp_force(s->pos, s->vel, s->angvel, s->rad, s->Nebor1, s->pLevel, s->level_nNebors,
                   s->level_nPars, s->Nebor_Idx, s->pp, s->Num_Nebor, s->lqdCnt, s->lqdCnt_Old,
                   s->force, s->mom, s->rmom, n, n, s->ForceCap, s->stage, k);
  s->kern.wall_force(s->pos, s->vel, s->angvel, s->force, s->mom, s->rmom, s->rad, &s->cir,
                     s->pw, s->nwall, s->wlist, n, n, s->stage, k);
  s->flag = s->kern.update(s->rad, s->pos, s->vel, s->angvel, s->force, s->mom, s->rmom,
                           s->pMove, n, k);
  s->iter++;
  if (s->last_overflow) return -1;
  return rebuilt;
}
