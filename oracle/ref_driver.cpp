/*
 * ref_driver.cpp -- runs the reference's own kernels on the CPU (TEST INFRASTRUCTURE).
 *
 * Built by oracle/build_ref.sh together with the reference's kernel.cu,
 * ReadData.cpp, UnitReduce.cpp, DiaInput.cpp, DumpLoad.cpp and WriteTec.cpp
 * (compiled in place from the reference tree through oracle/ref_shim/) into
 * oracle/_ref/libdem_ref.so.  It exposes the reference kernels through the
 * oracle's kernel table (orc_kernels), so tests can drive the reference and the
 * oracle restatement with identical inputs and demand identical outputs.
 *
 * Each __global__ kernel is a host function here; the driver calls it once per
 * linear thread index with the launch geometry the reference's wrappers use
 * (ParticleSystem.cu:45-289).
 */
#include "heydem.h"  // the reference's header, through the shim

extern "C" {
#include "dem_oracle.h"
}

#include <vector>

thread_local uint3 threadIdx;
thread_local uint3 blockIdx;
thread_local dim3 blockDim;
thread_local dim3 gridDim;
/* kernel.cu:688 `extern __shared__ int sharedHash[]` (block-serial here) */
thread_local int sharedHash[1025];

/* constant memory of kernel.cu:15-19 */
extern MatType d_Mat[NUM_MAT];
extern LIQUID d_lqd;
extern PARAMETER d_Params;
extern calParaPP d_cal;
extern calParaPP d_pWcal;

static_assert(sizeof(o_cylinder) == sizeof(CylinderBC), "CylinderBC layout");
static_assert(sizeof(o_parameter) == sizeof(PARAMETER), "PARAMETER layout");
static_assert(sizeof(o_mat) == sizeof(MatType), "MatType layout");
static_assert(sizeof(o_liquid) == sizeof(LIQUID), "LIQUID layout");
static_assert(sizeof(o_calpara) == sizeof(calParaPP), "calParaPP layout");
static_assert(sizeof(ov3) == sizeof(double3), "double3 layout");
static_assert(sizeof(oi3) == sizeof(int3), "int3 layout");

static void load_consts(const o_consts* k) {
  std::memcpy(d_Mat, k->mat, sizeof(d_Mat));
  std::memcpy(&d_lqd, &k->lqd, sizeof(d_lqd));
  std::memcpy(&d_Params, &k->prm, sizeof(d_Params));
  std::memcpy(&d_cal, &k->cal, sizeof(d_cal));
  std::memcpy(&d_pWcal, &k->pwcal, sizeof(d_pWcal));
}

static inline void set_thread(int idx, int block) {
  blockDim = dim3(block, 1, 1);
  blockIdx = make_uint3(idx / block, 0, 0);
  threadIdx = make_uint3(idx % block, 0, 0);
}

static SEARCHCELL to_cell(o_searchcell c) {
  SEARCHCELL s;
  s.numCells = c.numCells;
  s.gridSize = reinterpret_cast<int3*>(c.gridSize);
  s.Cellsize = c.Cellsize;
  return s;
}

static PPCONTACT_HISTORY to_pp(o_history h) {
  PPCONTACT_HISTORY r;
  std::memset(&r, 0, sizeof(r));
  r.dispt = reinterpret_cast<double3*>(h.dispt);
  r.nDsp = h.nDsp; r.nDsp_mx = h.nDsp_mx; r.plstRad = h.plstRad; r.plstDfm = h.plstDfm;
  r.stage = h.stage; r.lqdBrg = h.lqdBrg;
  return r;
}

static PWCONTACT_HISTORY to_pw(o_history h) {
  PWCONTACT_HISTORY r;
  r.dispt = reinterpret_cast<double3*>(h.dispt);
  r.nDsp = h.nDsp; r.nDsp_mx = h.nDsp_mx; r.plstRad = h.plstRad; r.plstDfm = h.plstDfm;
  r.stage = h.stage; r.lqdBrg = h.lqdBrg;
  return r;
}

#define DV3(p) reinterpret_cast<double3*>(const_cast<ov3*>(p))
#define IP(p) const_cast<int*>(p)
#define DP(p) const_cast<double*>(p)

static void k_calc_hash(int* hash, int* index, const int* pLevel, o_searchcell cell,
                        const int* Ncell_Idx, const ov3* pos, int n, const o_consts* k) {
  load_consts(k);
  SEARCHCELL c = to_cell(cell);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    set_thread(i, 32);
    calcHashG(hash, index, IP(pLevel), c, IP(Ncell_Idx), DV3(pos), n);
  }
}

static void k_find_cell_start(int* cellStart, int* cellEnd, const int* hash, int n, int numCells) {
  /* ParticleSystem.cu:83-103: memset to 0xff, then the smem-halo kernel,
   * executed block by block with threads in order */
  std::memset(cellStart, 0xff, sizeof(int) * (size_t)numCells);
  std::memset(cellEnd, 0xff, sizeof(int) * (size_t)numCells);
  int block = n < 64 ? n : 64;
  if (block <= 0) return;
  int nb = (n + block - 1) / block;
  std::vector<int> idx(1, 0);
  for (int b = 0; b < nb; b++) {
    for (int t = 0; t < block; t++) {  // phase 1 and 2 interleave correctly in order
      set_thread(b * block + t, block);
      reorderDataAndFindCellStartG(cellStart, cellEnd, IP(hash), idx.data(), n);
    }
  }
}

static int k_neighbor_find(const ov3* pos, const int* sortedIndex, const int* cellStart,
                           const int* cellEnd, const int* pLevel, o_searchcell cell,
                           const int* Ncell_Idx, const double* Level_size,
                           const int* level_nPars, const int* level_nNebors, int nLevels,
                           int* Nebor1, const int* Nebor_Idx, int* Num_Nebor, int n,
                           const double* rad, const o_consts* k) {
  load_consts(k);
  SEARCHCELL c = to_cell(cell);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; i++) {
    set_thread(i, 128);
    NeighborFindG(DV3(pos), IP(sortedIndex), IP(cellStart), IP(cellEnd), IP(pLevel), c,
                  IP(Ncell_Idx), DP(Level_size), IP(level_nPars), IP(level_nNebors), nLevels,
                  Nebor1, IP(Nebor_Idx), Num_Nebor, n, DP(rad));
  }
  /* the reference has no capacity check; report lists that overran */
  int over = 0;
  for (int i = 0; i < n; i++)
    if (Num_Nebor[i] > level_nNebors[pLevel[i]]) over++;
  return over;
}

static void k_wall_list(const ov3* pos, const double* rad, const o_cylinder* cir, int* wlist,
                        int* nwall, int n, const o_consts* k) {
  load_consts(k);
  CylinderBC c;
  std::memcpy(&c, cir, sizeof(c));
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    set_thread(i, 128);
    CirWallListG(DV3(pos), DP(rad), &c, wlist, 3 * sizeof(int), nwall, n);
  }
}

static void k_carry_pp(const int* Nebor1, const int* Nebor1_Old, const int* pLevel,
                       const int* level_nNebors, const int* level_nPars, const int* Nebor_Idx,
                       o_history old_h, o_history cur_h, const int* Num_Nebor,
                       const int* Num_Nebor_Old, int n) {
  PPCONTACT_HISTORY o = to_pp(old_h), c = to_pp(cur_h);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; i++) {
    set_thread(i, 256);
    HstryCopyG(IP(Nebor1), IP(Nebor1_Old), IP(pLevel), IP(level_nNebors), IP(level_nPars),
               IP(Nebor_Idx), o, c, IP(Num_Nebor), IP(Num_Nebor_Old), n, n);
  }
}

static void k_carry_pw(const int* wlist, const int* wlist_old, o_history old_h, o_history cur_h,
                       const int* nwall, const int* nwall_old, int n, int NP) {
  PWCONTACT_HISTORY o = to_pw(old_h), c = to_pw(cur_h);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    set_thread(i, 128);
    HstryCopyPWG(IP(wlist), IP(wlist_old), 3 * sizeof(int), 3 * sizeof(int), o, c, IP(nwall),
                 IP(nwall_old), n, NP);
  }
}

static void k_pp_force(const ov3* pos, const ov3* vel, const ov3* angvel, const double* rad,
                       const int* Nebor1, const int* pLevel, const int* level_nNebors,
                       const int* level_nPars, const int* Nebor_Idx, o_history h,
                       const int* Num_Nebor, int* lqdCnt, const int* lqdCnt_Old, ov3* force,
                       ov3* mom, double* rmom, int n, int NP, int ForceCap, int stage,
                       const o_consts* k) {
  load_consts(k);
  PPCONTACT_HISTORY hh = to_pp(h);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; i++) {
    set_thread(i, threadsPerBlock);
    PPForceCalcG(DV3(pos), DV3(vel), DV3(angvel), DP(rad), IP(Nebor1), IP(pLevel),
                 IP(level_nNebors), IP(level_nPars), IP(Nebor_Idx), hh, IP(Num_Nebor), lqdCnt,
                 IP(lqdCnt_Old), DV3(force), DV3(mom), rmom, n, NP, ForceCap, stage);
  }
}

static void k_wall_force(const ov3* pos, const ov3* vel, const ov3* angvel, ov3* force,
                         ov3* mom, double* rmom, const double* rad, o_cylinder* cir,
                         o_history h, const int* nwall, const int* wlist, int n, int NP,
                         int stage, const o_consts* k) {
  load_consts(k);
  PWCONTACT_HISTORY hh = to_pw(h);
  CylinderBC* c = reinterpret_cast<CylinderBC*>(cir);
  if (n <= 0) return;
  /* index 0 moves the top wall; run it first so every reader sees one value */
  set_thread(0, threadsPerBlock);
  CirPWInterG(DV3(pos), DV3(vel), DV3(angvel), DV3(force), DV3(mom), rmom, DP(rad), c, hh,
              IP(nwall), IP(wlist), 3 * sizeof(int), n, NP, stage);
#pragma omp parallel for schedule(static)
  for (int i = 1; i < n; i++) {
    set_thread(i, threadsPerBlock);
    CirPWInterG(DV3(pos), DV3(vel), DV3(angvel), DV3(force), DV3(mom), rmom, DP(rad), c, hh,
                IP(nwall), IP(wlist), 3 * sizeof(int), n, NP, stage);
  }
}

static int k_update(const double* rad, ov3* pos, ov3* vel, ov3* angvel, const ov3* force,
                    const ov3* mom, double* rmom, double* pMove, int n, const o_consts* k) {
  load_consts(k);
  int flag = 0;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    set_thread(i, 256);
    UpdateSystemG(DP(rad), DV3(pos), DV3(vel), DV3(angvel), DV3(force), DV3(mom), rmom, &flag,
                  pMove, n);
  }
  return flag;
}

static const orc_kernels g_ref_kernels = {k_calc_hash, k_find_cell_start, k_neighbor_find,
                                          k_wall_list, k_carry_pp,        k_carry_pw,
                                          k_pp_force,  k_wall_force,      k_update};

extern "C" const orc_kernels* ref_kernels(void) { return &g_ref_kernels; }

/* kernel.cu:65-81 through a one-particle constant load */
extern __device__ double fCap(double Splus, double ijVol, double effectR);
extern "C" double ref_fcap(double Splus, double ijVol, double effectR, const o_consts* k) {
  load_consts(k);
  return fCap(Splus, ijVol, effectR);
}

/* ReadData.cpp:41 + UnitReduce.cpp:6 in main.cpp's order (:227, :312), for the
 * host set-up parity test.  Runs in the current directory (reads
 * <genfile>.in, optional <genfile>_dia.dat; appends <genfile>_Log.dat). */
extern "C" int ref_read_setup(const char* genfile, int NP, int nLevels, double* Level_size,
                              int* pLevel, int* level_nNebors, int* level_nPars,
                              int* Nebor_Idx, o_cylinder* cir, double* feed /*[2] Lmin Lmax*/,
                              o_mat* mat /*[2]*/, o_liquid* lqd, o_parameter* prm,
                              double* InitParSize, int* ForceCap, double* dem /*[11]*/,
                              int* load_stage, double* load_tPacking, int* load_nOut,
                              double* rad, int* numCells, oi3* gridSize, double* Cellsize,
                              double* unit /*[7]*/) {
  CylinderBC* h_Cir = nullptr;
  CylinderBC* d_Cir = nullptr;
  FeedZone fz;
  SIMULATION sim;
  LOADMODE load;
  UNIT u;
  std::memset(&sim, 0, sizeof(sim));
  std::memset(&load, 0, sizeof(load));
  std::memset(&u, 0, sizeof(u));
  SEARCHCELL cell;
  cell.numCells = numCells;
  cell.gridSize = reinterpret_cast<int3*>(gridSize);
  cell.Cellsize = Cellsize;
  char gen[64];
  std::snprintf(gen, sizeof(gen), "%s", genfile);
  *ForceCap = 0;
  ReadData(Level_size, pLevel, level_nNebors, level_nPars, Nebor_Idx, h_Cir, d_Cir, &fz,
           reinterpret_cast<MatType*>(mat), reinterpret_cast<LIQUID*>(lqd),
           reinterpret_cast<PARAMETER*>(prm), InitParSize, ForceCap, &sim, &load, rad, cell, NP,
           nLevels, gen, 0);
  UnitReduce(&u, h_Cir, &fz, &load, rad, reinterpret_cast<MatType*>(mat),
             reinterpret_cast<LIQUID*>(lqd), *InitParSize, &sim, reinterpret_cast<PARAMETER*>(prm),
             cell, Level_size, nLevels, NP, 0, gen);
  std::memcpy(cir, h_Cir, sizeof(CylinderBC));
  feed[0] = fz.Lmin;
  feed[1] = fz.Lmax;
  dem[0] = sim.dt; dem[1] = sim.dtFactor; dem[2] = sim.cutGap; dem[3] = sim.ctime;
  dem[4] = sim.simTime; dem[5] = sim.fdtime; dem[6] = sim.outtime; dem[7] = sim.dumptime;
  dem[8] = sim.outinterval; dem[9] = sim.fdinterval; dem[10] = (double)sim.iter;
  *load_stage = load.stage;
  *load_tPacking = load.tPacking;
  *load_nOut = load.nOutPacking;
  unit[0] = u.rlunit; unit[1] = u.rmunit; unit[2] = u.rfunit; unit[3] = u.reunit;
  unit[4] = u.rsunit; unit[5] = u.rtunit; unit[6] = u.rvunit;
  std::free(h_Cir);
  std::free(d_Cir);
  return 0;
}
