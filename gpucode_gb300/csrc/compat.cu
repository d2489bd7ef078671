/*
 * compat.cu -- the reference heyDEM C API on this library's kernels.
 *
 * Every function declared in the reference's heydem.h:366-613 that lives in
 * Allocation.cpp, kernel.cu:22-50 or ParticleSystem.cu, with the same symbol,
 * signature, argument meaning and data layouts, so the reference driver
 * (main.cpp) links against libdem_gb300 unchanged.  Host I/O functions
 * (ReadData, UnitReduce, ...) are in host_io.cpp.
 *
 * Behaviour kept from the reference: void returns; legacy default stream;
 * process-global constant set (setMaterial & co.), so the API is not
 * re-entrant; CUDA failures print and exit(-1) like cutilSafeCall
 * (heydem.h:28-35).  Behaviour changed: a neighbour list that would overrun
 * its level's slots stops at capacity instead of writing out of bounds, and
 * dem_compat_errors() reports it (the reference writes past the buffer,
 * kernel.cu:833-836); thrust is replaced by the counting cell sort.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>

#include "dem_internal.h"

/* process globals (Allocation.cpp:5-18) */
double3 *hPos = nullptr, *hVel = nullptr, *hAngVel = nullptr, *hForce = nullptr;
double* hRad = nullptr;
double3 *dPos = nullptr, *dVel = nullptr, *dAngVel = nullptr, *dForce = nullptr, *dMom = nullptr;
double *dRMom = nullptr, *dRad = nullptr;
int *d_GridParticleHash = nullptr, *d_GridParticleIndex = nullptr, *d_CellStart = nullptr,
    *d_CellEnd = nullptr;

namespace {

dem::DevConsts g_consts; /* the constant-memory set (kernel.cu:15-19) */

/* device-side helpers the reference's wrappers never needed: the sort's
 * scratch and the error word */
struct CompatDevice {
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  int* err = nullptr;
};
CompatDevice g_dev;

/* the arithmetic of PpInterCalc / CirPWCalc / UpdateSystem: DEM_PREC_FP64 (the
 * reference's) unless DEM_COMPAT_PRECISION=mixed is set in the environment or
 * dem_compat_set_precision chose otherwise; -1 until first asked */
int g_precision = -1;

int compat_precision() {
  if (g_precision < 0) {
    const char* e = std::getenv("DEM_COMPAT_PRECISION");
    g_precision = (e && std::strcmp(e, "mixed") == 0) ? DEM_PREC_MIXED : DEM_PREC_FP64;
  }
  return g_precision;
}

void ensure_small() {
  if (!g_dev.err) {
    DEM_REF_CHECK(cudaMalloc((void**)&g_dev.err, sizeof(int)));
    DEM_REF_CHECK(cudaMemset(g_dev.err, 0, sizeof(int)));
  }
}

void* ensure_scratch(size_t bytes) {
  if (bytes > g_dev.scratch_bytes) {
    if (g_dev.scratch) DEM_REF_CHECK(cudaFree(g_dev.scratch));
    g_dev.scratch = nullptr;
    g_dev.scratch_bytes = 0;
    DEM_REF_CHECK(cudaMalloc(&g_dev.scratch, bytes));
    g_dev.scratch_bytes = bytes;
  }
  return g_dev.scratch;
}

dem::HistSoA soa(const PPCONTACT_HISTORY& h) {
  dem::HistSoA s;
  s.dispt = h.dispt; s.nDsp = h.nDsp; s.nDsp_mx = h.nDsp_mx; s.plstRad = h.plstRad;
  s.plstDfm = h.plstDfm; s.stage = h.stage; s.lqdBrg = h.lqdBrg;
  return s;
}
dem::HistSoA soa(const PWCONTACT_HISTORY& h) {
  dem::HistSoA s;
  s.dispt = h.dispt; s.nDsp = h.nDsp; s.nDsp_mx = h.nDsp_mx; s.plstRad = h.plstRad;
  s.plstDfm = h.plstDfm; s.stage = h.stage; s.lqdBrg = h.lqdBrg;
  return s;
}

void ok_or_exit(dem_status st) {
  if (st != DEM_OK) {
    std::fprintf(stderr, "libdem_gb300: %s\n", dem_last_error());
    std::exit(-1);
  }
}

dem::LevelView view(SEARCHCELL c, int* ncell_idx, double* level_size, int* npars, int* nneb, int nl) {
  dem::LevelView lv;
  lv.cell_size = c.Cellsize;
  lv.grid_size = c.gridSize;
  lv.ncell_idx = ncell_idx;
  lv.level_size = level_size;
  lv.level_npars = npars;
  lv.level_nnebors = nneb;
  lv.n_levels = nl;
  return lv;
}

}  // namespace

extern "C" {

/* reads and clears the compat path's device error word: bit 1 = neighbour-slot
 * overflow, bit 4 = a particle hashed outside the cell grid */
dem_status dem_compat_set_precision(int precision) {
  if (precision != DEM_PREC_FP64 && precision != DEM_PREC_MIXED)
    return dem::fail(DEM_ERR_ARG, "dem_compat_set_precision: DEM_PREC_FP64 or DEM_PREC_MIXED");
  g_precision = precision;
  return DEM_OK;
}

int dem_compat_precision(void) { return compat_precision(); }

int dem_compat_errors(void) {
  if (!g_dev.err) return 0;
  int v = 0;
  DEM_REF_CHECK(cudaMemcpy(&v, g_dev.err, sizeof(int), cudaMemcpyDeviceToHost));
  DEM_REF_CHECK(cudaMemset(g_dev.err, 0, sizeof(int)));
  return v;
}

/* ---------------- constants (kernel.cu:22-50) ---------------- */
void setMaterial(MatType* h_Mat) { std::memcpy(g_consts.mat, h_Mat, sizeof(g_consts.mat)); }
void setLiquid(LIQUID* h_lqd) { g_consts.lqd = *h_lqd; }
void setParameters(PARAMETER* h_Params) { g_consts.prm = *h_Params; }
void setCalpara(calParaPP* h_cal, calParaPW* h_pWcal) {
  g_consts.cal = *h_cal;
  std::memcpy(&g_consts.pwcal, h_pWcal, sizeof(calParaPP));
}

void IndexOffset(int* d_Num, int* d_nei, int Nn) { ok_or_exit(dem::inclusive_scan_small(d_Num, d_nei, Nn, 0)); }

/* ---------------- allocation (Allocation.cpp) ---------------- */
void ParticleInfoAlloc(int NP) {
  const size_t n = (size_t)(NP > 0 ? NP : 1);
  hPos = (double3*)std::calloc(n, sizeof(double3));
  hVel = (double3*)std::calloc(n, sizeof(double3));
  hForce = (double3*)std::calloc(n, sizeof(double3));
  hAngVel = (double3*)std::calloc(n, sizeof(double3));
  hRad = (double*)std::calloc(n, sizeof(double));
  DEM_REF_CHECK(cudaMalloc((void**)&dPos, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMalloc((void**)&dVel, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMalloc((void**)&dAngVel, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMalloc((void**)&dForce, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMalloc((void**)&dMom, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMalloc((void**)&dRMom, n * sizeof(double)));
  DEM_REF_CHECK(cudaMalloc((void**)&dRad, n * sizeof(double)));
  DEM_REF_CHECK(cudaMemset(dPos, 0, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMemset(dVel, 0, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMemset(dAngVel, 0, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMemset(dForce, 0, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMemset(dMom, 0, n * sizeof(double3)));
  DEM_REF_CHECK(cudaMemset(dRMom, 0, n * sizeof(double)));
  DEM_REF_CHECK(cudaMemset(dRad, 0, n * sizeof(double)));
}

static void alloc_hist_fields(double3** dispt, double** a, double** b, double** c, double** d, int** st,
                              int** lb, size_t n, bool device) {
  if (device) {
    DEM_REF_CHECK(cudaMalloc((void**)dispt, n * sizeof(double3)));
    DEM_REF_CHECK(cudaMalloc((void**)a, n * sizeof(double)));
    DEM_REF_CHECK(cudaMalloc((void**)b, n * sizeof(double)));
    DEM_REF_CHECK(cudaMalloc((void**)c, n * sizeof(double)));
    DEM_REF_CHECK(cudaMalloc((void**)d, n * sizeof(double)));
    DEM_REF_CHECK(cudaMalloc((void**)st, n * sizeof(int)));
    DEM_REF_CHECK(cudaMalloc((void**)lb, n * sizeof(int)));
    DEM_REF_CHECK(cudaMemset(*dispt, 0, n * sizeof(double3)));
    DEM_REF_CHECK(cudaMemset(*a, 0, n * sizeof(double)));
    DEM_REF_CHECK(cudaMemset(*b, 0, n * sizeof(double)));
    DEM_REF_CHECK(cudaMemset(*c, 0, n * sizeof(double)));
    DEM_REF_CHECK(cudaMemset(*d, 0, n * sizeof(double)));
    DEM_REF_CHECK(cudaMemset(*st, 0, n * sizeof(int)));
    DEM_REF_CHECK(cudaMemset(*lb, 0, n * sizeof(int)));
  } else {
    *dispt = (double3*)std::calloc(n, sizeof(double3));
    *a = (double*)std::calloc(n, sizeof(double));
    *b = (double*)std::calloc(n, sizeof(double));
    *c = (double*)std::calloc(n, sizeof(double));
    *d = (double*)std::calloc(n, sizeof(double));
    *st = (int*)std::calloc(n, sizeof(int));
    *lb = (int*)std::calloc(n, sizeof(int));
  }
}

void WallCntHstry_Alloc(PWCONTACT_HISTORY* h, PWCONTACT_HISTORY* d, PWCONTACT_HISTORY* d_old, int nWallCnt) {
  const size_t n = (size_t)(nWallCnt > 0 ? nWallCnt : 1);
  alloc_hist_fields(&h->dispt, &h->nDsp, &h->nDsp_mx, &h->plstRad, &h->plstDfm, &h->stage, &h->lqdBrg, n, false);
  alloc_hist_fields(&d->dispt, &d->nDsp, &d->nDsp_mx, &d->plstRad, &d->plstDfm, &d->stage, &d->lqdBrg, n, true);
  alloc_hist_fields(&d_old->dispt, &d_old->nDsp, &d_old->nDsp_mx, &d_old->plstRad, &d_old->plstDfm, &d_old->stage,
                    &d_old->lqdBrg, n, true);
}

void PPCntHstry_Alloc(PPCONTACT_HISTORY* h, PPCONTACT_HISTORY* d, PPCONTACT_HISTORY* d_old, int nPPCnt) {
  const size_t n = (size_t)(nPPCnt > 0 ? nPPCnt : 1);
  std::memset(h, 0, sizeof(*h));
  std::memset(d, 0, sizeof(*d));
  std::memset(d_old, 0, sizeof(*d_old));
  alloc_hist_fields(&h->dispt, &h->nDsp, &h->nDsp_mx, &h->plstRad, &h->plstDfm, &h->stage, &h->lqdBrg, n, false);
  alloc_hist_fields(&d->dispt, &d->nDsp, &d->nDsp_mx, &d->plstRad, &d->plstDfm, &d->stage, &d->lqdBrg, n, true);
  alloc_hist_fields(&d_old->dispt, &d_old->nDsp, &d_old->nDsp_mx, &d_old->plstRad, &d_old->plstDfm, &d_old->stage,
                    &d_old->lqdBrg, n, true);
}

void NeborListAlloc(int** h_Num_Nebor, int** h_1DNebor, double** d_pMoveforReBld, int** d_Num_Nebor,
                    int** d_Num_Nebor_Old, int** d_Nebor1, int** d_Nebor1_Old, int** h_Num_stlWall,
                    int** h_StlWList_1D, int** d_Num_StlWall, int** d_Num_StlWall_Old, int** d_StlW_List,
                    int** d_StlW_List_Old, size_t* pitch_Sw1, size_t* pitch_Sw2, int NP, int nPPCnt,
                    int StlMaxWallPerBall) {
  const size_t n = (size_t)(NP > 0 ? NP : 1), m = (size_t)(nPPCnt > 0 ? nPPCnt : 1);
  *h_Num_Nebor = (int*)std::calloc(n, sizeof(int));
  *h_1DNebor = (int*)std::calloc(m, sizeof(int));
  DEM_REF_CHECK(cudaMalloc((void**)d_Num_Nebor, n * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)d_Num_Nebor_Old, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_Num_Nebor, 0, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_Num_Nebor_Old, 0, n * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)d_Nebor1, m * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)d_Nebor1_Old, m * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_Nebor1, 0, m * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_Nebor1_Old, 0, m * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)d_pMoveforReBld, n * sizeof(double)));
  /* the reference clears only NP bytes here (Allocation.cpp:212); all of it is cleared */
  DEM_REF_CHECK(cudaMemset(*d_pMoveforReBld, 0, n * sizeof(double)));
  *h_Num_stlWall = (int*)std::calloc(n, sizeof(int));
  DEM_REF_CHECK(cudaMalloc((void**)d_Num_StlWall, n * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)d_Num_StlWall_Old, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_Num_StlWall, 0, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_Num_StlWall_Old, 0, n * sizeof(int)));
  *h_StlWList_1D = (int*)std::calloc(n * (size_t)StlMaxWallPerBall, sizeof(int));
  DEM_REF_CHECK(cudaMallocPitch((void**)d_StlW_List, pitch_Sw1, StlMaxWallPerBall * sizeof(int), n));
  DEM_REF_CHECK(cudaMallocPitch((void**)d_StlW_List_Old, pitch_Sw2, StlMaxWallPerBall * sizeof(int), n));
  DEM_REF_CHECK(cudaMemset2D(*d_StlW_List, *pitch_Sw1, 0, StlMaxWallPerBall * sizeof(int), n));
  DEM_REF_CHECK(cudaMemset2D(*d_StlW_List_Old, *pitch_Sw2, 0, StlMaxWallPerBall * sizeof(int), n));
}

void FeedZoneAlloc(FeedZone** Feedcube) { *Feedcube = (FeedZone*)std::calloc(1, sizeof(FeedZone)); }

void ParamAlloc(SIMULATION** h_dem, UNIT** Rdu, int** h_lqdCnt, int** d_lqdCnt, int** d_lqdCnt_Old,
                MatType** h_Mat, LIQUID** h_lqd, PARAMETER** h_Params, SEARCHCELL* h_cell, SEARCHCELL* d_cell,
                int nLevels, int NP) {
  const size_t n = (size_t)(NP > 0 ? NP : 1), L = (size_t)(nLevels > 0 ? nLevels : 1);
  *h_dem = (SIMULATION*)std::calloc(1, sizeof(SIMULATION));
  *Rdu = (UNIT*)std::calloc(1, sizeof(UNIT));
  *h_lqdCnt = (int*)std::calloc(n, sizeof(int));
  DEM_REF_CHECK(cudaMalloc((void**)d_lqdCnt, n * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)d_lqdCnt_Old, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_lqdCnt, 0, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(*d_lqdCnt_Old, 0, n * sizeof(int)));
  h_cell->Cellsize = (double*)std::calloc(L, sizeof(double));
  h_cell->gridSize = (int3*)std::calloc(L, sizeof(int3));
  h_cell->numCells = (int*)std::calloc(L, sizeof(int));
  DEM_REF_CHECK(cudaMalloc((void**)&d_cell->Cellsize, L * sizeof(double)));
  DEM_REF_CHECK(cudaMalloc((void**)&d_cell->gridSize, L * sizeof(int3)));
  DEM_REF_CHECK(cudaMalloc((void**)&d_cell->numCells, L * sizeof(int)));
  *h_Mat = (MatType*)std::calloc(DEM_NUM_MAT, sizeof(MatType));
  *h_lqd = (LIQUID*)std::calloc(1, sizeof(LIQUID));
  *h_Params = (PARAMETER*)std::calloc(1, sizeof(PARAMETER));
}

void SearchCellAlloc(int NP, int numCells) {
  const size_t n = (size_t)(NP > 0 ? NP : 1), c = (size_t)(numCells > 0 ? numCells : 1);
  DEM_REF_CHECK(cudaMalloc((void**)&d_GridParticleHash, n * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)&d_GridParticleIndex, n * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)&d_CellStart, c * sizeof(int)));
  DEM_REF_CHECK(cudaMalloc((void**)&d_CellEnd, c * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(d_GridParticleHash, 0, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(d_GridParticleIndex, 0, n * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(d_CellStart, 0, c * sizeof(int)));
  DEM_REF_CHECK(cudaMemset(d_CellEnd, 0, c * sizeof(int)));
}

void VarInit(double3** dForce_, double3** dMom_, double** dRMom_, int** d_lqdCnt, int** d_lqdCnt_Old, int NP) {
  ok_or_exit(dem::var_init(*dForce_, *dMom_, *dRMom_, *d_lqdCnt, *d_lqdCnt_Old, NP, 0));
}

/* ---------------- per-step wrappers (ParticleSystem.cu:141-375) ---------------- */

void BldNeborList(int* hash, int* index, int* cellStart, int* cellEnd, int* d_pLevel, SEARCHCELL d_cell,
                  int* d_Ncell_Idx, double* d_Level_size, int* d_level_nPars, int* d_level_nNebors, int nLevels,
                  double3* pos, int Sys_nCells, int* d_Nebor1, int* d_Nebor_Idx, int* d_Num_Nebor,
                  int TotalParticle, double* rad) {
  ensure_small();
  dem::LevelView lv = view(d_cell, d_Ncell_Idx, d_Level_size, d_level_nPars, d_level_nNebors, nLevels);
  void* scratch = ensure_scratch(dem::sort_scratch_bytes(TotalParticle, Sys_nCells));
  ok_or_exit(dem::cell_sort(pos, d_pLevel, nullptr, TotalParticle, lv, g_consts, Sys_nCells, hash, index,
                            cellStart, cellEnd, scratch, g_dev.err, 0));
  ok_or_exit(dem::neighbor_find(pos, rad, index, cellStart, cellEnd, d_pLevel, d_Nebor_Idx, lv, g_consts, d_Nebor1,
                                d_Num_Nebor, TotalParticle, g_dev.err, 0));
}

void BldCirWall(double3* pos, double* rad, CylinderBC* d_Cir, int* d_StlW_List, size_t pitch_Sw1,
                int* d_Num_StlWall, int TotalParticle) {
  ok_or_exit(dem::wall_list(pos, rad, d_Cir, d_StlW_List, pitch_Sw1, d_Num_StlWall, TotalParticle, g_consts, 0));
}

void HstryCopy(int* d_Nebor1, int* d_OldNebor1, int* d_pLevel, int* d_level_nNebors, int* d_level_nPars,
               int* d_Nebor_Idx, PPCONTACT_HISTORY old_h, PPCONTACT_HISTORY cur_h, int* d_Num_Nebor,
               int* d_Num_Nebor_Old, int TotalParticle, int NP) {
  (void)NP;
  ok_or_exit(dem::history_carry_pp(d_Nebor1, d_OldNebor1, d_pLevel, d_Nebor_Idx, d_Nebor_Idx, d_level_nPars,
                                   d_level_nNebors, soa(old_h), soa(cur_h), d_Num_Nebor, d_Num_Nebor_Old, nullptr,
                                   nullptr, TotalParticle, 0));
}

void HstryCopyPW(int* d_StlW_List, int* d_StlW_List_Old, size_t pitch_w1, size_t pitch_w2,
                 PWCONTACT_HISTORY old_h, PWCONTACT_HISTORY cur_h, int* d_Num_StlWall, int* d_Num_StlWall_Old,
                 int TotalParticle, int NP) {
  ok_or_exit(dem::history_carry_pw(d_StlW_List, pitch_w1, d_StlW_List_Old, pitch_w2, soa(old_h), soa(cur_h),
                                   d_Num_StlWall, d_Num_StlWall_Old, nullptr, TotalParticle, NP, NP, 0));
}

void PpInterCalc(double3* pos, double3* vel, double3* angvel, double* rad, int* d_Nebor1, int* d_pLevel,
                 int* d_level_nNebors, int* d_level_nPars, int* d_Nebor_Idx, PPCONTACT_HISTORY h,
                 int* d_Num_Nebor, int* d_lqdCnt, int* d_lqdCnt_Old, double3* force, double3* mom, double* rmom,
                 int TotalParticle, int NP, int ForceCap, int stage) {
  (void)NP;
  if (compat_precision() == DEM_PREC_MIXED) {
    ok_or_exit(dem::pp_force_ref_mixed(pos, vel, angvel, rad, d_Nebor1, d_pLevel, d_level_nPars, d_level_nNebors,
                                       d_Nebor_Idx, soa(h), d_Num_Nebor, d_lqdCnt, d_lqdCnt_Old, force, mom, rmom,
                                       TotalParticle, ForceCap, stage, g_consts, 0));
    return;
  }
  /* the spheres' liquid shares go to the library's scratch (the neighbour
   * build's sort scratch, idle between builds on the same stream) */
  double* share = ForceCap == 1 ? static_cast<double*>(ensure_scratch((size_t)TotalParticle * sizeof(double)))
                                : nullptr;
  ok_or_exit(dem::pp_force64(pos, vel, angvel, rad, d_Nebor1, d_pLevel, d_level_nPars, d_level_nNebors,
                             d_Nebor_Idx, soa(h), d_Num_Nebor, d_lqdCnt, d_lqdCnt_Old, force, mom, rmom,
                             TotalParticle, ForceCap, stage, g_consts, nullptr, share, 0));
}

void CirPWCalc(double3* pos, double3* vel, double3* angvel, double3* force, double3* mom, double* rmom, double* rad,
               CylinderBC* d_Cir, PWCONTACT_HISTORY h, int* d_Num_StlWall, int* d_StlW_List, size_t pitch_Sw1,
               int TotalParticle, int NP, int stage) {
  if (compat_precision() == DEM_PREC_MIXED) {
    ok_or_exit(dem::wall_force_ref_mixed(pos, vel, angvel, force, mom, rmom, rad, d_Cir, soa(h), d_Num_StlWall,
                                         d_StlW_List, pitch_Sw1, TotalParticle, NP, stage, g_consts, 0));
    return;
  }
  ok_or_exit(dem::wall_force64(pos, vel, angvel, force, mom, rmom, rad, d_Cir, soa(h), d_Num_StlWall, d_StlW_List,
                               pitch_Sw1, TotalParticle, NP, stage, g_consts, nullptr, true, 0));
}

void UpdateSystem(double* rad, double3* pos, double3* vel, double3* angvel, double3* force, double3* mom,
                  double* rmom, int* d_ReNebld, double* d_pMoveforReBld, int TotalParticle) {
  if (compat_precision() == DEM_PREC_MIXED) {
    ok_or_exit(dem::update_ref_mixed(rad, pos, vel, angvel, force, mom, rmom, d_ReNebld, d_pMoveforReBld,
                                     TotalParticle, g_consts, 0));
    return;
  }
  ok_or_exit(dem::update64(rad, pos, vel, angvel, force, mom, rmom, d_ReNebld, d_pMoveforReBld, TotalParticle,
                           g_consts, 0));
}

void NeborToCPU(int* h_Num_Nebor, int* d_Num_Nebor, int* h_1DNebor, int* d_Nebor1, int* h_Num_stlWall,
                int* d_Num_StlWall, int* h_StlWList_1D, int* d_StlW_List, PPCONTACT_HISTORY h_pp,
                PPCONTACT_HISTORY d_pp, PWCONTACT_HISTORY h_pw, PWCONTACT_HISTORY d_pw, int NP, int nPPCnt,
                size_t pitch_Sw1, int StlMaxWallPerBall) {
  const size_t n = (size_t)NP, m = (size_t)nPPCnt, w = (size_t)NP * StlMaxWallPerBall;
  const cudaMemcpyKind D2H = cudaMemcpyDeviceToHost;
  DEM_REF_CHECK(cudaMemcpy(h_Num_Nebor, d_Num_Nebor, n * sizeof(int), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_1DNebor, d_Nebor1, m * sizeof(int), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.dispt, d_pp.dispt, m * sizeof(double3), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.nDsp, d_pp.nDsp, m * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.nDsp_mx, d_pp.nDsp_mx, m * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.plstRad, d_pp.plstRad, m * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.plstDfm, d_pp.plstDfm, m * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.stage, d_pp.stage, m * sizeof(int), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pp.lqdBrg, d_pp.lqdBrg, m * sizeof(int), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_Num_stlWall, d_Num_StlWall, n * sizeof(int), D2H));
  DEM_REF_CHECK(cudaMemcpy2D(h_StlWList_1D, StlMaxWallPerBall * sizeof(int), d_StlW_List, pitch_Sw1,
                             StlMaxWallPerBall * sizeof(int), n, D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.dispt, d_pw.dispt, w * sizeof(double3), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.nDsp, d_pw.nDsp, w * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.nDsp_mx, d_pw.nDsp_mx, w * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.plstRad, d_pw.plstRad, w * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.plstDfm, d_pw.plstDfm, w * sizeof(double), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.stage, d_pw.stage, w * sizeof(int), D2H));
  DEM_REF_CHECK(cudaMemcpy(h_pw.lqdBrg, d_pw.lqdBrg, w * sizeof(int), D2H));
}

void WallCntHstryCopy(PWCONTACT_HISTORY old_h, PWCONTACT_HISTORY cur_h, int nWallCnt) {
  ok_or_exit(dem::history_rotate(soa(old_h), soa(cur_h), nWallCnt, 0));
}

void PPCntHstryCopy(PPCONTACT_HISTORY old_h, PPCONTACT_HISTORY cur_h, int nPPCnt) {
  ok_or_exit(dem::history_rotate(soa(old_h), soa(cur_h), nPPCnt, 0));
}

}  // extern "C"

/* ---------------- BldNeborList without device allocation ----------------
 *
 * Some callers may not allocate device memory while they step: a driver that
 * reserves the card's memory once, up front, for a fixed plan of particle
 * buffers, and loops that cannot take the device-wide synchronisation that
 * cudaFree implies (BldNeborList above frees and re-allocates its scratch cache
 * when the particle count grows; the reference's thrust sort allocates on every
 * call).  BldNeborListNoAlloc gives them the same neighbour build with the
 * cell sort's scratch in a fixed array of device memory that the library image
 * carries, so the call itself never allocates. */

namespace {

/* 16 MiB: the sort's keys and ranks (2 ints per particle), one int per scan
 * tile of 2048 cells and 64 spare ints -- about 2 million particles.  Nothing
 * in it has to start at zero: within one call every word is written before it
 * is read. */
constexpr size_t kStaticSortScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_static_sort_scratch[kStaticSortScratchBytes];

/* The array's device address in the current context, looked up on every call:
 * the lookup is a table read once the library's device code is loaded, and a
 * cached address would go stale when the caller resets the device
 * (cudaDeviceReset) or a new primary context loads the code elsewhere.  The
 * name g_static_sort_scratch is a host-side stand-in in host code: only this
 * address may be handed to kernels. */
dem_status static_scratch(void** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_static_sort_scratch);
  if (e != cudaSuccess) return dem::cuda_check(e, "BldNeborListNoAlloc: cudaGetSymbolAddress");
  if (!p) return dem::fail(DEM_ERR_CUDA, "BldNeborListNoAlloc: the static scratch has no device address");
  *out = p;
  return DEM_OK;
}

}  // namespace

extern "C" int BldNeborListNoAlloc(int* hash, int* index, int* cellStart, int* cellEnd, int* d_pLevel,
                                   SEARCHCELL d_cell, int* d_Ncell_Idx, double* d_Level_size,
                                   int* d_level_nPars, int* d_level_nNebors, int nLevels, double3* pos,
                                   int Sys_nCells, int* d_Nebor1, int* d_Nebor_Idx, int* d_Num_Nebor,
                                   int TotalParticle, double* rad, int* d_err) {
  if (TotalParticle < 0 || Sys_nCells <= 0 || nLevels <= 0)
    return dem::fail(DEM_ERR_ARG, "BldNeborListNoAlloc: bad sizes (TotalParticle " + std::to_string(TotalParticle) +
                                      ", Sys_nCells " + std::to_string(Sys_nCells) + ", nLevels " +
                                      std::to_string(nLevels) + ")");
  if (!d_err) return dem::fail(DEM_ERR_ARG, "BldNeborListNoAlloc: d_err is NULL (pass a zeroed device int)");
  const size_t need = dem::sort_scratch_bytes(TotalParticle, Sys_nCells);
  if (need > kStaticSortScratchBytes)
    return dem::fail(DEM_ERR_ARG, "BldNeborListNoAlloc: " + std::to_string(TotalParticle) + " particles and " +
                                      std::to_string(Sys_nCells) + " cells need " + std::to_string(need) +
                                      " bytes of sort scratch; the static scratch holds " +
                                      std::to_string(kStaticSortScratchBytes) + " (use BldNeborList)");
  void* scratch = nullptr;
  dem_status st = static_scratch(&scratch);
  if (st != DEM_OK) return st;
  dem::LevelView lv = view(d_cell, d_Ncell_Idx, d_Level_size, d_level_nPars, d_level_nNebors, nLevels);
  st = dem::cell_sort(pos, d_pLevel, nullptr, TotalParticle, lv, g_consts, Sys_nCells, hash, index, cellStart,
                      cellEnd, scratch, d_err, 0);
  if (st != DEM_OK) return st;
  return dem::neighbor_find(pos, rad, index, cellStart, cellEnd, d_pLevel, d_Nebor_Idx, lv, g_consts, d_Nebor1,
                            d_Num_Nebor, TotalParticle, d_err, 0);
}
