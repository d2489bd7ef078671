/*
 * refgpu.cu -- timing harness for the reference's own GPU kernels on this GPU.
 *
 * A reported baseline, not part of the product.  The reference's kernel.cu is
 * compiled for sm_103a into a cubin (baseline/Makefile, from the reference
 * sources); this harness loads it with the driver API and runs the
 * reference's time step in the order of main.cpp:433-568:
 *
 *   D2H read of the rebuild flag (main.cpp:470)
 *   if flagged: copy list/count/wall list to *Old and rotate the histories
 *               (ParticleSystem.cu:336-375), zero pMove, BldNeborList =
 *               calcHashG, thrust::sort_by_key, two 0xff memsets,
 *               reorderDataAndFindCellStartG, NeighborFindG
 *               (ParticleSystem.cu:44-130), CirWallListG, HstryCopyG,
 *               HstryCopyPWG (ParticleSystem.cu:170-230)
 *   VarInit (Allocation.cpp:308-317: one copy, four memsets)
 *   PPForceCalcG, CirPWInterG (ParticleSystem.cu:232-270, L1-preferred)
 *   memset of the flag, UpdateSystemG (ParticleSystem.cu:276-290)
 *
 * with the reference's launch shapes.  Buffers are laid out as Allocation.cpp
 * does (SoA histories, pitched wall list).  The neighbour list and the
 * histories get one extra level's worth of slots at the end: NeighborFindG
 * writes past its slots when a particle has more neighbours than its level
 * allows (kernel.cu:833-836), and the padding keeps such a write inside the
 * allocation; the run reports whether any count exceeded its level's slots.
 */
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/device_ptr.h>
#include <thrust/sort.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "heydem_gb300.h"

namespace {

std::string g_err;

bool ok_rt(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}
bool ok_drv(CUresult r, const char* what) {
  if (r == CUDA_SUCCESS) return true;
  const char* s = nullptr;
  cuGetErrorString(r, &s);
  g_err = std::string(what) + ": " + (s ? s : "unknown driver error");
  return false;
}

void grid_of(int n, int block, unsigned& blocks, unsigned& threads) { /* ParticleSystem.cu:28-33 */
  threads = (unsigned)(n < block ? n : block);
  if (threads == 0) threads = 1;
  blocks = (unsigned)((n + threads - 1) / threads);
  if (blocks == 0) blocks = 1;
}

__global__ void k_touch(const int4* p, size_t n, int* sink) {
  int acc = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int4 v = p[i];
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (acc == 0x7fffffff) *sink = acc;
}

struct Hist {
  double3* dispt = nullptr;
  double *nDsp = nullptr, *nDsp_mx = nullptr, *plstRad = nullptr, *plstDfm = nullptr;
  int *stage = nullptr, *lqdBrg = nullptr;
};

template <class T>
bool dalloc(T** p, size_t count, std::vector<void*>& owned) {
  if (!ok_rt(cudaMalloc((void**)p, count * sizeof(T) + 16), "cudaMalloc")) return false;
  owned.push_back(*p);
  return ok_rt(cudaMemset(*p, 0, count * sizeof(T) + 16), "cudaMemset");
}

bool hist_alloc(Hist& h, size_t m, std::vector<void*>& owned) {
  return dalloc(&h.dispt, m, owned) && dalloc(&h.nDsp, m, owned) && dalloc(&h.nDsp_mx, m, owned) &&
         dalloc(&h.plstRad, m, owned) && dalloc(&h.plstDfm, m, owned) && dalloc(&h.stage, m, owned) &&
         dalloc(&h.lqdBrg, m, owned);
}
PPCONTACT_HISTORY as_pp(const Hist& h) {
  PPCONTACT_HISTORY r;
  std::memset(&r, 0, sizeof(r));
  r.dispt = h.dispt; r.nDsp = h.nDsp; r.nDsp_mx = h.nDsp_mx; r.plstRad = h.plstRad; r.plstDfm = h.plstDfm;
  r.stage = h.stage; r.lqdBrg = h.lqdBrg;
  return r;
}
PWCONTACT_HISTORY as_pw(const Hist& h) {
  PWCONTACT_HISTORY r;
  r.dispt = h.dispt; r.nDsp = h.nDsp; r.nDsp_mx = h.nDsp_mx; r.plstRad = h.plstRad; r.plstDfm = h.plstDfm;
  r.stage = h.stage; r.lqdBrg = h.lqdBrg;
  return r;
}
/* PPCntHstryCopy / WallCntHstryCopy (ParticleSystem.cu:336-375): old <- cur, cur <- 0 */
bool hist_rotate(const Hist& old_h, const Hist& cur, size_t m) {
  const cudaMemcpyKind D2D = cudaMemcpyDeviceToDevice;
  return ok_rt(cudaMemcpy(old_h.dispt, cur.dispt, m * sizeof(double3), D2D), "rotate") &&
         ok_rt(cudaMemcpy(old_h.nDsp, cur.nDsp, m * sizeof(double), D2D), "rotate") &&
         ok_rt(cudaMemcpy(old_h.nDsp_mx, cur.nDsp_mx, m * sizeof(double), D2D), "rotate") &&
         ok_rt(cudaMemcpy(old_h.plstRad, cur.plstRad, m * sizeof(double), D2D), "rotate") &&
         ok_rt(cudaMemcpy(old_h.plstDfm, cur.plstDfm, m * sizeof(double), D2D), "rotate") &&
         ok_rt(cudaMemcpy(old_h.stage, cur.stage, m * sizeof(int), D2D), "rotate") &&
         ok_rt(cudaMemcpy(old_h.lqdBrg, cur.lqdBrg, m * sizeof(int), D2D), "rotate") &&
         ok_rt(cudaMemset(cur.dispt, 0, m * sizeof(double3)), "rotate") &&
         ok_rt(cudaMemset(cur.nDsp, 0, m * sizeof(double)), "rotate") &&
         ok_rt(cudaMemset(cur.nDsp_mx, 0, m * sizeof(double)), "rotate") &&
         ok_rt(cudaMemset(cur.plstRad, 0, m * sizeof(double)), "rotate") &&
         ok_rt(cudaMemset(cur.plstDfm, 0, m * sizeof(double)), "rotate") &&
         ok_rt(cudaMemset(cur.stage, 0, m * sizeof(int)), "rotate") &&
         ok_rt(cudaMemset(cur.lqdBrg, 0, m * sizeof(int)), "rotate");
}

}  // namespace

extern "C" {

typedef struct refgpu_stats {
  double step_ms;       /* mean wall time of a timed step on the device (events), flag read included */
  double force_ms;      /* mean PPForceCalcG time per timed step */
  double wall_ms;       /* mean CirPWInterG time */
  double update_ms;     /* mean UpdateSystemG time */
  int rebuilds;         /* list rebuilds inside the timed steps */
  int overflow;         /* 1 if a neighbour count exceeded its level's slots at any rebuild */
  long long contacts;   /* unused (0) */
} refgpu_stats;

const char* refgpu_last_error(void) { return g_err.c_str(); }

/* Runs `warmup` untimed then `steps` timed reference steps from the given
 * state (histories start empty).  flush/flush_bytes: a device buffer larger
 * than L2, written and read before every timed step outside the timing
 * (NULL: no eviction).  out_pos (may be NULL) receives the final positions. */
int refgpu_run(const char* cubin_path, const dem_setup* s, const double* pos, const double* vel,
               const double* angvel, const double* rad, const int* plevel, const int* nidx, int warmup,
               int steps, void* flush, size_t flush_bytes, double* out_pos, refgpu_stats* st) {
  g_err.clear();
  std::memset(st, 0, sizeof(*st));
  const int n = s->np, L = s->n_levels, C = s->sys_ncells;
  if (n <= 0 || L <= 0 || L > DEM_MAX_LEVELS || C <= 0) {
    g_err = "bad set-up sizes";
    return -1;
  }
  if (!ok_rt(cudaFree(0), "context")) return -2;
  CUmodule mod;
  if (!ok_drv(cuModuleLoad(&mod, cubin_path), "cuModuleLoad")) return -3;
  auto fn = [&](const char* name, CUfunction* f) { return ok_drv(cuModuleGetFunction(f, mod, name), name); };
  CUfunction fHash, fRange, fNeb, fWall, fCarry, fCarryPW, fForce, fPW, fUpd;
  if (!fn("calcHashG", &fHash) || !fn("reorderDataAndFindCellStartG", &fRange) || !fn("NeighborFindG", &fNeb) ||
      !fn("CirWallListG", &fWall) || !fn("HstryCopyG", &fCarry) || !fn("HstryCopyPWG", &fCarryPW) ||
      !fn("PPForceCalcG", &fForce) || !fn("CirPWInterG", &fPW) || !fn("UpdateSystemG", &fUpd)) {
    cuModuleUnload(mod);
    return -3;
  }
  cuFuncSetCacheConfig(fForce, CU_FUNC_CACHE_PREFER_L1);
  cuFuncSetCacheConfig(fPW, CU_FUNC_CACHE_PREFER_L1);
  cuFuncSetCacheConfig(fUpd, CU_FUNC_CACHE_PREFER_L1);

  /* constant memory (kernel.cu:15-19, set as kernel.cu:22-50 does) */
  auto setc = [&](const char* name, const void* src, size_t bytes) {
    CUdeviceptr p;
    size_t b = 0;
    if (!ok_drv(cuModuleGetGlobal(&p, &b, mod, name), name)) return false;
    if (b != bytes) {
      g_err = std::string(name) + ": size mismatch " + std::to_string(b) + " vs " + std::to_string(bytes);
      return false;
    }
    return ok_drv(cuMemcpyHtoD(p, src, bytes), name);
  };
  calParaPP pwcal;
  std::memcpy(&pwcal, &s->pwcal, sizeof(pwcal));
  if (!setc("d_Mat", s->mat, sizeof(s->mat)) || !setc("d_lqd", &s->lqd, sizeof(LIQUID)) ||
      !setc("d_Params", &s->prm, sizeof(PARAMETER)) || !setc("d_cal", &s->cal, sizeof(calParaPP)) ||
      !setc("d_pWcal", &pwcal, sizeof(calParaPP))) {
    cuModuleUnload(mod);
    return -4;
  }

  std::vector<void*> owned;
  int rc = 0;
  const size_t NP = (size_t)n;
  size_t S = (size_t)s->n_pp_slots;
  /* padding: one more level's worth of slots for the widest level */
  size_t pad = 0;
  for (int l = 0; l < L; l++) pad = std::max(pad, (size_t)s->level_npars[l] * (size_t)s->level_nnebors[l]);
  const size_t Sp = S + pad;
  const size_t W = 3 * NP; /* nWallCnt = StlMaxWallPerBall * NP */
  double3 *dPos, *dVel, *dAng, *dForce, *dMom;
  double *dRad, *dRMom, *dPMove, *dLevelSize, *dCellSize;
  int *dLevel, *dNidx, *dNpars, *dNneb, *dNumCells, *dNcellIdx, *dHash, *dIndex, *dCS, *dCE, *dNeb, *dNebOld,
      *dNum, *dNumOld, *dNw, *dNwOld, *dLqd, *dLqdOld, *dFlag;
  int3* dGrid;
  CylinderBC* dCyl;
  Hist pp, ppOld, pw, pwOld;
  int *dWl = nullptr, *dWlOld = nullptr;
  size_t pitch1 = 0, pitch2 = 0;
  cudaEvent_t e0, e1, f0, f1, w0, w1, u0, u1;
  bool ev = false;
  int* sink = nullptr;
  std::vector<int> cnt(NP), hidx(NP), hlev(NP);

  if (!(dalloc(&dPos, NP, owned) && dalloc(&dVel, NP, owned) && dalloc(&dAng, NP, owned) &&
        dalloc(&dForce, NP, owned) && dalloc(&dMom, NP, owned) && dalloc(&dRad, NP, owned) &&
        dalloc(&dRMom, NP, owned) && dalloc(&dPMove, NP, owned) && dalloc(&dLevelSize, L, owned) &&
        dalloc(&dCellSize, L, owned) && dalloc(&dLevel, NP, owned) && dalloc(&dNidx, NP, owned) &&
        dalloc(&dNpars, L, owned) && dalloc(&dNneb, L, owned) && dalloc(&dNumCells, L, owned) &&
        dalloc(&dNcellIdx, L, owned) && dalloc(&dHash, NP, owned) && dalloc(&dIndex, NP, owned) &&
        dalloc(&dCS, (size_t)C, owned) && dalloc(&dCE, (size_t)C, owned) && dalloc(&dNeb, Sp, owned) &&
        dalloc(&dNebOld, Sp, owned) && dalloc(&dNum, NP, owned) && dalloc(&dNumOld, NP, owned) &&
        dalloc(&dNw, NP, owned) && dalloc(&dNwOld, NP, owned) && dalloc(&dLqd, NP, owned) &&
        dalloc(&dLqdOld, NP, owned) && dalloc(&dFlag, 1, owned) && dalloc(&dGrid, L, owned) &&
        dalloc(&dCyl, 1, owned) && dalloc(&sink, 1, owned) && hist_alloc(pp, Sp, owned) &&
        hist_alloc(ppOld, Sp, owned) && hist_alloc(pw, W, owned) && hist_alloc(pwOld, W, owned))) {
    rc = -5;
    goto done;
  }
  if (!ok_rt(cudaMallocPitch((void**)&dWl, &pitch1, 3 * sizeof(int), NP), "pitch") ||
      !ok_rt(cudaMallocPitch((void**)&dWlOld, &pitch2, 3 * sizeof(int), NP), "pitch")) {
    rc = -5;
    goto done;
  }
  owned.push_back(dWl);
  owned.push_back(dWlOld);
  cudaMemset2D(dWl, pitch1, 0, 3 * sizeof(int), NP);
  cudaMemset2D(dWlOld, pitch2, 0, 3 * sizeof(int), NP);
  {
    const cudaMemcpyKind H2D = cudaMemcpyHostToDevice;
    if (!(ok_rt(cudaMemcpy(dPos, pos, NP * sizeof(double3), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dVel, vel, NP * sizeof(double3), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dAng, angvel, NP * sizeof(double3), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dRad, rad, NP * sizeof(double), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dLevel, plevel, NP * sizeof(int), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dNidx, nidx, NP * sizeof(int), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dLevelSize, s->level_size, L * sizeof(double), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dCellSize, s->cell_size, L * sizeof(double), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dNpars, s->level_npars, L * sizeof(int), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dNneb, s->level_nnebors, L * sizeof(int), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dNumCells, s->num_cells, L * sizeof(int), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dNcellIdx, s->ncell_idx, L * sizeof(int), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dGrid, s->grid_size, L * sizeof(int3), H2D), "h2d") &&
          ok_rt(cudaMemcpy(dCyl, &s->cyl, sizeof(CylinderBC), H2D), "h2d"))) {
      rc = -6;
      goto done;
    }
    std::memcpy(hlev.data(), plevel, NP * sizeof(int));
  }
  if (!(ok_rt(cudaEventCreate(&e0), "event") && ok_rt(cudaEventCreate(&e1), "event") &&
        ok_rt(cudaEventCreate(&f0), "event") && ok_rt(cudaEventCreate(&f1), "event") &&
        ok_rt(cudaEventCreate(&w0), "event") && ok_rt(cudaEventCreate(&w1), "event") &&
        ok_rt(cudaEventCreate(&u0), "event") && ok_rt(cudaEventCreate(&u1), "event"))) {
    rc = -7;
    goto done;
  }
  ev = true;
  {
    SEARCHCELL cell;
    cell.numCells = dNumCells;
    cell.gridSize = dGrid;
    cell.Cellsize = dCellSize;
    int nn = n, NPi = n, nL = L, force_cap = s->force_cap, stage = s->load_stage;
    size_t p1 = pitch1, p2 = pitch2;
    const int total = warmup + steps;
    bool first = true;
    double step_ms = 0, force_ms = 0, wall_ms = 0, upd_ms = 0;
    for (int it = 0; it < total && rc == 0; it++) {
      const bool timed = it >= warmup;
      if (timed && flush && flush_bytes >= 32) {
        const size_t half = flush_bytes / 2 / 16 * 16;
        cudaMemsetAsync(flush, it & 0xff, half, 0);
        k_touch<<<1216, 256>>>((const int4*)((char*)flush + half), half / 16, sink);
      }
      if (timed) cudaEventRecord(e0, 0);
      int hflag = 0;
      if (!ok_rt(cudaMemcpy(&hflag, dFlag, sizeof(int), cudaMemcpyDeviceToHost), "flag read")) { rc = -8; break; }
      if (hflag > 0 || first) {
        if (!first) {
          const cudaMemcpyKind D2D = cudaMemcpyDeviceToDevice;
          cudaMemcpy(dNumOld, dNum, NP * sizeof(int), D2D);
          cudaMemcpy(dNebOld, dNeb, S * sizeof(int), D2D);
          if (!hist_rotate(ppOld, pp, S)) { rc = -8; break; }
          cudaMemcpy(dNwOld, dNw, NP * sizeof(int), D2D);
          cudaMemcpy2D(dWlOld, pitch2, dWl, pitch1, 3 * sizeof(int), NP, D2D);
          if (!hist_rotate(pwOld, pw, W)) { rc = -8; break; }
        }
        cudaMemset(dPMove, 0, NP * sizeof(double));
        unsigned b, t;
        grid_of(n, 32, b, t);
        {
          void* a[] = {&dHash, &dIndex, &dLevel, &cell, &dNcellIdx, &dPos, &nn};
          if (!ok_drv(cuLaunchKernel(fHash, b, 1, 1, t, 1, 1, 0, 0, a, nullptr), "calcHashG")) { rc = -9; break; }
        }
        thrust::sort_by_key(thrust::device_ptr<int>(dHash), thrust::device_ptr<int>(dHash + n),
                            thrust::device_ptr<int>(dIndex));
        cudaMemset(dCS, 0xff, (size_t)C * sizeof(int));
        cudaMemset(dCE, 0xff, (size_t)C * sizeof(int));
        grid_of(n, 64, b, t);
        {
          void* a[] = {&dCS, &dCE, &dHash, &dIndex, &nn};
          if (!ok_drv(cuLaunchKernel(fRange, b, 1, 1, t, 1, 1, (t + 1) * sizeof(int), 0, a, nullptr),
                      "reorderDataAndFindCellStartG")) { rc = -9; break; }
        }
        grid_of(n, 128, b, t);
        {
          void* a[] = {&dPos, &dIndex, &dCS, &dCE, &dLevel, &cell, &dNcellIdx, &dLevelSize, &dNpars, &dNneb,
                       &nL, &dNeb, &dNidx, &dNum, &nn, &dRad};
          if (!ok_drv(cuLaunchKernel(fNeb, b, 1, 1, t, 1, 1, 0, 0, a, nullptr), "NeighborFindG")) { rc = -9; break; }
        }
        {
          void* a[] = {&dPos, &dRad, &dCyl, &dWl, &p1, &dNw, &nn};
          if (!ok_drv(cuLaunchKernel(fWall, b, 1, 1, t, 1, 1, 0, 0, a, nullptr), "CirWallListG")) { rc = -9; break; }
        }
        if (!first) {
          PPCONTACT_HISTORY ho = as_pp(ppOld), hc = as_pp(pp);
          grid_of(n, 256, b, t);
          void* a[] = {&dNeb, &dNebOld, &dLevel, &dNneb, &dNpars, &dNidx, &ho, &hc, &dNum, &dNumOld, &nn, &NPi};
          if (!ok_drv(cuLaunchKernel(fCarry, b, 1, 1, t, 1, 1, 0, 0, a, nullptr), "HstryCopyG")) { rc = -9; break; }
          PWCONTACT_HISTORY wo = as_pw(pwOld), wc = as_pw(pw);
          grid_of(n, 128, b, t);
          void* a2[] = {&dWl, &dWlOld, &p1, &p2, &wo, &wc, &dNw, &dNwOld, &nn, &NPi};
          if (!ok_drv(cuLaunchKernel(fCarryPW, b, 1, 1, t, 1, 1, 0, 0, a2, nullptr), "HstryCopyPWG")) { rc = -9; break; }
        }
        /* slot capacity check of this build (the padding absorbed any overrun) */
        if (!ok_rt(cudaMemcpy(cnt.data(), dNum, NP * sizeof(int), cudaMemcpyDeviceToHost), "counts")) { rc = -8; break; }
        for (size_t i = 0; i < NP; i++)
          if (cnt[i] > s->level_nnebors[hlev[i]]) st->overflow = 1;
        if (timed) st->rebuilds++;
        first = false;
      }
      /* VarInit (Allocation.cpp:308-317) */
      cudaMemcpy(dLqdOld, dLqd, NP * sizeof(int), cudaMemcpyDeviceToDevice);
      cudaMemset(dLqd, 0, NP * sizeof(int));
      cudaMemset(dForce, 0, NP * sizeof(double3));
      cudaMemset(dMom, 0, NP * sizeof(double3));
      cudaMemset(dRMom, 0, NP * sizeof(double));
      {
        const unsigned b = (unsigned)((n + 127) / 128);
        PPCONTACT_HISTORY hc = as_pp(pp);
        void* a[] = {&dPos, &dVel, &dAng, &dRad, &dNeb, &dLevel, &dNneb, &dNpars, &dNidx, &hc, &dNum, &dLqd,
                     &dLqdOld, &dForce, &dMom, &dRMom, &nn, &NPi, &force_cap, &stage};
        if (timed) cudaEventRecord(f0, 0);
        if (!ok_drv(cuLaunchKernel(fForce, b, 1, 1, 128, 1, 1, 0, 0, a, nullptr), "PPForceCalcG")) { rc = -9; break; }
        if (timed) cudaEventRecord(f1, 0);
        PWCONTACT_HISTORY wc = as_pw(pw);
        void* a2[] = {&dPos, &dVel, &dAng, &dForce, &dMom, &dRMom, &dRad, &dCyl, &wc, &dNw, &dWl, &p1, &nn, &NPi,
                      &stage};
        if (timed) cudaEventRecord(w0, 0);
        if (!ok_drv(cuLaunchKernel(fPW, b, 1, 1, 128, 1, 1, 0, 0, a2, nullptr), "CirPWInterG")) { rc = -9; break; }
        if (timed) cudaEventRecord(w1, 0);
      }
      cudaMemset(dFlag, 0, sizeof(int));
      {
        unsigned b, t;
        grid_of(n, 256, b, t);
        void* a[] = {&dRad, &dPos, &dVel, &dAng, &dForce, &dMom, &dRMom, &dFlag, &dPMove, &nn};
        if (timed) cudaEventRecord(u0, 0);
        if (!ok_drv(cuLaunchKernel(fUpd, b, 1, 1, t, 1, 1, 0, 0, a, nullptr), "UpdateSystemG")) { rc = -9; break; }
        if (timed) cudaEventRecord(u1, 0);
      }
      if (timed) {
        cudaEventRecord(e1, 0);
        if (!ok_rt(cudaEventSynchronize(e1), "step")) { rc = -10; break; }
        float a = 0, bb = 0, c = 0, d = 0;
        cudaEventElapsedTime(&a, e0, e1);
        cudaEventElapsedTime(&bb, f0, f1);
        cudaEventElapsedTime(&c, w0, w1);
        cudaEventElapsedTime(&d, u0, u1);
        step_ms += a;
        force_ms += bb;
        wall_ms += c;
        upd_ms += d;
      }
    }
    if (rc == 0 && !ok_rt(cudaDeviceSynchronize(), "run")) rc = -10;
    if (rc == 0 && steps > 0) {
      st->step_ms = step_ms / steps;
      st->force_ms = force_ms / steps;
      st->wall_ms = wall_ms / steps;
      st->update_ms = upd_ms / steps;
    }
    if (rc == 0 && out_pos && !ok_rt(cudaMemcpy(out_pos, dPos, NP * sizeof(double3), cudaMemcpyDeviceToHost), "d2h"))
      rc = -6;
  }
done:
  if (ev) {
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(f0); cudaEventDestroy(f1);
    cudaEventDestroy(w0); cudaEventDestroy(w1); cudaEventDestroy(u0); cudaEventDestroy(u1);
  }
  for (void* p : owned) cudaFree(p);
  cuModuleUnload(mod);
  return rc;
}

}  // extern "C"
