/*
 * tune.cu -- the autotuner: neighbour skin, cell size and the step kernel's
 * block size for a given bed, chosen by timing short runs of the real engine.
 *
 * Each candidate builds its set-up from the same input (the skin scales
 * CUTGAPFORNEIGHBORLIST, ReadData.cpp:363; the cell size multiplies the
 * reference's (1 + 1.4 cut) 2 r_level, ReadData.cpp:365), creates a context
 * with the block size, loads the same state (and batched systems), runs
 * warm-up steps -- the first one builds the lists -- and then times trial
 * steps with CUDA events on the context's stream.  Rebuilds inside the trial
 * count: a small skin pays in rebuilds what it saves per step.
 */
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "dem_internal.h"

extern "C" dem_status dem_scale_cells(dem_setup* s, double factor);

namespace {

dem_status trial(const dem_input* in, const double* dia, const double3* pos, const double3* vel, dem_options opt,
                 double skin, double cell, int block, const dem_tune_space* sp, int n_sys, const int* sys,
                 const CylinderBC* cyl, const int* wet, dem_setup* out_setup, double* rate) {
  dem_input ii = *in;
  ii.cut_gap = in->cut_gap * skin;
  const int n = in->np;
  std::vector<double> rad((size_t)n);
  std::vector<int> plevel((size_t)n), nidx((size_t)n);
  dem_setup s;
  dem_status st = dem_build_setup(&ii, dia, &s, rad.data(), plevel.data(), nidx.data());
  if (st == DEM_OK) st = dem_scale_cells(&s, cell);
  if (st != DEM_OK) return st;
  opt.block_size = block;
  dem_ctx* c = nullptr;
  st = dem_create(&s, rad.data(), plevel.data(), nidx.data(), &opt, &c);
  if (st != DEM_OK) return st;
  if (st == DEM_OK) st = dem_set_state(c, pos, vel, nullptr);
  if (st == DEM_OK && n_sys > 0) st = dem_set_systems(c, n_sys, sys, cyl, wet);
  if (st == DEM_OK) st = dem_step(c, sp->warmup_steps);
  if (st == DEM_OK) st = dem_sync(c);
  cudaEvent_t a = nullptr, b = nullptr;
  if (st == DEM_OK) st = dem::cuda_check(cudaEventCreate(&a), "autotune event");
  if (st == DEM_OK) st = dem::cuda_check(cudaEventCreate(&b), "autotune event");
  cudaStream_t cs = (cudaStream_t)dem_stream(c);
  if (st == DEM_OK) {
    cudaEventRecord(a, cs);
    st = dem_step(c, sp->trial_steps);
    cudaEventRecord(b, cs);
  }
  if (st == DEM_OK) st = dem_sync(c);
  float ms = 0.f;
  if (st == DEM_OK) st = dem::cuda_check(cudaEventElapsedTime(&ms, a, b), "autotune timing");
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  dem_destroy(c);
  if (st == DEM_OK) {
    *rate = ms > 0.f ? (double)n * sp->trial_steps / (ms * 1e-3) : 0.0;
    if (out_setup) *out_setup = s;
  }
  return st;
}

}  // namespace

extern "C" dem_status dem_autotune(const dem_input* in, const double* dia, const double3* pos, const double3* vel,
                                   const dem_options* base, const dem_tune_space* space, int n_sys,
                                   const int* system_of_particle, const CylinderBC* cyl, const int* wet,
                                   dem_setup* best_setup, dem_options* best_opt, dem_tune_result* rep) {
  if (!in || !dia || !pos || !space || !best_setup || !best_opt)
    return dem::fail(DEM_ERR_ARG, "dem_autotune: null argument");
  const int ns = space->n_skin, nc = space->n_cell, nb = space->n_block;
  if (ns < 1 || nc < 1 || nb < 1 || ns > 8 || nc > 8 || nb > 4 || ns * nc * nb > 64 || space->trial_steps < 1 ||
      space->warmup_steps < 1)
    return dem::fail(DEM_ERR_ARG, "dem_autotune: candidate space out of range");
  dem_options opt;
  if (base) opt = *base;
  else dem_default_options(&opt);
  dem_tune_result r;
  std::memset(&r, 0, sizeof(r));
  r.best_rate = -1.0;
  for (int i = 0; i < ns; i++)
    for (int j = 0; j < nc; j++)
      for (int k = 0; k < nb; k++) {
        double rate = 0.0;
        dem_setup s;
        const dem_status st = trial(in, dia, pos, vel, opt, space->skin_scale[i], space->cell_scale[j],
                                    space->block_size[k], space, n_sys, system_of_particle, cyl, wet, &s, &rate);
        if (st != DEM_OK) return st;
        r.rate[r.n_tried++] = rate;
        if (rate > r.best_rate) {
          r.best_rate = rate;
          r.skin_scale = space->skin_scale[i];
          r.cell_scale = space->cell_scale[j];
          r.block_size = space->block_size[k];
          *best_setup = s;
        }
      }
  *best_opt = opt;
  best_opt->block_size = r.block_size;
  if (rep) *rep = r;
  return DEM_OK;
}
