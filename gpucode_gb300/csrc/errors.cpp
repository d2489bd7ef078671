/*
 * errors.cpp -- error reporting and small runtime helpers of libdem_gb300.
 */
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <string>

#include "dem_internal.h"

namespace {
thread_local std::string g_last_error;
}

namespace dem {

void set_error(const std::string& msg) { g_last_error = msg; }
bool last_error_empty() { return g_last_error.empty(); }

dem_status fail(dem_status code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

dem_status cuda_check(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return DEM_OK;
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? DEM_ERR_NOMEM : DEM_ERR_CUDA;
}

void ref_check(cudaError_t e, const char* file, int line) {
  if (e == cudaSuccess) return;
  std::fprintf(stderr, "%s(%i) : cudaSafeCall() Runtime API error %d: %s.\n", file, line, (int)e,
               cudaGetErrorString(e));
  std::exit(-1);
}

dem_status cuda_alloc(void** p, size_t bytes) {
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    *p = nullptr;
    return cuda_check(e, "cudaMalloc");
  }
  return DEM_OK;
}

}  // namespace dem

extern "C" const char* dem_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* dem_version(void) {
  return "libdem_gb300 0.1 (sm_103a; FP64 reference-formula path + FP32-force/FP64-state path)";
}

/* sizes and field offsets of the public structs, so bindings written in other
 * languages can check their layout: returns the number of values written */
#include <cstddef>
extern "C" int dem_abi_layout(long long* out, int cap) {
  const long long v[] = {
      (long long)sizeof(CylinderBC),        (long long)offsetof(CylinderBC, R),
      (long long)sizeof(MatType),           (long long)sizeof(LIQUID),
      (long long)sizeof(PARAMETER),         (long long)offsetof(PARAMETER, SearchGap),
      (long long)sizeof(calParaPP),         (long long)sizeof(UNIT),
      (long long)sizeof(SIMULATION),        (long long)sizeof(LOADMODE),
      (long long)sizeof(FeedZone),          (long long)sizeof(dem_input),
      (long long)offsetof(dem_input, mat),  (long long)offsetof(dem_input, dt_override),
      (long long)sizeof(dem_setup),         (long long)offsetof(dem_setup, cyl),
      (long long)offsetof(dem_setup, mat),  (long long)offsetof(dem_setup, prm),
      (long long)offsetof(dem_setup, unit), (long long)offsetof(dem_setup, sim),
      (long long)offsetof(dem_setup, load), (long long)offsetof(dem_setup, level_size),
      (long long)offsetof(dem_setup, grid_size), (long long)offsetof(dem_setup, sys_ncells),
      (long long)offsetof(dem_setup, n_pp_slots), (long long)offsetof(dem_setup, rad_max),
      (long long)sizeof(dem_options),       (long long)sizeof(dem_stats),
      (long long)sizeof(PPCONTACT_HISTORY), (long long)sizeof(PWCONTACT_HISTORY),
      (long long)sizeof(SEARCHCELL),        (long long)sizeof(dem_liquid_model),
      (long long)offsetof(dem_liquid_model, seed)};
  const int n = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < n && i < cap; i++) out[i] = v[i];
  return n;
}
