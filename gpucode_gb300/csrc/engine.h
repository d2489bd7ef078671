/*
 * engine.h -- the native engine's context (dem_ctx), shared by engine.cu and mixed.cu.
 *
 * Device memory layout (N particles, S neighbour slots, C cells):
 *  - particle state in cell order (reorder = 1) or caller order: pos, vel,
 *    angv (FP64 double3), rad, pmove (FP64), lqd (bridge count of the last
 *    step), id (caller id), plevel, nidx (rank inside the level: the slot
 *    column), plus tmp_* copies used while permuting;
 *  - neighbour lists: nebor[S] level/slot-major (slot(q,k) = base[L] +
 *    k*npars[L] + nidx[q], coalesced across consecutive particles for a fixed
 *    k), num_nebor[N]; wall lists wlist[N][3], nwall[N];
 *  - contact history: 64-byte ContactRec per slot (+ one bridge byte), and
 *    3N wall records (slot (a, q) at a*N + q);
 *  - *_old copies of the used slots, written at the start of a rebuild and
 *    read by the carry-over (fixed pointers, so a rebuild can sit inside a
 *    CUDA-graph conditional node);
 *  - mixed precision: FP32 shadow state read by neighbours, double-buffered
 *    per step (see mixed.cu).
 */
#pragma once

#include <cuda_runtime.h>

#include <utility>
#include <vector>

#include "dem_internal.h"

namespace dem {

struct MixedState; /* mixed.cu */

/* device-side step chaining (chain.cu): the device-launchable graphs of one
 * step (with and without the countdown) and of a rebuild, per shadow parity,
 * and the countdown of the running chain */
struct StepCtl {
  int left;
  int pad;
  cudaGraphExec_t step[2], single[2], rebuild[2];
};

struct EngineBufs {
  /* particle state */
  double3 *pos, *vel, *angv;
  double *rad, *pmove;
  int *lqd, *lqd_old, *id, *plevel, *nidx;
  int* inv; /* inv[id[q]] = q: the cell position of each caller index, renewed at every rebuild */
  double3 *tmp_pos, *tmp_vel, *tmp_angv;
  double3* tmp_out; /* 2 N: staging of exported arrays beside the three above */
  double* tmp_rad;
  int *tmp_lqd, *tmp_id, *tmp_plevel;
  double3 *force, *mom;
  double* rmom;
  /* lists */
  int *nebor, *num_nebor, *wlist, *nwall;
  int *nebor_old, *num_nebor_old, *wlist_old, *nwall_old, *nidx_old;
  /* history */
  ContactRec *rec, *rec_old, *wrec, *wrec_old;
  unsigned char *brg, *brg_old;
  /* sort */
  int *sorted_hash, *sorted_src, *old_to_new, *cell_start, *cell_end;
  int* cell_off; /* every cell's offset in sorted order, and the total (C + 1) */
  void* scratch;
  /* level tables */
  double* cell_size;
  int3* grid_size;
  int *ncell_idx, *npars, *nneb;
  double* level_size;
  CylinderBC* cyl; /* one cylinder, or one per system when systems are batched */
  /* batched systems (NULL for one system): system of each particle id, and
   * whether each system is wet */
  int *sys_of_id, *sys_wet;
  int n_sys;
  /* control words: flag (rebuild count from the integrator), need (host
   * request), err (error bits), counters (u64[8]) */
  int *flag, *need, *err;
  unsigned long long* counters;
};

}  // namespace dem

struct dem_ctx {
  dem_setup s;
  dem_options opt;
  int n;
  long long slots;
  cudaStream_t stream;
  /* host transfers: the copy stream and its events (xev[0]: the upload's
   * copies done; xev[1..5]: an export array gathered; xev[6]: the export's
   * copies done) */
  cudaStream_t xfer;
  cudaEvent_t xev[7];
  dem::DevConsts k;
  dem::LevelView lv;
  int lstart[DEM_MAX_LEVELS];
  dem::EngineBufs b;
  std::vector<void*> allocs;
  long long iter;
  long long rebuilds_host;
  double ctime;
  dem::MixedState* mx;
  /* CUDA graphs of opt.graph_steps steps, one per starting shadow parity, and
   * of one step (the remainder of a dem_step call) */
  cudaGraphExec_t graph_exec[2];
  cudaGraphExec_t graph_one[2];
  int parity; /* mixed: which shadow buffer the next step reads */
  int moving_walls; /* a cylinder's top wall moves (topv != 0): moved before every step's wall contacts */
  /* device-side step chaining (mixed precision): 0 not built yet, 1 built,
   * -1 unavailable (the conditional-node graphs run instead); the graphs
   * (instantiated for device launch) and a host-instantiated copy of the
   * one-step graph for dem_step(1) (launched from the host, a device-launch
   * graph starts ~5 us later); the control block on the device; and, while a
   * chained step is captured, the rebuild request word that gates its
   * kernels (NULL otherwise) */
  int chain_state;
  cudaGraphExec_t chain_step[2], chain_single[2], chain_rebuild[2];
  cudaGraphExec_t chain_single_host[2];
  dem::StepCtl* chain_ctl;
  const int* step_gate;
  /* dem_profile_kernels: when set, the rebuild and the step record an event
   * after each of their kernels (NULL otherwise, and always during capture) */
  std::vector<std::pair<const char*, cudaEvent_t>>* marks;
  /* dem_e2e_parts: when set, six timing events the host-facing calls record
   * at their boundaries (upload start, upload copies done, import queued,
   * step queued, export start, export copies done); NULL otherwise */
  cudaEvent_t* trace;
  /* learned capillary closure (DEM_CAP_MLP): the staged network on the device
   * (NULL until dem_set_capnet) and the particles' contact angles */
  void* cap_w;
  float theta_max;
  unsigned long long theta_seed;
  /* the liquid-bridge model (dem_set_liquid_model; mode 0: the reference's) */
  dem::LiquidModel lm;
};

namespace dem {

/* mixed.cu */
dem_status mixed_create(dem_ctx* c);
void mixed_destroy(dem_ctx* c);
/* regenerate shadow buffer `which` from the FP64 master state */
dem_status mixed_shadows(dem_ctx* c, int which, cudaStream_t s);
/* the neighbour build's FP32 prefilter over shadow buffer `which` */
Prefilter mixed_prefilter(dem_ctx* c, int which);
/* one fused step reading shadows `which`, writing shadows 1 - which */
dem_status mixed_step(dem_ctx* c, int which, cudaStream_t s);
/* a state import without a rebuild request: the host arrays already in the
 * tmp buffers, gathered into cell order with the shadow buffer `which`
 * rewritten, in one launch */
dem_status mixed_import(dem_ctx* c, int which, int has_v, int has_w, cudaStream_t s);
/* the same from mapped host arrays in caller order (hv, hw may be NULL: zero);
 * inv[i] is caller index i's cell position */
dem_status mixed_import_mapped(dem_ctx* c, int which, const int* inv, const double3* hp, const double3* hv,
                               const double3* hw, cudaStream_t s);
/* the mixed step's pair loop: one thread per particle (true) or warp-cooperative */
bool mixed_thread_loop(const dem_ctx* c);
/* the name of the step kernel mixed_step launches, e.g. "k_step_mixed<1,0>" */
const char* mixed_step_kernel_name(const dem_ctx* c);
/* copy the last step's bridge counts from the shadow `which` to the master */
dem_status mixed_pre_rebuild(dem_ctx* c, int which, cudaStream_t s);
/* download the last step's force totals into the FP64 force array */
dem_status mixed_force_to_master(dem_ctx* c, cudaStream_t s);
/* the last step's forces, FP32, cell order (x, y, z, unused) */
const float4* mixed_force_shadow(const dem_ctx* c);

/* chain.cu: the chaining kernel after a step (tail-launches the rebuild and
 * the next step), the countdown, and the reset of the rebuild request */
dem_status chain_launch_tail(StepCtl* ctl, int* flag, int* need, int* err, int parity, bool single, cudaStream_t s);
dem_status chain_set_left(StepCtl* ctl, int nsteps, cudaStream_t s);
dem_status chain_clear_request(int* flag, int* need, cudaStream_t s);

}  // namespace dem
