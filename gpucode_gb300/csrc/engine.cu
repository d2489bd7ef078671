/*
 * engine.cu -- the native DEM engine (dem_* API) on one GB300.
 *
 * One time step is the reference's main.cpp:466-564 sequence -- rebuild when
 * the last integration flagged it, then p-p forces, wall forces, integration
 * -- with three GB300-specific changes:
 *  - the rebuild decision is taken on the device: each step starts with a
 *    one-thread kernel that reads the rebuild flag and sets the condition of a
 *    CUDA-graph IF node whose body is the whole rebuild, so a graph of many
 *    steps replays with no host round trip (the reference copies the flag to
 *    the host every step, main.cpp:470);
 *  - particles are kept in cell order: every rebuild permutes the particle
 *    state by the cell sort, so neighbours of consecutive particles are close
 *    in memory, and neighbour slots of consecutive particles are adjacent;
 *  - contact history is 64-byte records (one per slot) instead of seven
 *    parallel arrays; a rebuild copies only the used slots to the *_old
 *    buffers and the carry-over writes every used new slot (match -> copy,
 *    else zero), replacing the reference's full-array copy + memset
 *    (ParticleSystem.cu:336-375).
 *
 * Precision: DEM_PREC_FP64 runs the reference formulas (step64.cu) on these
 * buffers; DEM_PREC_MIXED runs the fused FP32-force / FP64-state kernel of
 * mixed.cu.
 */
#include <cuda_runtime.h>
#include <chrono>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dem_device.cuh"
#include "engine.h"

namespace dem {
namespace {

inline int grid_for(long long n, int block) { return n <= 0 ? 1 : (int)((n + block - 1) / block); }

template <class T>
dem_status dalloc(dem_ctx* c, T** p, size_t count) {
  void* q = nullptr;
  dem_status st = cuda_alloc(&q, sizeof(T) * (count ? count : 1));
  if (st != DEM_OK) return st;
  cudaError_t e = cudaMemset(q, 0, sizeof(T) * (count ? count : 1));
  if (e != cudaSuccess) {
    cudaFree(q);
    return cuda_check(e, "cudaMemset");
  }
  c->allocs.push_back(q);
  *p = (T*)q;
  return DEM_OK;
}

__global__ void k_zero_int(int* p, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = 0;
}

/* R1: copy the used slots (and wall slots) to the *_old buffers */
__global__ void k_copy_old(const int* __restrict__ nebor, const int* __restrict__ num_nebor,
                           const int* __restrict__ nidx, const int* __restrict__ plevel,
                           const int* __restrict__ npars, const int* __restrict__ nneb,
                           const ContactRec* __restrict__ rec, const unsigned char* __restrict__ brg,
                           const int* __restrict__ wlist, const int* __restrict__ nwall,
                           const ContactRec* __restrict__ wrec, int* __restrict__ nebor_old,
                           int* __restrict__ num_nebor_old, int* __restrict__ nidx_old,
                           ContactRec* __restrict__ rec_old, unsigned char* __restrict__ brg_old,
                           int* __restrict__ wlist_old, int* __restrict__ nwall_old,
                           ContactRec* __restrict__ wrec_old, int n, unsigned long long* counters) {
  const int p = reversed_block_thread(); /* the longest slot lists first */
  if (p == 0 && counters) counters[4] += 1; /* rebuilds */
  if (p >= n) return;
  const int L = plevel[p];
  const long long stride = npars[L];
  const long long base = slot_base(L, npars, nneb) + nidx[p];
  const int nn = num_nebor[p];
  for (int a = 0; a < nn; a++) {
    const long long s = base + a * stride;
    nebor_old[s] = nebor[s];
    rec_old[s] = rec[s];
    brg_old[s] = brg[s];
  }
  num_nebor_old[p] = nn;
  nidx_old[p] = nidx[p];
  const int nw = nwall[p];
  nwall_old[p] = nw;
  for (int a = 0; a < nw; a++) {
    wlist_old[3 * p + a] = wlist[3 * p + a];
    wrec_old[(long long)a * n + p] = wrec[(long long)a * n + p];
  }
}

/* R3: gather the particle state into sorted order */
__global__ void k_permute(const int* __restrict__ src, int n, const double3* __restrict__ pos,
                          const double3* __restrict__ vel, const double3* __restrict__ angv,
                          const double* __restrict__ rad, const int* __restrict__ lqd, const int* __restrict__ id,
                          const int* __restrict__ plevel, double3* __restrict__ tpos, double3* __restrict__ tvel,
                          double3* __restrict__ tangv, double* __restrict__ trad, int* __restrict__ tlqd,
                          int* __restrict__ tid, int* __restrict__ tplevel, int* __restrict__ old_to_new) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int p = src[q];
  tpos[q] = pos[p];
  tvel[q] = vel[p];
  tangv[q] = angv[p];
  trad[q] = rad[p];
  tlqd[q] = lqd[p];
  tid[q] = id[p];
  tplevel[q] = plevel[p];
  old_to_new[p] = q;
}

struct LevelStart {
  int v[DEM_MAX_LEVELS];   /* first sorted position of each level */
  int cnt[DEM_MAX_LEVELS]; /* particles per level */
};

/* R3b: copy back, recompute the level rank (sorted order is level-major), clear the path length */
__global__ void k_copy_back(int n, const double3* __restrict__ tpos, const double3* __restrict__ tvel,
                            const double3* __restrict__ tangv, const double* __restrict__ trad,
                            const int* __restrict__ tlqd, const int* __restrict__ tid,
                            const int* __restrict__ tplevel, double3* __restrict__ pos, double3* __restrict__ vel,
                            double3* __restrict__ angv, double* __restrict__ rad, int* __restrict__ lqd,
                            int* __restrict__ id, int* __restrict__ plevel, int* __restrict__ nidx,
                            double* __restrict__ pmove, LevelStart ls, int* __restrict__ err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  pos[q] = tpos[q];
  vel[q] = tvel[q];
  angv[q] = tangv[q];
  rad[q] = trad[q];
  lqd[q] = tlqd[q];
  id[q] = tid[q];
  const int L = tplevel[q];
  plevel[q] = L;
  int r = q - ls.v[L];
  /* a particle hashed into another level's cell range (only possible on the
   * far face of the grid) would break level-major order */
  if (r < 0 || r >= ls.cnt[L]) {
    atomicOr(err, 4);
    r = 0;
  }
  nidx[q] = r;
  pmove[q] = 0.0;
}

/* R6: carry-over into the new lists: matched slot -> copy, else zero */
__global__ void k_carry(const int* __restrict__ nebor, const int* __restrict__ num_nebor, const int* __restrict__ nidx,
                        const int* __restrict__ plevel, const int* __restrict__ npars, const int* __restrict__ nneb,
                        const int* __restrict__ nebor_old, const int* __restrict__ num_nebor_old,
                        const int* __restrict__ nidx_old, const ContactRec* __restrict__ rec_old,
                        const unsigned char* __restrict__ brg_old, ContactRec* __restrict__ rec,
                        unsigned char* __restrict__ brg, const int* __restrict__ wlist, const int* __restrict__ nwall,
                        const int* __restrict__ wlist_old, const int* __restrict__ nwall_old,
                        const ContactRec* __restrict__ wrec_old, ContactRec* __restrict__ wrec,
                        const int* __restrict__ src, const int* __restrict__ old_to_new, int n) {
  const int q = reversed_block_thread(); /* the longest slot lists first */
  if (q >= n) return;
  const int p = src ? src[q] : q;
  const int L = plevel[q];
  const long long stride = npars[L];
  const long long lb = slot_base(L, npars, nneb);
  const long long nb = lb + nidx[q], ob = lb + nidx_old[p];
  const int nn = num_nebor[q], no = num_nebor_old[p];
  ContactRec zero;
  zero.dx = zero.dy = zero.dz = zero.nDsp = zero.nDsp_mx = zero.plstRad = zero.plstDfm = 0.0;
  zero.stage = 0;
  for (int a = 0; a < nn; a++) {
    const long long s = nb + a * stride;
    const int partner = nebor[s];
    long long hit = -1;
    for (int b = 0; b < no; b++) {
      const long long t = ob + b * stride;
      int j = nebor_old[t];
      if (old_to_new) j = old_to_new[j];
      if (j == partner) hit = t; /* the reference lets the last match win */
    }
    if (hit >= 0) {
      rec[s] = rec_old[hit];
      brg[s] = brg_old[hit];
    } else {
      rec[s] = zero;
      brg[s] = 0;
    }
  }
  const int nw = nwall[q], nwo = nwall_old[p];
  for (int a = 0; a < nw; a++) {
    const int w = wlist[3 * q + a];
    long long hit = -1;
    for (int b = 0; b < nwo; b++)
      if (wlist_old[3 * p + b] == w) hit = (long long)b * n + p;
    wrec[(long long)a * n + q] = hit >= 0 ? wrec_old[hit] : zero;
  }
}

/* device-side rebuild decision: the IF node runs the rebuild when the last
 * integration flagged a particle or the host asked for one; the flag is then
 * cleared for this step's integrator to set again */
__global__ void k_decide(cudaGraphConditionalHandle h, int* flag, int* need) {
  const unsigned v = (*flag > 0 || *need != 0) ? 1u : 0u;
  *flag = 0;
  *need = 0;
  cudaGraphSetConditional(h, v);
}

__global__ void k_import(int n, const int* __restrict__ id, const double3* __restrict__ hp,
                         const double3* __restrict__ hv, const double3* __restrict__ hw, double3* __restrict__ pos,
                         double3* __restrict__ vel, double3* __restrict__ angv, int has_v, int has_w) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int i = id[q];
  pos[q] = hp[i];
  vel[q] = has_v ? hv[i] : make_double3(0.0, 0.0, 0.0);
  angv[q] = has_w ? hw[i] : make_double3(0.0, 0.0, 0.0);
}

/* inv[id[q]] = q: the cell-order position of each caller index */
__global__ void k_inverse(int n, const int* __restrict__ id, int* __restrict__ inv) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) inv[id[q]] = q;
}

/* dst[i] = src[inv[i]]: caller order, gathered from cell order and written in
 * order, ready for one contiguous copy to the host */
__global__ void k_export_gather(int n, const int* __restrict__ inv, const double3* __restrict__ src,
                                double3* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[inv[i]];
}

/* A caller's host array that kernels may read or write directly: page-locked
 * (cudaHostAlloc, cudaMallocHost, cudaHostRegister) and mapped on the current
 * device from its first byte to its last, with one contiguous device view;
 * NULL otherwise, and the copy engines move it through device staging. */
void* mapped_view(const void* p, size_t bytes) {
  if (!p || bytes == 0) return nullptr;
  cudaPointerAttributes a0, a1;
  std::memset(&a0, 0, sizeof(a0));
  std::memset(&a1, 0, sizeof(a1));
  const char* last = static_cast<const char*>(p) + (bytes - 1);
  if (cudaPointerGetAttributes(&a0, p) != cudaSuccess || cudaPointerGetAttributes(&a1, last) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  if (static_cast<const char*>(a1.devicePointer) - static_cast<const char*>(a0.devicePointer) != (ptrdiff_t)(bytes - 1))
    return nullptr;
  return a0.devicePointer;
}

/* The state import from mapped host arrays: thread i reads the caller's
 * element i (a warp reads 768 contiguous bytes over the host link) and
 * writes it at its cell position inv[i] */
__global__ void k_import_mapped(int n, const int* __restrict__ inv, const double3* __restrict__ hp,
                                const double3* __restrict__ hv, const double3* __restrict__ hw,
                                double3* __restrict__ pos, double3* __restrict__ vel, double3* __restrict__ angv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int q = inv[i];
  pos[q] = hp[i];
  vel[q] = hv ? hv[i] : make_double3(0.0, 0.0, 0.0);
  angv[q] = hw ? hw[i] : make_double3(0.0, 0.0, 0.0);
}

/* The state export into mapped host arrays in caller order (array k =
 * blockIdx.y).  An array of n double3 is 3n doubles; thread t writes doubles
 * 2t and 2t + 1 -- component c of particle i is double 3i + c, read from cell
 * position inv[i] -- as one 16-byte store, so a warp writes 512 contiguous
 * bytes over the host link (three 8-byte stores 24 bytes apart per particle
 * leave partial lines: a third of the link's rate, measured).  A destination
 * that is not 16-byte aligned takes 8-byte stores. */
struct ExportSet {
  const void* src[5];
  int kind[5]; /* 0: double3 array, 1: float4 array (x y z), 2: zeros */
  double* dst[5];
  int count;
};
__device__ __forceinline__ double export_value(const void* src, int kind, int q, int c) {
  if (kind == 0) return static_cast<const double*>(src)[3LL * q + c];
  if (kind == 1) return (double)static_cast<const float*>(src)[4LL * q + c];
  return 0.0;
}
__global__ void k_export_mapped(int n, const int* __restrict__ inv, ExportSet x) {
  const int k = blockIdx.y;
  if (k >= x.count) return;
  const void* src = x.src[k];
  const int kind = x.kind[k];
  double* __restrict__ dst = x.dst[k];
  const long long m = 3LL * n;
  const long long e = 2LL * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
  if (e >= m) return;
  const long long i0 = e / 3, i1 = (e + 1) / 3;
  const double v0 = export_value(src, kind, inv[i0], (int)(e - 3 * i0));
  if (e + 1 < m) {
    const double v1 = export_value(src, kind, inv[i1], (int)(e + 1 - 3 * i1));
    if ((reinterpret_cast<size_t>(dst) & 15) == 0) {
      *reinterpret_cast<double2*>(dst + e) = make_double2(v0, v1);
    } else {
      dst[e] = v0;
      dst[e + 1] = v1;
    }
  } else {
    dst[e] = v0;
  }
}

__global__ void k_check_finite(int n, const double3* __restrict__ pos, const double3* __restrict__ vel,
                               int* __restrict__ err) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double3 p = pos[q], v = vel[q];
  if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(v.x) && isfinite(v.y) && isfinite(v.z)))
    atomicOr(err, 2);
}

/* ------------------------------------------------------------------ */

HistAoS hist_pp(dem_ctx* c) { return HistAoS{c->b.rec, c->b.brg}; }
HistAoS hist_pw(dem_ctx* c) { return HistAoS{c->b.wrec, nullptr}; }

/* dem_profile_kernels: an event after the kernel(s) just enqueued */
void mark(dem_ctx* c, cudaStream_t s, const char* name) {
  if (!c->marks) return;
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  c->marks->emplace_back(name, e);
}

/* The whole rebuild, enqueued on s (graph-capturable: fixed pointers, no host sync). */
dem_status enqueue_rebuild(dem_ctx* c, cudaStream_t s, int parity) {
  EngineBufs& b = c->b;
  const int n = c->n;
  const bool reorder = c->opt.reorder != 0;
  dem_status st;
  if (c->opt.precision == DEM_PREC_MIXED) {
    st = mixed_pre_rebuild(c, parity, s);
    if (st != DEM_OK) return st;
    mark(c, s, "k_lqd_from_shadow");
  }
  k_copy_old<<<grid_for(n, 128), 128, 0, s>>>(b.nebor, b.num_nebor, b.nidx, b.plevel, b.npars, b.nneb, b.rec, b.brg,
                                               b.wlist, b.nwall, b.wrec, b.nebor_old, b.num_nebor_old, b.nidx_old,
                                               b.rec_old, b.brg_old, b.wlist_old, b.nwall_old, b.wrec_old, n,
                                               b.counters);
  mark(c, s, "k_copy_old");
  st = cell_sort(b.pos, b.plevel, reorder ? b.id : nullptr, n, c->lv, c->k, c->s.sys_ncells, b.sorted_hash,
                 b.sorted_src, b.cell_start, b.cell_end, b.scratch, b.err, s, b.cell_off);
  if (st != DEM_OK) return st;
  mark(c, s, "cell sort (k_hash_count .. k_cell_order)");
  if (reorder) {
    k_permute<<<grid_for(n, 256), 256, 0, s>>>(b.sorted_src, n, b.pos, b.vel, b.angv, b.rad, b.lqd, b.id, b.plevel,
                                                b.tmp_pos, b.tmp_vel, b.tmp_angv, b.tmp_rad, b.tmp_lqd, b.tmp_id,
                                                b.tmp_plevel, b.old_to_new);
    mark(c, s, "k_permute");
    LevelStart ls;
    for (int l = 0; l < DEM_MAX_LEVELS; l++) {
      ls.v[l] = l < c->s.n_levels ? c->lstart[l] : 0;
      ls.cnt[l] = l < c->s.n_levels ? c->s.level_npars[l] : 0;
    }
    k_copy_back<<<grid_for(n, 256), 256, 0, s>>>(n, b.tmp_pos, b.tmp_vel, b.tmp_angv, b.tmp_rad, b.tmp_lqd, b.tmp_id,
                                                  b.tmp_plevel, b.pos, b.vel, b.angv, b.rad, b.lqd, b.id, b.plevel,
                                                  b.nidx, b.pmove, ls, b.err);
    mark(c, s, "k_copy_back");
  } else {
    cudaError_t e = cudaMemsetAsync(b.pmove, 0, sizeof(double) * (size_t)n, s);
    if (e != cudaSuccess) return cuda_check(e, "pmove reset");
  }
  Prefilter pre{nullptr, 0.f};
  if (c->opt.precision == DEM_PREC_MIXED) {
    /* the permuted state's shadows: read by the next step and by the build's prefilter */
    st = mixed_shadows(c, parity, s);
    if (st != DEM_OK) return st;
    pre = mixed_prefilter(c, parity);
    mark(c, s, "k_shadows");
  }
  st = neighbor_find(b.pos, b.rad, reorder ? nullptr : b.sorted_src, b.cell_start, b.cell_end, b.plevel, b.nidx,
                     c->lv, c->k, b.nebor, b.num_nebor, n, b.err, s, pre, b.cell_off);
  if (st != DEM_OK) return st;
  mark(c, s, "k_neighbor_find");
  st = wall_list(b.pos, b.rad, b.cyl, b.wlist, 3 * sizeof(int), b.nwall, n, c->k, s, b.id, b.sys_of_id);
  if (st != DEM_OK) return st;
  mark(c, s, "k_wall_list");
  k_carry<<<grid_for(n, 128), 128, 0, s>>>(b.nebor, b.num_nebor, b.nidx, b.plevel, b.npars, b.nneb, b.nebor_old,
                                           b.num_nebor_old, b.nidx_old, b.rec_old, b.brg_old, b.rec, b.brg, b.wlist,
                                           b.nwall, b.wlist_old, b.nwall_old, b.wrec_old, b.wrec,
                                           reorder ? b.sorted_src : nullptr, reorder ? b.old_to_new : nullptr, n);
  mark(c, s, "k_carry");
  /* the caller-order view of the new cell order, for the state import and export */
  k_inverse<<<grid_for(n, 256), 256, 0, s>>>(n, b.id, b.inv);
  mark(c, s, "k_inverse");
  return cuda_check(cudaGetLastError(), "rebuild launch");
}

/* One step's force + integration kernels (graph-capturable). */
dem_status enqueue_step(dem_ctx* c, cudaStream_t s, int parity) {
  EngineBufs& b = c->b;
  const int n = c->n;
  if (c->opt.precision == DEM_PREC_MIXED) return mixed_step(c, parity, s);
  dem_status st = var_init(b.force, b.mom, b.rmom, b.lqd, b.lqd_old, n, s);
  if (st != DEM_OK) return st;
  /* the export staging is idle during a step: it holds the spheres' liquid shares */
  st = pp_force64<HistAoS>(b.pos, b.vel, b.angv, b.rad, b.nebor, b.plevel, b.npars, b.nneb, b.nidx, hist_pp(c),
                           b.num_nebor, b.lqd, b.lqd_old, b.force, b.mom, b.rmom, n, c->s.force_cap,
                           c->s.load_stage, c->k, b.counters, reinterpret_cast<double*>(b.tmp_out), s, b.id, c->lm);
  if (st != DEM_OK) return st;
  st = wall_force64<HistAoS>(b.pos, b.vel, b.angv, b.force, b.mom, b.rmom, b.rad, b.cyl, hist_pw(c), b.nwall,
                             b.wlist, 3 * sizeof(int), n, n, c->s.load_stage, c->k, b.counters,
                             c->s.cyl.topv != 0.0, s);
  if (st != DEM_OK) return st;
  return update64(b.rad, b.pos, b.vel, b.angv, b.force, b.mom, b.rmom, b.flag, b.pmove, n, c->k, s);
}

void destroy_graph(dem_ctx* c) {
  for (int p = 0; p < 2; p++) {
    cudaGraphExec_t* all[6] = {&c->graph_exec[p],   &c->graph_one[p],     &c->chain_step[p],
                               &c->chain_single[p], &c->chain_rebuild[p], &c->chain_single_host[p]};
    for (cudaGraphExec_t* g : all) {
      if (*g) cudaGraphExecDestroy(*g);
      *g = nullptr;
    }
  }
  /* rebuilt on the next step against the new configuration */
  if (c->chain_state > 0) c->chain_state = 0;
}

/* G steps: [decide -> IF(rebuild) -> step] x G; the mixed path's shadow
 * parity alternates from start_parity */
dem_status build_graph(dem_ctx* c, int G, int start_parity, cudaGraphExec_t* out) {
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_check(e, "capture stream");
  cudaGraph_t g = nullptr;
  dem_status st = DEM_OK;
  auto ck = [&](cudaError_t err, const char* what) {
    if (st == DEM_OK && err != cudaSuccess) st = cuda_check(err, what);
    return st == DEM_OK;
  };
  if (!ck(cudaGraphCreate(&g, 0), "cudaGraphCreate")) {
    cudaStreamDestroy(cs);
    return st;
  }
  cudaGraphNode_t prev = nullptr;
  for (int step = 0; step < G && st == DEM_OK; step++) {
    const int parity = (c->opt.precision == DEM_PREC_MIXED) ? ((start_parity + step) & 1) : 0;
    cudaGraphConditionalHandle h;
    if (!ck(cudaGraphConditionalHandleCreate(&h, g, 0, 0), "conditional handle")) break;
    cudaGraphNode_t nd;
    cudaKernelNodeParams kp;
    std::memset(&kp, 0, sizeof(kp));
    void* args[3] = {&h, &c->b.flag, &c->b.need};
    kp.func = (void*)k_decide;
    kp.gridDim = dim3(1);
    kp.blockDim = dim3(1);
    kp.kernelParams = args;
    if (!ck(cudaGraphAddKernelNode(&nd, g, prev ? &prev : nullptr, prev ? 1 : 0, &kp), "decide node")) break;
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t nc;
    if (!ck(cudaGraphAddNode(&nc, g, &nd, nullptr, 1, &cp), "conditional node")) break;
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    if (!ck(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed),
            "capture rebuild"))
      break;
    dem_status rs = enqueue_rebuild(c, cs, parity);
    cudaGraph_t body_out = nullptr;
    cudaError_t ee = cudaStreamEndCapture(cs, &body_out);
    if (rs != DEM_OK) {
      st = rs;
      break;
    }
    if (!ck(ee, "end capture rebuild")) break;
    cudaGraph_t sg = nullptr;
    if (!ck(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed), "capture step")) break;
    dem_status ss = enqueue_step(c, cs, parity);
    ee = cudaStreamEndCapture(cs, &sg);
    if (ss != DEM_OK) {
      st = ss;
      if (sg) cudaGraphDestroy(sg);
      break;
    }
    if (!ck(ee, "end capture step")) break;
    cudaGraphNode_t ns;
    ck(cudaGraphAddChildGraphNode(&ns, g, &nc, 1, sg), "step node");
    cudaGraphDestroy(sg);
    prev = ns;
  }
  if (st == DEM_OK) {
    cudaGraphExec_t ex = nullptr;
    if (ck(cudaGraphInstantiate(&ex, g, 0), "cudaGraphInstantiate")) *out = ex;
  }
  cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  return st;
}

/* capture what `enqueue` puts on a stream into a graph instantiated for
 * device launch and uploaded, and (host_out) into a second instantiation for
 * launch from the host */
template <class F>
dem_status capture_device_graph(dem_ctx* c, F enqueue, cudaGraphExec_t* out, cudaGraphExec_t* host_out = nullptr) {
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_check(e, "capture stream");
  cudaGraph_t g = nullptr;
  dem_status st = DEM_OK;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    st = enqueue(cs);
    const cudaError_t ee = cudaStreamEndCapture(cs, &g);
    if (st == DEM_OK && ee != cudaSuccess) st = cuda_check(ee, "end capture");
  } else {
    st = cuda_check(e, "begin capture");
  }
  if (st == DEM_OK) {
    e = cudaGraphInstantiateWithFlags(out, g, cudaGraphInstantiateFlagDeviceLaunch);
    if (e == cudaSuccess) e = cudaGraphUpload(*out, c->stream);
    if (e != cudaSuccess) st = cuda_check(e, "device graph instantiate");
  }
  if (st == DEM_OK && host_out) {
    e = cudaGraphInstantiate(host_out, g, 0);
    if (e == cudaSuccess) e = cudaGraphUpload(*host_out, c->stream);
    if (e != cudaSuccess) st = cuda_check(e, "graph instantiate");
  }
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  return st;
}

/* the chained step graphs of the mixed path: S[p] (countdown), S1[p] (one
 * step), R[p] (rebuild), and the control block that names them */
dem_status build_chain(dem_ctx* c) {
  EngineBufs& b = c->b;
  dem_status st = DEM_OK;
  if (!c->chain_ctl) {
    void* p = nullptr;
    st = cuda_alloc(&p, sizeof(StepCtl));
    if (st != DEM_OK) return st;
    c->allocs.push_back(p);
    c->chain_ctl = (StepCtl*)p;
  }
  for (int p = 0; p < 2 && st == DEM_OK; p++) {
    st = capture_device_graph(
        c,
        [&](cudaStream_t cs) {
          dem_status r = chain_clear_request(b.flag, b.need, cs);
          return r == DEM_OK ? enqueue_rebuild(c, cs, p) : r;
        },
        &c->chain_rebuild[p]);
    for (int single = 0; single < 2 && st == DEM_OK; single++) {
      st = capture_device_graph(
          c,
          [&](cudaStream_t cs) {
            c->step_gate = b.need;
            dem_status r = enqueue_step(c, cs, p);
            c->step_gate = nullptr;
            return r == DEM_OK ? chain_launch_tail(c->chain_ctl, b.flag, b.need, b.err, p, single != 0, cs) : r;
          },
          single ? &c->chain_single[p] : &c->chain_step[p], single ? &c->chain_single_host[p] : nullptr);
    }
  }
  if (st == DEM_OK) {
    StepCtl h;
    std::memset(&h, 0, sizeof(h));
    for (int p = 0; p < 2; p++) {
      h.step[p] = c->chain_step[p];
      h.single[p] = c->chain_single[p];
      h.rebuild[p] = c->chain_rebuild[p];
    }
    st = cuda_check(cudaMemcpy(c->chain_ctl, &h, sizeof(h), cudaMemcpyHostToDevice), "step chain control");
  }
  return st;
}

/* one host-driven step: read the flag, rebuild if needed, step */
dem_status host_step(dem_ctx* c) {
  int hv[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(&hv[0], c->b.flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hv[1], c->b.need, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_check(e, "flag read");
  e = cudaMemsetAsync(c->b.flag, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->b.need, 0, sizeof(int), c->stream);
  if (e != cudaSuccess) return cuda_check(e, "flag reset");
  dem_status st;
  if (hv[0] > 0 || hv[1] != 0) {
    st = enqueue_rebuild(c, c->stream, c->parity);
    if (st != DEM_OK) return st;
  }
  st = enqueue_step(c, c->stream, c->parity);
  if (st != DEM_OK) return st;
  if (c->opt.precision == DEM_PREC_MIXED) c->parity ^= 1;
  c->iter++;
  c->ctime += c->s.sim.dt;
  return DEM_OK;
}

int graph_len(const dem_ctx* c) { return c->opt.graph_steps > 0 ? c->opt.graph_steps : 16; }

}  // namespace
}  // namespace dem

using namespace dem;

namespace {

/* device bytes of dem_create for N particles, S slots, C cells: the sums of
 * its allocation list (kept next to it), plus 2 MiB of rounding per allocation */
dem_memory memory_of(long long N, long long S, long long C, const dem_options* o) {
  dem_memory m;
  m.per_particle = 3 * 24 + 2 * 8 + 6 * 4      /* pos vel angv, rad pmove, lqd lqd_old id inv plevel nidx */
                   + 3 * 24 + 8 + 3 * 4        /* tmp copies used while permuting */
                   + 2 * 24                    /* staging of the force and moment exports */
                   + 2 * 24 + 8                /* force mom rmom */
                   + 4 + 12 + 4 + 4 + 12 + 4 + 4 /* num_nebor wlist nwall and their copies, nidx_old */
                   + 2 * 3 * 64                /* wall records and their copies */
                   + 3 * 4 + 2 * 4;            /* sorted hash / source, old_to_new, sort scratch */
  if (o && o->precision == DEM_PREC_MIXED) m.per_particle += 9 * 16; /* FP32 shadows */
  m.per_slot = 2 * (4 + 64 + 1);               /* list entry, record, bridge flag, and their copies */
  m.per_cell = 3 * 4;                         /* cell start, end, offset */
  m.slots = S;
  const long long allocations = 64;
  m.total = N * m.per_particle + S * m.per_slot + C * m.per_cell + ((C + 2047) / 2048 + 64) * 4 +
            allocations * (2LL << 20);
  if (o && o->capillary == DEM_CAP_MLP) m.total += 16 << 10;
  return m;
}

}  // namespace

extern "C" dem_status dem_memory_estimate(const dem_setup* s, const dem_options* o, dem_memory* out) {
  if (!s || !out) return fail(DEM_ERR_ARG, "dem_memory_estimate: null argument");
  dem_options d;
  if (!o) {
    dem_default_options(&d);
    o = &d;
  }
  *out = memory_of(s->np, s->n_pp_slots, s->sys_ncells, o);
  return DEM_OK;
}

extern "C" dem_status dem_fit_memory(dem_setup* s, const dem_options* o, double budget_bytes, int min_slots,
                                     double* factor) {
  if (!s || min_slots < 1 || !(budget_bytes > 0.0)) return fail(DEM_ERR_ARG, "dem_fit_memory: bad arguments");
  dem_options d;
  if (!o) {
    dem_default_options(&d);
    o = &d;
  }
  const int L = s->n_levels;
  auto slots_at = [&](double f, int* nneb) {
    long long S = 0;
    for (int l = 0; l < L; l++) {
      const int orig = s->level_nnebors[l];
      int v = (int)std::floor(f * orig);
      v = std::min(orig, std::max(v, std::min(min_slots, orig)));
      if (nneb) nneb[l] = v;
      S += (long long)v * s->level_npars[l];
    }
    return S;
  };
  auto bytes_at = [&](double f) { return (double)memory_of(s->np, slots_at(f, nullptr), s->sys_ncells, o).total; };
  double f = 1.0;
  if (bytes_at(1.0) > budget_bytes) {
    if (bytes_at(0.0) > budget_bytes)
      return fail(DEM_ERR_NOMEM, "dem_fit_memory: " + std::to_string(s->np) + " particles do not fit " +
                                     std::to_string(budget_bytes / 1e9) + " GB even at " +
                                     std::to_string(min_slots) + " slots per particle");
    double lo = 0.0, hi = 1.0;
    for (int it = 0; it < 60; it++) {
      const double mid = 0.5 * (lo + hi);
      if (bytes_at(mid) <= budget_bytes) lo = mid;
      else hi = mid;
    }
    f = lo;
  }
  int nneb[DEM_MAX_LEVELS];
  s->n_pp_slots = slots_at(f, nneb);
  for (int l = 0; l < L; l++) s->level_nnebors[l] = nneb[l];
  if (factor) *factor = f;
  return DEM_OK;
}

extern "C" void dem_default_options(dem_options* o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = DEM_PREC_MIXED;
  o->capillary = DEM_CAP_FORMULA;
  o->block_size = 0;
  o->reorder = 1;
  o->use_graph = 1;
}

extern "C" dem_status dem_create(const dem_setup* s, const double* rad, const int* plevel, const int* nebor_idx,
                                 const dem_options* opt, dem_ctx** out) {
  if (!s || !rad || !plevel || !nebor_idx || !out) return fail(DEM_ERR_ARG, "dem_create: null argument");
  *out = nullptr;
  if (s->np <= 0 || s->n_levels < 1 || s->n_levels > DEM_MAX_LEVELS || s->sys_ncells <= 0 || s->n_pp_slots <= 0)
    return fail(DEM_ERR_ARG, "dem_create: set-up sizes out of range");
  dem_ctx* c = new dem_ctx();
  c->s = *s;
  if (opt) c->opt = *opt;
  else dem_default_options(&c->opt);
  if (c->opt.precision == DEM_PREC_MIXED && !c->opt.reorder) {
    delete c;
    return fail(DEM_ERR_ARG, "dem_create: the mixed-precision path needs reorder = 1");
  }
  if (c->opt.capillary == DEM_CAP_MLP && c->opt.precision != DEM_PREC_MIXED) {
    delete c;
    return fail(DEM_ERR_ARG, "dem_create: the learned capillary closure runs on the mixed-precision path only");
  }
  c->n = s->np;
  c->slots = s->n_pp_slots;
  c->mx = nullptr;
  c->graph_exec[0] = c->graph_exec[1] = nullptr;
  c->graph_one[0] = c->graph_one[1] = nullptr;
  c->moving_walls = s->cyl.topv != 0.0 ? 1 : 0;
  c->marks = nullptr;
  c->parity = 0;
  c->cap_w = nullptr;
  c->theta_max = 0.52359878f; /* 30 degrees */
  c->theta_seed = 0;
  c->iter = 0;
  c->ctime = 0.0;
  std::memcpy(c->k.mat, s->mat, sizeof(c->k.mat));
  c->k.lqd = s->lqd;
  c->k.prm = s->prm;
  c->k.cal = s->cal;
  std::memcpy(&c->k.pwcal, &s->pwcal, sizeof(calParaPP));
  int acc = 0;
  for (int l = 0; l < DEM_MAX_LEVELS; l++) {
    c->lstart[l] = acc;
    if (l < s->n_levels) acc += s->level_npars[l];
  }
  if (acc != s->np) {
    delete c;
    return fail(DEM_ERR_ARG, "dem_create: level particle counts do not add up to np");
  }
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking);
  for (cudaEvent_t& ev : c->xev)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    for (cudaEvent_t ev : c->xev)
      if (ev) cudaEventDestroy(ev);
    if (c->xfer) cudaStreamDestroy(c->xfer);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return cuda_check(e, "cudaStreamCreate");
  }
  EngineBufs& b = c->b;
  std::memset(&b, 0, sizeof(b));
  const size_t N = (size_t)c->n, S = (size_t)c->slots, C = (size_t)s->sys_ncells, L = (size_t)s->n_levels;
  dem_status st = DEM_OK;
#define A(ptr, count) \
  if (st == DEM_OK) st = dalloc(c, &(ptr), (count))
  A(b.pos, N); A(b.vel, N); A(b.angv, N); A(b.rad, N); A(b.pmove, N); A(b.lqd, N); A(b.lqd_old, N);
  A(b.id, N); A(b.inv, N); A(b.plevel, N); A(b.nidx, N);
  A(b.tmp_pos, N); A(b.tmp_vel, N); A(b.tmp_angv, N); A(b.tmp_rad, N); A(b.tmp_lqd, N); A(b.tmp_id, N);
  A(b.tmp_out, 2 * N);
  A(b.tmp_plevel, N);
  A(b.force, N); A(b.mom, N); A(b.rmom, N);
  A(b.nebor, S); A(b.num_nebor, N); A(b.wlist, 3 * N); A(b.nwall, N);
  A(b.nebor_old, S); A(b.num_nebor_old, N); A(b.wlist_old, 3 * N); A(b.nwall_old, N); A(b.nidx_old, N);
  A(b.rec, S); A(b.rec_old, S); A(b.brg, S); A(b.brg_old, S); A(b.wrec, 3 * N); A(b.wrec_old, 3 * N);
  A(b.sorted_hash, N); A(b.sorted_src, N); A(b.old_to_new, N); A(b.cell_start, C); A(b.cell_end, C);
  A(b.cell_off, C + 1);
  A(b.cell_size, L); A(b.grid_size, L); A(b.ncell_idx, L); A(b.npars, L); A(b.nneb, L); A(b.level_size, L);
  A(b.cyl, 1); A(b.flag, 1); A(b.need, 1); A(b.err, 1); A(b.counters, 8);
#undef A
  if (st == DEM_OK) {
    void* sc = nullptr;
    st = cuda_alloc(&sc, sort_scratch_bytes(c->n, s->sys_ncells));
    if (st == DEM_OK) {
      c->allocs.push_back(sc);
      b.scratch = sc;
    }
  }
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (st != DEM_OK) return;
    cudaError_t ee = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    if (ee != cudaSuccess) st = cuda_check(ee, "upload");
  };
  up(b.cell_size, s->cell_size, sizeof(double) * L);
  up(b.grid_size, s->grid_size, sizeof(int3) * L);
  up(b.ncell_idx, s->ncell_idx, sizeof(int) * L);
  up(b.npars, s->level_npars, sizeof(int) * L);
  up(b.nneb, s->level_nnebors, sizeof(int) * L);
  up(b.level_size, s->level_size, sizeof(double) * L);
  up(b.cyl, &s->cyl, sizeof(CylinderBC));
  up(b.rad, rad, sizeof(double) * N);
  up(b.plevel, plevel, sizeof(int) * N);
  if (st == DEM_OK) {
    std::vector<int> ids(N);
    for (size_t i = 0; i < N; i++) ids[i] = (int)i;
    up(b.id, ids.data(), sizeof(int) * N);
    up(b.inv, ids.data(), sizeof(int) * N);
  }
  up(b.nidx, nebor_idx, sizeof(int) * N);
  const int one = 1;
  up(b.need, &one, sizeof(int));
  c->lv.cell_size = b.cell_size;
  c->lv.grid_size = b.grid_size;
  c->lv.ncell_idx = b.ncell_idx;
  c->lv.level_size = b.level_size;
  c->lv.level_npars = b.npars;
  c->lv.level_nnebors = b.nneb;
  c->lv.n_levels = s->n_levels;
  if (st == DEM_OK && c->opt.precision == DEM_PREC_MIXED) st = mixed_create(c);
  if (st != DEM_OK) {
    dem_destroy(c);
    return st;
  }
  *out = c;
  return DEM_OK;
}

extern "C" dem_status dem_set_systems(dem_ctx* c, int n_sys, const int* system_of_particle, const CylinderBC* cyl,
                                      const int* wet) {
  if (!c || n_sys < 1 || !system_of_particle || !cyl) return fail(DEM_ERR_ARG, "dem_set_systems: bad arguments");
  if (c->opt.precision != DEM_PREC_MIXED)
    return fail(DEM_ERR_ARG, "dem_set_systems: batched systems run on the mixed-precision path");
  if (c->b.sys_of_id) return fail(DEM_ERR_STATE, "dem_set_systems: the systems are already set");
  for (int i = 0; i < c->n; i++)
    if (system_of_particle[i] < 0 || system_of_particle[i] >= n_sys)
      return fail(DEM_ERR_ARG, "dem_set_systems: particle " + std::to_string(i) + " has system " +
                                   std::to_string(system_of_particle[i]) + " outside [0, " +
                                   std::to_string(n_sys) + ")");
  std::vector<int> w(n_sys, c->s.force_cap == 1 ? 1 : 0);
  if (wet)
    for (int k = 0; k < n_sys; k++) w[k] = wet[k] ? 1 : 0;
  EngineBufs& b = c->b;
  CylinderBC* cyls = nullptr;
  int *sys = nullptr, *sw = nullptr;
  dem_status st = dalloc(c, &cyls, (size_t)n_sys);
  if (st == DEM_OK) st = dalloc(c, &sys, (size_t)c->n);
  if (st == DEM_OK) st = dalloc(c, &sw, (size_t)n_sys);
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (st != DEM_OK) return;
    cudaError_t e = cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) st = cuda_check(e, "dem_set_systems upload");
  };
  up(cyls, cyl, sizeof(CylinderBC) * (size_t)n_sys);
  up(sys, system_of_particle, sizeof(int) * (size_t)c->n);
  up(sw, w.data(), sizeof(int) * (size_t)n_sys);
  if (st != DEM_OK) return st;
  b.cyl = cyls;
  c->moving_walls = 0;
  for (int k = 0; k < n_sys; k++)
    if (cyl[k].topv != 0.0) c->moving_walls = 1;
  b.sys_of_id = sys;
  b.sys_wet = sw;
  b.n_sys = n_sys;
  /* graphs captured the single-cylinder pointers: rebuild them; and the wall
   * lists must be rebuilt against the new cylinders */
  destroy_graph(c);
  const int one = 1;
  return cuda_check(cudaMemcpy(b.need, &one, sizeof(int), cudaMemcpyHostToDevice), "dem_set_systems");
}

extern "C" dem_status dem_destroy(dem_ctx* c) {
  if (!c) return DEM_OK;
  cudaStreamSynchronize(c->stream);
  destroy_graph(c);
  if (c->mx) mixed_destroy(c);
  for (void* p : c->allocs) cudaFree(p);
  for (cudaEvent_t ev : c->xev) cudaEventDestroy(ev);
  cudaStreamDestroy(c->xfer);
  cudaStreamDestroy(c->stream);
  delete c;
  return DEM_OK;
}

extern "C" void* dem_stream(dem_ctx* c) { return c ? (void*)c->stream : nullptr; }

extern "C" int dem_step_chained(dem_ctx* c) { return c && c->chain_state == 1 ? 1 : 0; }

extern "C" const char* dem_step_kernel(dem_ctx* c) {
  if (!c) return "";
  if (c->opt.precision == DEM_PREC_MIXED) return mixed_step_kernel_name(c);
  return "k_pp_force64 + k_wall_force64 + k_update64";
}

extern "C" dem_status dem_set_liquid_model(dem_ctx* c, const dem_liquid_model* m) {
  if (!c || !m) return fail(DEM_ERR_ARG, "dem_set_liquid_model: null argument");
  if (m->mode != DEM_LIQUID_REFERENCE && m->mode != DEM_LIQUID_PER_CONTACT)
    return fail(DEM_ERR_ARG, "dem_set_liquid_model: unknown mode " + std::to_string(m->mode));
  if (m->mode == DEM_LIQUID_PER_CONTACT &&
      !(m->vol_min > 0.0 && m->vol_max >= m->vol_min && m->vol_max < 1.0 && m->theta_max >= 0.0 &&
        m->theta_max < 1.5707963267948966))
    return fail(DEM_ERR_ARG, "dem_set_liquid_model: need 0 < vol_min <= vol_max < 1 and 0 <= theta_max < pi/2");
  if (c->chain_state != 0 || c->graph_exec[0] || c->graph_exec[1] || c->graph_one[0] || c->graph_one[1])
    return fail(DEM_ERR_STATE, "dem_set_liquid_model: set the liquid model before the first dem_step");
  c->lm.mode = m->mode;
  c->lm.vol_min = m->vol_min;
  c->lm.vol_max = m->vol_max;
  c->lm.theta_max = (float)m->theta_max;
  c->lm.seed = m->seed;
  /* the learned closure's contact-angle input is the same per-particle angle */
  if (m->mode == DEM_LIQUID_PER_CONTACT) {
    c->theta_max = (float)m->theta_max;
    c->theta_seed = m->seed;
  }
  return DEM_OK;
}

extern "C" dem_status dem_set_state(dem_ctx* c, const double3* pos, const double3* vel, const double3* angvel) {
  return dem_set_state_ex(c, pos, vel, angvel, 1);
}

namespace {
/* The state import (dem_set_state_ex).  wait: return once the caller's arrays
 * have been read; otherwise return with the reads queued on the context's
 * stream (dem_advance, which waits at its end). */
dem_status state_import(dem_ctx* c, const double3* pos, const double3* vel, const double3* angvel,
                        int request_rebuild, bool wait) {
  if (!c || !pos) return fail(DEM_ERR_ARG, "dem_set_state: null argument");
  const size_t N = (size_t)c->n;
  EngineBufs& b = c->b;
  if (c->trace) cudaEventRecord(c->trace[0], c->stream);
  /* page-locked caller arrays: one kernel reads them over the host link and
   * writes the cell-ordered state (and, mixed, its shadows) directly */
  const size_t bytes = sizeof(double3) * N;
  const double3* mp = static_cast<const double3*>(mapped_view(pos, bytes));
  const double3* mv = vel ? static_cast<const double3*>(mapped_view(vel, bytes)) : nullptr;
  const double3* mw = angvel ? static_cast<const double3*>(mapped_view(angvel, bytes)) : nullptr;
  if (mp && (!vel || mv) && (!angvel || mw)) {
    if (!request_rebuild && c->opt.precision == DEM_PREC_MIXED) {
      dem_status st = mixed_import_mapped(c, c->parity, b.inv, mp, mv, mw, c->stream);
      if (st != DEM_OK) return st;
    } else {
      k_import_mapped<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, b.inv, mp, mv, mw, b.pos, b.vel, b.angv);
    }
    /* the event the host waits on comes last, so the trace's are done too */
    cudaError_t e = cudaSuccess;
    if (c->trace) e = cudaEventRecord(c->trace[1], c->stream);
    if (e == cudaSuccess && c->trace) e = cudaEventRecord(c->trace[2], c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->xev[0], c->stream);
    if (e == cudaSuccess && request_rebuild) {
      const int one = 1;
      e = cudaMemcpyAsync(b.need, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream);
    }
    if (e != cudaSuccess) return cuda_check(e, "dem_set_state import");
    /* the caller's arrays are free again once the import has read them */
    return wait ? cuda_check(cudaEventSynchronize(c->xev[0]), "dem_set_state") : DEM_OK;
  }
  /* other host arrays (caller order) go to the tmp buffers (copy engine),
   * then a gather by id into cell order */
  cudaError_t e = cudaMemcpyAsync(b.tmp_pos, pos, sizeof(double3) * N, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && vel) e = cudaMemcpyAsync(b.tmp_vel, vel, sizeof(double3) * N, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && angvel)
    e = cudaMemcpyAsync(b.tmp_angv, angvel, sizeof(double3) * N, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess && c->trace) e = cudaEventRecord(c->trace[1], c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->xev[0], c->stream);
  if (e != cudaSuccess) return cuda_check(e, "dem_set_state upload");
  if (!request_rebuild && c->opt.precision == DEM_PREC_MIXED) {
    /* the neighbours read the shadow copy: the import refreshes it from the
     * new state in the same pass */
    dem_status st = mixed_import(c, c->parity, vel != nullptr, angvel != nullptr, c->stream);
    if (st != DEM_OK) return st;
  } else {
    k_import<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, b.id, b.tmp_pos, b.tmp_vel, b.tmp_angv, b.pos,
                                                           b.vel, b.angv, vel != nullptr, angvel != nullptr);
  }
  if (request_rebuild) {
    const int one = 1;
    e = cudaMemcpyAsync(b.need, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_check(e, "dem_set_state");
  }
  if (c->trace) cudaEventRecord(c->trace[2], c->stream);
  /* the caller's arrays are free again once the copies are done; the import
   * and the shadows run on behind them, ahead of the next step */
  if (!wait) return DEM_OK;
  e = cudaEventSynchronize(c->xev[0]);
  return cuda_check(e, "dem_set_state");
}
}  // namespace

extern "C" dem_status dem_set_state_ex(dem_ctx* c, const double3* pos, const double3* vel, const double3* angvel,
                                       int request_rebuild) {
  return state_import(c, pos, vel, angvel, request_rebuild, true);
}

extern "C" dem_status dem_advance(dem_ctx* c, double3* pos, double3* vel, double3* angvel, double3* force,
                                  int nsteps) {
  if (!c || !pos || nsteps < 0) return fail(DEM_ERR_ARG, "dem_advance: bad argument");
  /* import, steps and export queued back to back on the context's stream;
   * the host waits once, for the export */
  dem_status st = state_import(c, pos, vel, angvel, 0, false);
  if (st == DEM_OK) st = dem_step(c, nsteps);
  if (st == DEM_OK) st = dem_get_state(c, pos, vel, angvel, force, nullptr);
  return st;
}

extern "C" dem_status dem_get_state(dem_ctx* c, double3* pos, double3* vel, double3* angvel, double3* force,
                                    double3* mom) {
  if (!c) return fail(DEM_ERR_ARG, "dem_get_state: null context");
  EngineBufs& b = c->b;
  const size_t N = (size_t)c->n;
  if (c->trace) cudaEventRecord(c->trace[4], c->stream);
  const bool mixed = c->opt.precision == DEM_PREC_MIXED;
  /* page-locked caller arrays: one kernel gathers every requested array
   * into caller order and writes it over the host link directly (mixed
   * precision: the forces from the step's FP32 totals, no moments) */
  {
    const size_t bytes = sizeof(double3) * N;
    double3* const host[5] = {pos, vel, angvel, force, mom};
    double3* view[5] = {};
    bool direct = pos || vel || angvel || force || mom;
    for (int k = 0; k < 5 && direct; k++) {
      if (!host[k]) continue;
      view[k] = static_cast<double3*>(mapped_view(host[k], bytes));
      direct = view[k] != nullptr;
    }
    if (direct) {
      const void* const dev[5] = {b.pos, b.vel, b.angv, mixed ? (const void*)mixed_force_shadow(c) : b.force,
                                  mixed ? nullptr : b.mom};
      const int kind[5] = {0, 0, 0, mixed ? 1 : 0, mixed ? 2 : 0};
      ExportSet x{};
      for (int k = 0; k < 5; k++) {
        if (!view[k]) continue;
        x.src[x.count] = dev[k];
        x.kind[x.count] = kind[k];
        x.dst[x.count] = reinterpret_cast<double*>(view[k]);
        x.count++;
      }
      const dim3 grid((unsigned)grid_for((3LL * c->n + 1) / 2, 256), (unsigned)x.count);
      k_export_mapped<<<grid, 256, 0, c->stream>>>(c->n, b.inv, x);
      cudaError_t e = cudaSuccess;
      if (c->trace) e = cudaEventRecord(c->trace[5], c->stream);
      if (e == cudaSuccess) e = cudaEventRecord(c->xev[6], c->stream);
      if (e != cudaSuccess) return cuda_check(e, "dem_get_state export");
      return cuda_check(cudaEventSynchronize(c->xev[6]), "dem_get_state");
    }
  }
  if (mixed && (force || mom)) {
    dem_status st = mixed_force_to_master(c, c->stream);
    if (st != DEM_OK) return st;
  }
  struct Item {
    double3* host;
    const double3* dev;
  } items[5] = {{pos, b.pos}, {vel, b.vel}, {angvel, b.angv}, {force, b.force}, {mom, b.mom}};
  /* caller order: each array gathered through the inverse of the cell order
   * into its own staging buffer on the compute stream; its copy to the host
   * starts on the copy stream as soon as that gather is done, while the next
   * array is gathered; the compute stream then waits for the copies (the
   * staging buffers are reused by the next import), the host for the last */
  double3* stage[5] = {b.tmp_pos, b.tmp_vel, b.tmp_angv, b.tmp_out, b.tmp_out + N};
  int k = 0;
  cudaError_t e = cudaSuccess;
  for (auto& it : items) {
    if (!it.host || e != cudaSuccess) continue;
    k_export_gather<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, b.inv, it.dev, stage[k]);
    e = cudaEventRecord(c->xev[1 + k], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->xfer, c->xev[1 + k], 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(it.host, stage[k], sizeof(double3) * N, cudaMemcpyDeviceToHost, c->xfer);
    k++;
  }
  if (e == cudaSuccess && c->trace) e = cudaEventRecord(c->trace[5], c->xfer);
  if (e == cudaSuccess) e = cudaEventRecord(c->xev[6], c->xfer);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->xev[6], 0);
  if (e != cudaSuccess) return cuda_check(e, "dem_get_state");
  return cuda_check(cudaEventSynchronize(c->xev[6]), "dem_get_state");
}

namespace {
dem_status step_calls(dem_ctx* c, int nsteps);
}

extern "C" dem_status dem_step(dem_ctx* c, int nsteps) {
  if (!c || nsteps < 0) return fail(DEM_ERR_ARG, "dem_step: bad argument");
  dem_status st = step_calls(c, nsteps);
  if (st == DEM_OK && c->trace) cudaEventRecord(c->trace[3], c->stream);
  return st;
}

namespace {
dem_status step_calls(dem_ctx* c, int nsteps) {
  dem_status st = DEM_OK;
  int left = nsteps;
  if (c->opt.use_graph && c->opt.precision == DEM_PREC_MIXED && c->n > 0 && c->chain_state >= 0 && nsteps > 0) {
    /* steps chained on the device: one host launch for the whole call */
    if (c->chain_state == 0) {
      st = build_chain(c);
      if (st == DEM_OK) {
        c->chain_state = 1;
      } else {
        /* this device or driver cannot launch these graphs from the device:
         * keep the conditional-node graphs */
        destroy_graph(c);
        c->chain_state = -1;
        cudaGetLastError();
      }
    }
    if (c->chain_state == 1) {
      const int p = c->parity;
      cudaError_t e;
      if (nsteps == 1) {
        /* the host-instantiated copy: it starts sooner, its k_chain
         * tail-launches the device graphs (rebuild, the step again) all the
         * same, and work queued after it waits for them */
        e = cudaGraphLaunch(c->chain_single_host[p], c->stream);
      } else {
        /* a long chain runs ~1.5 us per step faster started from the
         * device-launch copy, which outweighs that copy's later start */
        st = chain_set_left(c->chain_ctl, nsteps, c->stream);
        if (st != DEM_OK) return st;
        e = cudaGraphLaunch(c->chain_step[p], c->stream);
      }
      if (e != cudaSuccess) return cuda_check(e, "cudaGraphLaunch");
      c->iter += nsteps;
      c->ctime += nsteps * c->s.sim.dt;
      c->parity ^= (nsteps & 1);
      return DEM_OK;
    }
  }
  if (c->opt.use_graph) {
    const int G = graph_len(c);
    const bool mixed = c->opt.precision == DEM_PREC_MIXED;
    while (left >= G) {
      const int p = mixed ? c->parity : 0;
      if (!c->graph_exec[p]) {
        st = build_graph(c, G, p, &c->graph_exec[p]);
        if (st != DEM_OK) return st;
      }
      cudaError_t e = cudaGraphLaunch(c->graph_exec[p], c->stream);
      if (e != cudaSuccess) return cuda_check(e, "cudaGraphLaunch");
      left -= G;
      c->iter += G;
      c->ctime += G * c->s.sim.dt;
      if (mixed && (G & 1)) c->parity ^= 1;
    }
  }
  /* the remainder, one-step graphs (the rebuild decided on the device) */
  while (c->opt.use_graph && left > 0) {
    const int p = c->opt.precision == DEM_PREC_MIXED ? c->parity : 0;
    if (!c->graph_one[p]) {
      st = build_graph(c, 1, p, &c->graph_one[p]);
      if (st != DEM_OK) return st;
    }
    cudaError_t e = cudaGraphLaunch(c->graph_one[p], c->stream);
    if (e != cudaSuccess) return cuda_check(e, "cudaGraphLaunch");
    left--;
    c->iter++;
    c->ctime += c->s.sim.dt;
    if (c->opt.precision == DEM_PREC_MIXED) c->parity ^= 1;
  }
  while (left > 0) {
    st = host_step(c);
    if (st != DEM_OK) return st;
    left--;
  }
  return DEM_OK;
}
}  // namespace

extern "C" dem_status dem_e2e_parts(dem_ctx* c, double3* pos, double3* vel, double3* angvel, double3* force,
                                    int reps, double* out) {
  if (!c || !pos || !vel || !angvel || !force || !out || reps <= 0)
    return fail(DEM_ERR_ARG, "dem_e2e_parts: bad argument");
  if (c->trace) return fail(DEM_ERR_STATE, "dem_e2e_parts: already tracing");
  cudaEvent_t ev[6] = {};
  cudaError_t e = cudaSuccess;
  for (cudaEvent_t& x : ev)
    if (e == cudaSuccess) e = cudaEventCreate(&x);
  if (e != cudaSuccess) {
    for (cudaEvent_t x : ev)
      if (x) cudaEventDestroy(x);
    return cuda_check(e, "dem_e2e_parts: cudaEventCreate");
  }
  double acc[9] = {};
  dem_status st = dem_sync(c);
  for (int r = 0; r < reps && st == DEM_OK; r++) {
    c->trace = ev;
    const auto t0 = std::chrono::steady_clock::now();
    st = dem_set_state_ex(c, pos, vel, angvel, 0);
    const auto t1 = std::chrono::steady_clock::now();
    if (st == DEM_OK) st = dem_step(c, 1);
    const auto t2 = std::chrono::steady_clock::now();
    if (st == DEM_OK) st = dem_get_state(c, pos, vel, angvel, force, nullptr);
    const auto t3 = std::chrono::steady_clock::now();
    c->trace = nullptr;
    if (st != DEM_OK) break;
    float ms[5] = {};
    e = cudaEventElapsedTime(&ms[0], ev[0], ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[1], ev[1], ev[2]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[2], ev[2], ev[3]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[3], ev[3], ev[4]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[4], ev[4], ev[5]);
    if (e != cudaSuccess) {
      st = cuda_check(e, "dem_e2e_parts: cudaEventElapsedTime");
      break;
    }
    const auto msd = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    acc[0] += msd(t0, t3);
    for (int k = 0; k < 5; k++) acc[1 + k] += ms[k];
    acc[6] += msd(t0, t1);
    acc[7] += msd(t1, t2);
    acc[8] += msd(t2, t3);
  }
  c->trace = nullptr;
  for (cudaEvent_t x : ev) cudaEventDestroy(x);
  if (st != DEM_OK) return st;
  for (int k = 0; k < 9; k++) out[k] = acc[k] / reps;
  return DEM_OK;
}

namespace dem {
namespace {
/* reads a buffer with 16-byte loads; the result is stored only under a
 * condition the data cannot meet, so the loads are kept */
__global__ void k_l2_read(const uint4* __restrict__ p, size_t n16, unsigned* __restrict__ sink) {
  unsigned acc = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x) {
    const uint4 v = p[i];
    acc ^= v.x ^ v.y ^ v.z ^ v.w;
  }
  if (acc == 0x9E3779B9u && sink) *sink = acc;
}
}  // namespace
}  // namespace dem

extern "C" dem_status dem_l2_flush(void* stream, void* buf, size_t bytes) {
  if (!buf || bytes < 64) return fail(DEM_ERR_ARG, "dem_l2_flush: bad buffer");
  cudaStream_t s = (cudaStream_t)stream;
  const size_t half = (bytes / 2) & ~(size_t)15;
  cudaError_t e = cudaMemsetAsync(buf, 0x5a, half, s);
  if (e != cudaSuccess) return cuda_check(e, "dem_l2_flush memset");
  dem::k_l2_read<<<152 * 8, 256, 0, s>>>((const uint4*)((char*)buf + half), half / 16, (unsigned*)buf);
  return cuda_check(cudaGetLastError(), "dem_l2_flush read");
}

extern "C" dem_status dem_profile_step(dem_ctx* c, int reps, void* flush_buf, size_t flush_bytes,
                                       double* ms_avg) {
  if (!c || reps <= 0 || !ms_avg) return fail(DEM_ERR_ARG, "dem_profile_step: bad argument");
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) return cuda_check(e, "dem_profile_step events");
  double total = 0.0;
  dem_status st = DEM_OK;
  for (int r = 0; r < reps && st == DEM_OK; r++) {
    if (flush_buf && flush_bytes) {
      st = dem_l2_flush(c->stream, flush_buf, flush_bytes);
      if (st != DEM_OK) break;
    }
    e = cudaEventRecord(e0, c->stream);
    if (e != cudaSuccess) {
      st = cuda_check(e, "dem_profile_step");
      break;
    }
    st = enqueue_step(c, c->stream, c->parity);
    if (st != DEM_OK) break;
    e = cudaEventRecord(e1, c->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e != cudaSuccess) {
      st = cuda_check(e, "dem_profile_step timing");
      break;
    }
    total += ms;
    if (c->opt.precision == DEM_PREC_MIXED) c->parity ^= 1;
    c->iter++;
    c->ctime += c->s.sim.dt;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == DEM_OK) *ms_avg = total / reps;
  return st;
}

extern "C" dem_status dem_profile_kernels(dem_ctx* c, dem_kernel_time* out, int max_out, int* n_out) {
  if (!c || !out || max_out <= 0 || !n_out) return fail(DEM_ERR_ARG, "dem_profile_kernels: bad argument");
  std::vector<std::pair<const char*, cudaEvent_t>> marks;
  cudaEvent_t e0;
  cudaError_t e = cudaEventCreate(&e0);
  if (e != cudaSuccess) return cuda_check(e, "dem_profile_kernels");
  /* one host-launched step with a forced rebuild, an event after each kernel */
  e = cudaMemsetAsync(c->b.flag, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->b.need, 0, sizeof(int), c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e0, c->stream);
  dem_status st = cuda_check(e, "dem_profile_kernels");
  c->marks = &marks;
  if (st == DEM_OK) st = enqueue_rebuild(c, c->stream, c->parity);
  if (st == DEM_OK) st = enqueue_step(c, c->stream, c->parity);
  if (st == DEM_OK) mark(c, c->stream, c->opt.precision == DEM_PREC_MIXED ? "step kernel" : "FP64 step kernels");
  c->marks = nullptr;
  if (st == DEM_OK) st = cuda_check(cudaStreamSynchronize(c->stream), "dem_profile_kernels sync");
  int k = 0;
  cudaEvent_t prev = e0;
  for (auto& m : marks) {
    float ms = 0.f;
    if (st == DEM_OK && k < max_out && cudaEventElapsedTime(&ms, prev, m.second) == cudaSuccess) {
      std::memset(out[k].name, 0, sizeof(out[k].name));
      std::strncpy(out[k].name, m.first, sizeof(out[k].name) - 1);
      out[k].ms = ms;
      k++;
    }
    prev = m.second;
  }
  for (auto& m : marks) cudaEventDestroy(m.second);
  cudaEventDestroy(e0);
  if (st != DEM_OK) return st;
  *n_out = k;
  if (c->opt.precision == DEM_PREC_MIXED) c->parity ^= 1;
  c->iter++;
  c->ctime += c->s.sim.dt;
  return DEM_OK;
}

extern "C" dem_status dem_sync(dem_ctx* c) {
  if (!c) return fail(DEM_ERR_ARG, "dem_sync: null context");
  k_check_finite<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->b.pos, c->b.vel, c->b.err);
  int err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, c->b.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_check(e, "dem_sync");
  if (err & 1) return fail(DEM_ERR_OVERFLOW, "a neighbour list ran past its level's slot capacity");
  if (err & 2) return fail(DEM_ERR_NONFINITE, "non-finite particle state");
  if (err & 4) return fail(DEM_ERR_CELL, "a particle left the cell grid");
  if (err & 8) return fail(DEM_ERR_CUDA, "a step chained on the device could not launch the next graph");
  return DEM_OK;
}

extern "C" dem_status dem_get_stats(dem_ctx* c, dem_stats* st) {
  if (!c || !st) return fail(DEM_ERR_ARG, "dem_get_stats: null argument");
  unsigned long long ctr[8];
  int err = 0;
  cudaError_t e = cudaMemcpyAsync(ctr, c->b.counters, sizeof(ctr), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, c->b.err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_check(e, "dem_get_stats");
  std::memset(st, 0, sizeof(*st));
  st->iter = c->iter;
  st->rebuilds = (long long)ctr[4];
  st->nb_entries = (long long)ctr[0];
  st->contacts = (long long)ctr[1];
  st->bridges = (long long)ctr[2];
  st->wall_contacts = (long long)ctr[3];
  st->error_bits = err;
  st->ctime = c->ctime;
  st->cap_mlp = (long long)ctr[5];
  st->cap_fallback = (long long)ctr[6];
  return DEM_OK;
}

/* one history slot as dispt.xyz, nDsp, nDsp_mx, plstRad, plstDfm, stage */
static void decode_record(const ContactRec& x, bool mixed, double* o) {
  if (mixed) {
    MixedRec m;
    std::memcpy(&m, &x, sizeof(m));
    o[0] = m.dx; o[1] = m.dy; o[2] = m.dz; o[3] = m.nDsp; o[4] = m.nDsp_mx; o[5] = m.plstRad;
    o[6] = m.plstDfm; o[7] = (double)m.stage;
  } else {
    o[0] = x.dx; o[1] = x.dy; o[2] = x.dz; o[3] = x.nDsp; o[4] = x.nDsp_mx; o[5] = x.plstRad;
    o[6] = x.plstDfm; o[7] = (double)(int)(x.stage & 0xffffffff);
  }
}

extern "C" dem_status dem_get_neighbors(dem_ctx* c, int* counts, int* partners, int max_per) {
  if (!c || !counts || !partners || max_per <= 0) return fail(DEM_ERR_ARG, "dem_get_neighbors: bad argument");
  const size_t N = (size_t)c->n, S = (size_t)c->slots;
  std::vector<int> nebor(S), num(N), nidx(N), plevel(N), id(N);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(nebor.data(), c->b.nebor, sizeof(int) * S, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(num.data(), c->b.num_nebor, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nidx.data(), c->b.nidx, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(plevel.data(), c->b.plevel, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(id.data(), c->b.id, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_check(e, "dem_get_neighbors");
  long long base[DEM_MAX_LEVELS];
  long long acc = 0;
  for (int l = 0; l < c->s.n_levels; l++) {
    base[l] = acc;
    acc += (long long)c->s.level_nnebors[l] * c->s.level_npars[l];
  }
  for (size_t q = 0; q < N; q++) {
    const int i = id[q], L = plevel[q];
    if (num[q] > max_per) return fail(DEM_ERR_ARG, "dem_get_neighbors: max_per too small");
    counts[i] = num[q];
    for (int a = 0; a < num[q]; a++) {
      const long long sl = base[L] + (long long)a * c->s.level_npars[L] + nidx[q];
      partners[(size_t)i * max_per + a] = id[nebor[sl]];
    }
  }
  return DEM_OK;
}

extern "C" dem_status dem_get_history(dem_ctx* c, double* rec, int* brg, int max_per) {
  if (!c || !rec || max_per <= 0) return fail(DEM_ERR_ARG, "dem_get_history: bad argument");
  const size_t N = (size_t)c->n, S = (size_t)c->slots;
  std::vector<ContactRec> r(S);
  std::vector<unsigned char> bf(S);
  std::vector<int> num(N), nidx(N), plevel(N), id(N);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(r.data(), c->b.rec, sizeof(ContactRec) * S, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(bf.data(), c->b.brg, S, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(num.data(), c->b.num_nebor, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nidx.data(), c->b.nidx, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(plevel.data(), c->b.plevel, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(id.data(), c->b.id, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_check(e, "dem_get_history");
  long long base[DEM_MAX_LEVELS];
  long long acc = 0;
  for (int l = 0; l < c->s.n_levels; l++) {
    base[l] = acc;
    acc += (long long)c->s.level_nnebors[l] * c->s.level_npars[l];
  }
  for (size_t q = 0; q < N; q++) {
    const int i = id[q], L = plevel[q];
    if (num[q] > max_per) return fail(DEM_ERR_ARG, "dem_get_history: max_per too small");
    for (int a = 0; a < num[q]; a++) {
      const long long sl = base[L] + (long long)a * c->s.level_npars[L] + nidx[q];
      double* o = rec + ((size_t)i * max_per + a) * 8;
      decode_record(r[(size_t)sl], c->opt.precision == DEM_PREC_MIXED, o);
      if (brg) brg[(size_t)i * max_per + a] = bf[(size_t)sl];
    }
  }
  return DEM_OK;
}

extern "C" dem_status dem_get_aux(dem_ctx* c, double* pmove, int* lqd, int* nwall, int* wlist, double* wrec,
                                  int* flag) {
  if (!c) return fail(DEM_ERR_ARG, "dem_get_aux: null context");
  const size_t N = (size_t)c->n;
  if (c->opt.precision == DEM_PREC_MIXED) {
    dem_status st = mixed_force_to_master(c, c->stream);
    if (st != DEM_OK) return st;
  }
  std::vector<double> pm(N);
  std::vector<int> lq(N), nw(N), wl(3 * N), id(N);
  std::vector<ContactRec> wr(3 * N);
  int fl = 0;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e == cudaSuccess) e = cudaMemcpy(pm.data(), c->b.pmove, sizeof(double) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(lq.data(), c->b.lqd, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nw.data(), c->b.nwall, sizeof(int) * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(wl.data(), c->b.wlist, sizeof(int) * 3 * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(wr.data(), c->b.wrec, sizeof(ContactRec) * 3 * N, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(id.data(), c->b.id, sizeof(int) * N, cudaMemcpyDeviceToHost);
  int nd = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&fl, c->b.flag, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&nd, c->b.need, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_check(e, "dem_get_aux");
  /* a step chained on the device hands its move flag on as the rebuild
   * request: either one means the next step rebuilds first */
  if (fl <= 0 && nd != 0) fl = 1;
  for (size_t q = 0; q < N; q++) {
    const int i = id[q];
    if (pmove) pmove[i] = pm[q];
    if (lqd) lqd[i] = lq[q];
    if (nwall) nwall[i] = nw[q];
    for (int a = 0; a < 3; a++) {
      if (wlist) wlist[3 * (size_t)i + a] = wl[3 * q + a];
      if (wrec) {
        decode_record(wr[(size_t)a * N + q], c->opt.precision == DEM_PREC_MIXED, wrec + ((size_t)i * 3 + a) * 8);
      }
    }
  }
  if (flag) *flag = fl;
  return DEM_OK;
}

/* ---------------- checkpoint ---------------- */
namespace {
struct Blob {
  void* dev;
  size_t bytes;
};
std::vector<Blob> checkpoint_blobs(dem_ctx* c) {
  EngineBufs& b = c->b;
  const size_t N = (size_t)c->n, S = (size_t)c->slots;
  return {{b.pos, sizeof(double3) * N}, {b.vel, sizeof(double3) * N}, {b.angv, sizeof(double3) * N},
          {b.rad, sizeof(double) * N},  {b.pmove, sizeof(double) * N}, {b.lqd, sizeof(int) * N},
          {b.id, sizeof(int) * N},      {b.plevel, sizeof(int) * N},   {b.nidx, sizeof(int) * N},
          {b.nebor, sizeof(int) * S},   {b.num_nebor, sizeof(int) * N}, {b.wlist, sizeof(int) * 3 * N},
          {b.nwall, sizeof(int) * N},   {b.rec, sizeof(ContactRec) * S}, {b.brg, S},
          {b.wrec, sizeof(ContactRec) * 3 * N}, {b.flag, sizeof(int)}, {b.need, sizeof(int)},
          {b.cyl, sizeof(CylinderBC)}, {b.counters, sizeof(unsigned long long) * 8}};
}
const char kMagic[8] = {'D', 'E', 'M', 'G', 'B', '3', '0', '1'};
}  // namespace

extern "C" dem_status dem_save(dem_ctx* c, const char* path, int nBatch) {
  if (!c || !path) return fail(DEM_ERR_ARG, "dem_save: null argument");
  dem_status st = DEM_OK;
  if (c->b.sys_of_id) return fail(DEM_ERR_STATE, "dem_save: checkpoints of batched systems are not supported");
  if (c->opt.precision == DEM_PREC_MIXED && c->parity != 0)
    return fail(DEM_ERR_STATE, "dem_save: call after an even number of steps");
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_check(e, "dem_save");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(DEM_ERR_IO, std::string("cannot write ") + path);
  /* the text header LoadPara reads (DumpLoad.cpp:14-17) */
  std::fprintf(f, "SYSTEM Info\n%d %d %d\n", c->n, nBatch, c->n);
  std::fwrite(kMagic, 1, 8, f);
  long long hdr[4] = {c->iter, (long long)c->n, c->slots, (long long)c->opt.precision};
  std::fwrite(hdr, sizeof(hdr), 1, f);
  std::fwrite(&c->ctime, sizeof(double), 1, f);
  for (const Blob& bl : checkpoint_blobs(c)) {
    std::vector<char> h(bl.bytes);
    e = cudaMemcpy(h.data(), bl.dev, bl.bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
      st = cuda_check(e, "dem_save copy");
      break;
    }
    if (std::fwrite(h.data(), 1, bl.bytes, f) != bl.bytes) {
      st = fail(DEM_ERR_IO, "dem_save: short write");
      break;
    }
  }
  std::fclose(f);
  return st;
}

extern "C" dem_status dem_load(dem_ctx* c, const char* path) {
  if (!c || !path) return fail(DEM_ERR_ARG, "dem_load: null argument");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(DEM_ERR_IO, std::string("cannot read ") + path);
  int np = 0, nb = 0, tp = 0;
  char line[64];
  if (!std::fgets(line, sizeof(line), f) || std::strncmp(line, "SYSTEM Info", 11) != 0 ||
      std::fscanf(f, "%d %d %d", &np, &nb, &tp) != 3 || std::fgetc(f) != '\n') {
    std::fclose(f);
    return fail(DEM_ERR_IO, "dem_load: bad header");
  }
  char magic[8];
  long long hdr[4];
  double ct = 0.0;
  if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, kMagic, 8) != 0 || std::fread(hdr, sizeof(hdr), 1, f) != 1 ||
      std::fread(&ct, sizeof(double), 1, f) != 1) {
    std::fclose(f);
    return fail(DEM_ERR_IO, "dem_load: bad binary header");
  }
  if (hdr[1] != c->n || hdr[2] != c->slots || hdr[3] != c->opt.precision) {
    std::fclose(f);
    return fail(DEM_ERR_ARG, "dem_load: checkpoint does not match this context");
  }
  dem_status st = DEM_OK;
  for (const Blob& bl : checkpoint_blobs(c)) {
    std::vector<char> h(bl.bytes);
    if (std::fread(h.data(), 1, bl.bytes, f) != bl.bytes) {
      st = fail(DEM_ERR_IO, "dem_load: truncated checkpoint");
      break;
    }
    cudaError_t e = cudaMemcpy(bl.dev, h.data(), bl.bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      st = cuda_check(e, "dem_load copy");
      break;
    }
  }
  std::fclose(f);
  if (st != DEM_OK) return st;
  c->iter = hdr[0];
  c->ctime = ct;
  c->parity = 0;
  k_inverse<<<grid_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->b.id, c->b.inv);
  if (c->opt.precision == DEM_PREC_MIXED) st = mixed_shadows(c, 0, c->stream);
  if (st == DEM_OK) st = cuda_check(cudaStreamSynchronize(c->stream), "dem_load sync");
  return st;
}
