/*
 * dem_internal.h -- declarations shared by the translation units of libdem_gb300.
 * Not part of the public ABI (include/heydem_gb300.h is).
 */
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "heydem_gb300.h"
#include "liquid.cuh"

namespace dem {

/* ---------------- errors ---------------- */
void set_error(const std::string& msg);
bool last_error_empty();
dem_status fail(dem_status code, const std::string& msg);
/* cudaError -> DEM_ERR_CUDA with a message naming the call site */
dem_status cuda_check(cudaError_t e, const char* what);
/* reference-compatible failure: print like cutilSafeCall (heydem.h:28-35) and exit(-1) */
void ref_check(cudaError_t e, const char* file, int line);
#define DEM_REF_CHECK(x) ::dem::ref_check((x), __FILE__, __LINE__)

dem_status cuda_alloc(void** p, size_t bytes);

/* ---------------- host set-up helpers (host_io.cpp) ---------------- */
dem_status read_diameters(const char* path, double* hRad, int np);
void unit_reduce(dem_setup* s, double* hRad, int np, double gravity);
void derive_contact_constants(dem_setup* s);

/* ---------------- device-side parameter blocks (passed by value) ---------------- */

/* the constant-memory set of the reference (kernel.cu:15-19) */
struct DevConsts {
  MatType mat[2];
  LIQUID lqd;
  PARAMETER prm;
  calParaPP cal;
  calParaPP pwcal;
};

/* per-level search tables; device pointers (the reference keeps them in
 * device memory: d_cell, d_Ncell_Idx, d_Level_size, d_level_nPars,
 * d_level_nNebors) */
struct LevelView {
  const double* cell_size;
  const int3* grid_size;
  const int* ncell_idx; /* inclusive scan of cells per level */
  const double* level_size;
  const int* level_npars;
  const int* level_nnebors;
  int n_levels;
};

/* contact history, reference layout (heydem.h:153-190, the fields in use) */
struct HistSoA {
  double3* dispt;
  double* nDsp;
  double* nDsp_mx;
  double* plstRad;
  double* plstDfm;
  int* stage;
  int* lqdBrg;
};

/* one contact slot of the engine's history: dispt (3), nDsp, nDsp_mx,
 * plstRad, plstDfm, then the load stage in the low 32 bits of the last word.
 * 64 bytes = two DRAM sectors per contact. */
struct __align__(16) ContactRec {
  double dx, dy, dz, nDsp, nDsp_mx, plstRad, plstDfm;
  long long stage;
};
static_assert(sizeof(ContactRec) == 64, "ContactRec must be 64 bytes");

/* The same 64-byte slot as the mixed-precision path lays it out: the tangential
 * spring and the maximum overlap stay FP64 (they accumulate / are maxima over
 * the contact's life); an FP32 copy of the spring feeds the FP32 contact math;
 * the fields re-derived every step (current overlap, plastic radius and
 * offset) are FP32. */
struct __align__(16) MixedRec {
  double dx, dy, dz, nDsp_mx;
  float fx, fy, fz, nDsp;
  float plstRad, plstDfm;
  int stage, pad;
};
static_assert(sizeof(MixedRec) == 64, "MixedRec must be 64 bytes");

/* history in the engine's layout */
struct HistAoS {
  ContactRec* rec;
  unsigned char* brg; /* bridge flag per slot (NULL for walls) */
};

/* ---------------- kernel launchers (build.cu) ---------------- */

/* scratch the cell sort needs: 2*np + cells + block sums ints */
size_t sort_scratch_bytes(int np, int ncells);

/* Cell hash + stable counting sort + CellStart/CellEnd in one pass sequence.
 *   pos (AoS double3, n particles), plevel, order_key: the particle id the
 *   stable order uses for ties (NULL: the index itself).
 * Outputs sorted hash / sorted source index (position in the input arrays),
 * cell_start/cell_end (-1 for empty cells) and, if cell_off is not NULL,
 * every cell's offset in sorted order (ncells + 1 ints, the total last).
 * scratch must hold sort_scratch_bytes(n, ncells).  A hash outside
 * [0, ncells) sets bit 4 of *err (may be NULL).  Every launch goes to
 * `stream`. */
dem_status cell_sort(const double3* pos, const int* plevel, const int* order_key, int n,
                     LevelView lv, const DevConsts& k, int ncells, int* sorted_hash,
                     int* sorted_src, int* cell_start, int* cell_end, void* scratch, int* err,
                     cudaStream_t stream, int* cell_off = nullptr);

/* FP32 prefilter of the neighbour test (see build.cu): the high floats of
 * (position + offset, radius) and the bound of their distance error */
struct Prefilter {
  const float4* hi;
  float tol;
};

/* NeighborFindG semantics (kernel.cu:729-855) on AoS positions; sorted_src
 * maps sorted position -> particle index; writes the level/slot-major list.
 * Slot overflow sets bit 1 of *err and stops appending.  cell_off (from
 * cell_sort, may be NULL) lets a cell row's range be read with two loads. */
dem_status neighbor_find(const double3* pos, const double* rad, const int* sorted_src,
                         const int* cell_start, const int* cell_end, const int* plevel,
                         const int* nebor_idx, LevelView lv, const DevConsts& k, int* nebor,
                         int* num_nebor, int n, int* err, cudaStream_t stream,
                         Prefilter pre = Prefilter{nullptr, 0.f}, const int* cell_off = nullptr);

/* CirWallListG (kernel.cu:1034-1073); wall list pitched rows.  Batched
 * systems: sys_of_id[id[i]] selects particle i's cylinder in cyl[] (NULL: cyl[0]). */
dem_status wall_list(const double3* pos, const double* rad, const CylinderBC* cyl, int* wlist,
                     size_t pitch, int* nwall, int n, const DevConsts& k, cudaStream_t stream,
                     const int* id = nullptr, const int* sys_of_id = nullptr);

/* HstryCopyG (kernel.cu:869-911).  For re-ordered particles: old_src maps a
 * particle's new index to its previous index (NULL: unchanged), nebor_idx_old
 * holds the previous level ranks, and old_to_new translates partner indices of
 * the previous list (NULL: unchanged). */
dem_status history_carry_pp(const int* nebor, const int* nebor_old, const int* plevel,
                            const int* nebor_idx, const int* nebor_idx_old, const int* level_npars,
                            const int* level_nnebors, HistSoA old_h, HistSoA cur_h,
                            const int* num_nebor, const int* num_nebor_old, const int* old_src,
                            const int* old_to_new, int n, cudaStream_t stream);
/* HstryCopyPWG (kernel.cu:918-950); old_src maps new index -> old index */
dem_status history_carry_pw(const int* wlist, size_t pitch, const int* wlist_old, size_t pitch_old,
                            HistSoA old_h, HistSoA cur_h, const int* nwall, const int* nwall_old,
                            const int* old_src, int n, int NP_new, int NP_old,
                            cudaStream_t stream);
/* PPCntHstryCopy / WallCntHstryCopy (ParticleSystem.cu:336-375): old <- cur, cur <- 0 */
dem_status history_rotate(HistSoA old_h, HistSoA cur_h, long long count, cudaStream_t stream);

/* ---------------- FP64 step kernels (step64.cu) ---------------- */

/* VarInit (Allocation.cpp:308-317) as one kernel */
dem_status var_init(double3* force, double3* mom, double* rmom, int* lqd, int* lqd_old, int n,
                    cudaStream_t stream);
/* PPForceCalcG (kernel.cu:413-552); H = HistSoA (reference layout) or HistAoS.
 * lm: the liquid model (mode 0: the reference's); id: each particle's caller
 * id for the per-contact model's hashes (NULL: the index itself) */
template <class H>
dem_status pp_force64(const double3* pos, const double3* vel, const double3* angvel,
                      const double* rad, const int* nebor, const int* plevel,
                      const int* level_npars, const int* level_nnebors, const int* nebor_idx,
                      H h, const int* num_nebor, int* lqd, const int* lqd_old,
                      double3* force, double3* mom, double* rmom, int n, int force_cap, int stage,
                      const DevConsts& k, unsigned long long* counters, double* pvol, cudaStream_t stream,
                      const int* id = nullptr, LiquidModel lm = LiquidModel{0, 0.f, 0.0, 0.0, 0ull});
/* CirPWInterG (kernel.cu:958-1023).  move_wall: advance the top wall first
 * (the reference's particle-0 thread does this inside the kernel). */
template <class H>
dem_status wall_force64(const double3* pos, const double3* vel, const double3* angvel,
                        double3* force, double3* mom, double* rmom, const double* rad,
                        CylinderBC* cyl, H h, const int* nwall, const int* wlist,
                        size_t pitch, int n, int NP, int stage, const DevConsts& k,
                        unsigned long long* counters, bool move_wall, cudaStream_t stream);
/* UpdateSystemG (kernel.cu:563-606) */
dem_status update64(const double* rad, double3* pos, double3* vel, double3* angvel,
                    const double3* force, const double3* mom, double* rmom, int* flag,
                    double* pmove, int n, const DevConsts& k, cudaStream_t stream);

/* PpInterCalc / CirPWCalc / UpdateSystem in mixed precision on the reference's layouts
 * (mixed.cu): FP32 laws and bridges with Kahan sums, FP64 positions, springs
 * and peak overlaps; the reference's liquid model.  The wall call moves the
 * top wall first, as wall_force64 with move_wall does. */
dem_status pp_force_ref_mixed(const double3* pos, const double3* vel, const double3* angvel, const double* rad,
                              const int* nebor, const int* plevel, const int* level_npars, const int* level_nnebors,
                              const int* nebor_idx, HistSoA h, const int* num_nebor, int* lqd, const int* lqd_old,
                              double3* force, double3* mom, double* rmom, int n, int force_cap, int stage,
                              const DevConsts& k, cudaStream_t s);
dem_status wall_force_ref_mixed(const double3* pos, const double3* vel, const double3* angvel, double3* force,
                                double3* mom, double* rmom, const double* rad, CylinderBC* cyl, HistSoA h,
                                const int* nwall, const int* wlist, size_t pitch, int n, int NP, int stage,
                                const DevConsts& k, cudaStream_t s);
/* UpdateSystemG in the same mode: FP32 increments (mass, inertia, dv, dw,
 * path length) added to the FP64 state, as the fused step integrates */
dem_status update_ref_mixed(const double* rad, double3* pos, double3* vel, double3* angvel, const double3* force,
                            const double3* mom, double* rmom, int* flag, double* pmove, int n, const DevConsts& k,
                            cudaStream_t s);

/* device-level helpers */
dem_status inclusive_scan_small(const int* in, int* out, int n, cudaStream_t stream);

}  // namespace dem
