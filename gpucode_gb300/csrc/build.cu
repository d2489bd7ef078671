/*
 * build.cu -- neighbour-list rebuild kernels (sm_103a).
 *
 * Replaces the reference's rebuild chain (ParticleSystem.cu:141-163):
 * calcHashG -> thrust::sort_by_key -> reorderDataAndFindCellStartG ->
 * NeighborFindG, plus CirWallListG and the history carry-over kernels.
 *
 * The cell sort is a stable counting sort over cells instead of a radix sort
 * over hashes: (1) hash each particle and take an arrival rank in its cell with
 * one atomic, (2) exclusive-scan the per-cell counts (three-phase, no
 * inter-block waiting), which gives CellStart/CellEnd directly -- the
 * reference's two 0xff memsets and the boundary kernel disappear, (3) scatter
 * to sorted positions, (4) put each cell's few particles back into ascending
 * particle-id order so ties come out exactly as thrust's stable sort leaves
 * them.  The per-cell count lives in the CellEnd array until the scan
 * overwrites it, so the only scratch is two ints per particle plus one per
 * scan tile.
 *
 * The neighbour search keeps the reference's traversal order (level, z, y,
 * x-row of cells, sorted order inside the row) so lists match it entry for
 * entry, and evaluates the distance test in plain IEEE FP64 (this file is
 * compiled with -fmad=false) so the integer output is bit-exact.
 */
#include <cuda_runtime.h>

#include "dem_device.cuh"

namespace dem {

namespace {

constexpr int kRowBatch = 8; /* cell rows whose ranges the neighbour search reads at once */
constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread; /* cells per scan tile */

inline int div_up(long long a, long long b) { return (int)((a + b - 1) / b); }

/* (1) hash + arrival rank; count[] aliases cell_end[] and is zero on entry */
__global__ void k_hash_count(const double3* __restrict__ pos, const int* __restrict__ plevel, int n,
                             LevelView lv, double3 origin, int ncells, int* __restrict__ key,
                             int* __restrict__ rank, int* __restrict__ count, int* __restrict__ err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int lvl = plevel[i];
  int h = grid_hash(grid_pos(pos[i], lvl, lv, origin), lvl, lv);
  if (lvl != 0) h += lv.ncell_idx[lvl - 1];
  /* the reference clamps to gridSize (not gridSize-1, kernel.cu:627-629), so a
   * particle on the far face of the last level's grid hashes past the end; it
   * would write out of bounds there.  Flag it and keep it in the last cell. */
  if (h < 0 || h >= ncells) {
    if (err) atomicOr(err, 4);
    h = ncells - 1;
  }
  key[i] = h;
  rank[i] = atomicAdd(&count[h], 1);
}

/* block-wide exclusive scan of one int per thread; returns the block total */
__device__ __forceinline__ int block_exclusive_scan(int v, int& total) {
  __shared__ int warp_tot[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int t = lane < kScanThreads / 32 ? warp_tot[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < kScanThreads / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  const int warp_prefix = warp > 0 ? warp_tot[warp - 1] : 0;
  total = warp_tot[kScanThreads / 32 - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

/* (2a) per-tile totals */
__global__ void k_tile_sums(const int* __restrict__ count, int ncells, int* __restrict__ tile_sum) {
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPerThread;
  int s = 0;
#pragma unroll
  for (int e = 0; e < kScanPerThread; e++) {
    long long c = base + e;
    if (c < ncells) s += count[c];
  }
  int total;
  block_exclusive_scan(s, total);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

/* (2b) exclusive scan of the tile totals by one block (in place) */
__global__ void k_scan_tiles(int* __restrict__ tile_sum, int ntiles) {
  int carry = 0;
  for (int base = 0; base < ntiles; base += kScanThreads) {
    const int t = base + threadIdx.x;
    const int v = t < ntiles ? tile_sum[t] : 0;
    int total;
    const int ex = block_exclusive_scan(v, total);
    if (t < ntiles) tile_sum[t] = carry + ex;
    carry += total;
    __syncthreads();
  }
}

/* (2c) cell offsets -> CellStart / CellEnd (-1 for empty cells); count[] is
 * read from cell_end[] and overwritten in place.  cell_off (optional, ncells
 * + 1 entries) receives every cell's offset, empty or not, and the total */
__global__ void k_cell_ranges(int* __restrict__ cell_start, int* __restrict__ cell_end, int ncells,
                              const int* __restrict__ tile_off, int* __restrict__ cell_off) {
  const long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanPerThread;
  int c[kScanPerThread];
  int s = 0;
#pragma unroll
  for (int e = 0; e < kScanPerThread; e++) {
    long long q = base + e;
    c[e] = q < ncells ? cell_end[q] : 0;
    s += c[e];
  }
  int total;
  int off = block_exclusive_scan(s, total) + tile_off[blockIdx.x];
#pragma unroll
  for (int e = 0; e < kScanPerThread; e++) {
    long long q = base + e;
    if (q < ncells) {
      cell_start[q] = c[e] ? off : -1;
      cell_end[q] = c[e] ? off + c[e] : -1;
      if (cell_off) {
        cell_off[q] = off;
        if (q == ncells - 1) cell_off[ncells] = off + c[e];
      }
    }
    off += c[e];
  }
}

/* (3) scatter to sorted positions */
__global__ void k_scatter(const int* __restrict__ key, const int* __restrict__ rank, int n,
                          const int* __restrict__ cell_start, int* __restrict__ sorted_hash,
                          int* __restrict__ sorted_src) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int h = key[i];
  const int q = cell_start[h] + rank[i];
  sorted_hash[q] = h;
  sorted_src[q] = i;
}

/* (4) the first slot of each cell orders its cell by particle id (insertion
 * sort; cells hold a handful of particles) */
__global__ void k_cell_order(const int* __restrict__ sorted_hash, int* __restrict__ sorted_src,
                             const int* __restrict__ cell_start, const int* __restrict__ cell_end,
                             const int* __restrict__ order_key, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int h = sorted_hash[q];
  if (cell_start[h] != q) return;
  const int e = cell_end[h];
  for (int a = q + 1; a < e; a++) {
    const int v = sorted_src[a];
    const int kv = order_key ? order_key[v] : v;
    int b = a - 1;
    while (b >= q) {
      const int u = sorted_src[b];
      const int ku = order_key ? order_key[u] : u;
      if (ku <= kv) break;
      sorted_src[b + 1] = u;
      b--;
    }
    sorted_src[b + 1] = v;
  }
}

/* NeighborFindG (kernel.cu:729-855).  sorted_src == NULL means the particle
 * arrays are themselves in sorted order.
 *
 * Optional prefilter (pre.hi != NULL, particle arrays in sorted order): pre.hi
 * holds (x, y, z, r) as the high floats of (coordinate + offset) with every
 * coordinate in one binade, so hi_i - hi_j is exact in FP32; the FP32 distance
 * from those differences is within pre.tol of the exact one.  A candidate
 * farther than pre.tol from the cut-off is decided in FP32; only the band
 * around it takes the reference's FP64 test, so the list is bit-identical to
 * the all-FP64 build while almost no FP64 square roots are taken.
 *
 * Optional cell_off (every cell's offset in sorted order, empty cells
 * included, and the total after the last): a row's particles are then
 * [cell_off[first cell], cell_off[last cell + 1]) -- the same range, in the
 * same order, from two loads instead of two per cell of the row.  The search
 * is bound by these scattered loads, not by its arithmetic. */
__global__ void k_neighbor_find(const double3* __restrict__ pos, const double* __restrict__ rad,
                                const int* __restrict__ sorted_src, const int* __restrict__ cell_start,
                                const int* __restrict__ cell_end, const int* __restrict__ cell_off,
                                const int* __restrict__ plevel,
                                const int* __restrict__ nebor_idx, LevelView lv, double3 origin,
                                double search_gap, int* __restrict__ nebor,
                                int* __restrict__ num_nebor, int n, int* __restrict__ err, Prefilter pre) {
  const int i = reversed_block_thread(); /* the largest spheres' long searches first */
  if (i >= n) return;
  const double3 o = pos[i];
  const double ri = rad[i];
  const float4 hi_i = pre.hi ? pre.hi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float sg = (float)search_gap;
  const int L = plevel[i];
  const long long base = slot_base(L, lv.level_npars, lv.level_nnebors) + nebor_idx[i];
  const long long stride = lv.level_npars[L];
  const int cap = lv.level_nnebors[L];
  int count = 0;
  bool over = false;
  /* candidate q (sorted position): the distance test, then the append */
  auto visit = [&](int q) {
    const int j = sorted_src ? sorted_src[q] : q;
    if (j == i) return;
    bool in = false, decided = false;
    if (pre.hi) {
      const float4 hj = pre.hi[j];
      const float dx = hi_i.x - hj.x, dy = hi_i.y - hj.y, dz = hi_i.z - hj.z;
      const float dc = sqrtf(dx * dx + dy * dy + dz * dz);
      const float cut = (hj.w + hi_i.w) + sg;
      if (dc > cut + pre.tol) decided = true; /* certainly outside */
      else if (dc < cut - pre.tol) {          /* certainly inside */
        decided = true;
        in = true;
      }
    }
    if (!decided) in = len3(sub3(o, pos[j])) < rad[j] + ri + search_gap;
    if (!in) return;
    if (count >= cap) {
      over = true;
      return;
    }
    nebor[base + (long long)count * stride] = j;
    count++;
  };
  for (int iL = 0; iL < lv.n_levels; iL++) {
    const int3 g = grid_pos(o, iL, lv, origin);
    const int off = (int)ceil(lv.level_size[L] / lv.level_size[iL]);
    const int cell_sum = iL != 0 ? lv.ncell_idx[iL - 1] : 0;
    const int3 gs = lv.grid_size[iL];
    if (cell_off) {
      /* rows r = (z + off) W + (y + off), in the reference's (z, y) order;
       * the ranges of kRowBatch rows are read with independent loads before
       * their particles are visited in order */
      const int W = 2 * off + 1, R = W * W;
      for (int r0 = 0; r0 < R; r0 += kRowBatch) {
        int rf[kRowBatch], rl[kRowBatch];
#pragma unroll
        for (int b = 0; b < kRowBatch; b++) {
          rf[b] = rl[b] = 0;
          const int r = r0 + b;
          const int z = r / W - off, y = r % W - off;
          int3 s = make_int3(g.x - off, g.y + y, g.z + z);
          int3 e = make_int3(g.x + off, g.y + y, g.z + z);
          if (s.x < 0) s.x = 0;
          if (e.x > gs.x - 1) e.x = gs.x - 1;
          if (r < R && !(s.y < 0 || s.z < 0 || s.y > gs.y - 1 || s.z > gs.z - 1) && e.x >= s.x) {
            const int row = grid_hash(s, iL, lv) + cell_sum;
            rf[b] = __ldg(cell_off + row);
            rl[b] = __ldg(cell_off + row + (e.x - s.x) + 1);
          }
        }
#pragma unroll
        for (int b = 0; b < kRowBatch; b++)
          for (int q = rf[b]; q < rl[b]; q++) visit(q);
      }
      continue;
    }
    for (int z = -off; z <= off; z++) {
      for (int y = -off; y <= off; y++) {
        int3 s = make_int3(g.x - off, g.y + y, g.z + z);
        int3 e = make_int3(g.x + off, g.y + y, g.z + z);
        if (s.x < 0) s.x = 0;
        if (e.x > gs.x - 1) e.x = gs.x - 1;
        if (s.y < 0 || s.z < 0 || s.y > gs.y - 1 || s.z > gs.z - 1) continue;
        /* the row's particles: from the start of its first non-empty cell to
         * the end of its last one (cells of a row are consecutive in sorted
         * order).  The reference walks in from both ends one dependent load
         * at a time (kernel.cu:775-790); every cell's range is read here
         * with independent loads -- the same range, the same append order. */
        int first = -1, last = -1;
        const int row = grid_hash(s, iL, lv) + cell_sum;
        for (int x = 0; x <= e.x - s.x; x++) {
          const int cs = __ldg(cell_start + row + x), ce = __ldg(cell_end + row + x);
          if (first == -1) first = cs;
          if (ce != -1) last = ce;
        }
        if (first == -1 || last == -1) continue;
        for (int q = first; q < last; q++) visit(q);
      }
    }
  }
  num_nebor[i] = count;
  if (over) atomicOr(err, 1);
}

/* CirWallListG (kernel.cu:1034-1073) */
__global__ void k_wall_list(const double3* __restrict__ pos, const double* __restrict__ rad,
                            const CylinderBC* __restrict__ cyl, int* __restrict__ wlist, size_t pitch,
                            int* __restrict__ nwall, int n, double search_gap, const int* __restrict__ id,
                            const int* __restrict__ sys_of_id) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double3 p = pos[i];
  const double r = rad[i];
  /* batched systems: each particle meets its own system's cylinder */
  const CylinderBC c = cyl[sys_of_id ? sys_of_id[id[i]] : 0];
  int* row = (int*)((char*)wlist + (size_t)i * pitch);
  int m = 0;
  if (p.z >= (c.Tw - (2.0 * r + search_gap))) row[m++] = 0;
  if (p.z <= ((2.0 * r + search_gap) + c.Bw)) row[m++] = 1;
  /* the reference writes pow(pow(dx, 2) + pow(dy, 2), 0.5): squares and a
   * square root, correctly rounded (glibc's pow returns exactly these values,
   * and this file is built without FMA contraction), at the cost of one
   * FP64 square root instead of three FP64 pow calls */
  const double dx = c.cir.x - p.x, dy = c.cir.y - p.y;
  const double dist = sqrt(dx * dx + dy * dy);
  if (dist >= c.R - (2.0 * r + search_gap)) row[m++] = 2;
  nwall[i] = m;
}

__device__ __forceinline__ void copy_slot(const HistSoA& dst, long long d, const HistSoA& src, long long s) {
  dst.dispt[d] = src.dispt[s];
  dst.nDsp[d] = src.nDsp[s];
  dst.nDsp_mx[d] = src.nDsp_mx[s];
  dst.plstRad[d] = src.plstRad[s];
  dst.plstDfm[d] = src.plstDfm[s];
  dst.stage[d] = src.stage[s];
  dst.lqdBrg[d] = src.lqdBrg[s];
}

/* HstryCopyG (kernel.cu:869-911), with optional re-indexing of the old list */
__global__ void k_carry_pp(const int* __restrict__ nebor, const int* __restrict__ nebor_old,
                           const int* __restrict__ plevel, const int* __restrict__ nebor_idx,
                           const int* __restrict__ nebor_idx_old, const int* __restrict__ level_npars,
                           const int* __restrict__ level_nnebors, HistSoA old_h, HistSoA cur_h,
                           const int* __restrict__ num_nebor, const int* __restrict__ num_nebor_old,
                           const int* __restrict__ old_src, const int* __restrict__ old_to_new, int n) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int p = old_src ? old_src[q] : q;
  const int L = plevel[q];
  const long long stride = level_npars[L];
  const long long lb = slot_base(L, level_npars, level_nnebors);
  const long long nb = lb + nebor_idx[q];
  const long long ob = lb + nebor_idx_old[p];
  const int nn = num_nebor[q], no = num_nebor_old[p];
  for (int a = 0; a < nn; a++) {
    const long long ine = nb + a * stride;
    const int partner = nebor[ine];
    for (int b = 0; b < no; b++) {
      const long long jne = ob + b * stride;
      int j = nebor_old[jne];
      if (old_to_new) j = old_to_new[j];
      if (j == partner) copy_slot(cur_h, ine, old_h, jne);
    }
  }
}

/* HstryCopyPWG (kernel.cu:918-950) */
__global__ void k_carry_pw(const int* __restrict__ wlist, size_t pitch, const int* __restrict__ wlist_old,
                           size_t pitch_old, HistSoA old_h, HistSoA cur_h, const int* __restrict__ nwall,
                           const int* __restrict__ nwall_old, const int* __restrict__ old_src, int n,
                           int np_new, int np_old) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int p = old_src ? old_src[q] : q;
  const int* row = (const int*)((const char*)wlist + (size_t)q * pitch);
  const int* orow = (const int*)((const char*)wlist_old + (size_t)p * pitch_old);
  for (int a = 0; a < nwall[q]; a++) {
    const int w = row[a];
    for (int b = 0; b < nwall_old[p]; b++)
      if (orow[b] == w) copy_slot(cur_h, (long long)a * np_new + q, old_h, (long long)b * np_old + p);
  }
}

/* old <- cur, cur <- 0 over count slots (PPCntHstryCopy / WallCntHstryCopy) */
__global__ void k_rotate(HistSoA old_h, HistSoA cur_h, long long count) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (long long)gridDim.x * blockDim.x) {
    old_h.dispt[i] = cur_h.dispt[i];
    old_h.nDsp[i] = cur_h.nDsp[i];
    old_h.nDsp_mx[i] = cur_h.nDsp_mx[i];
    old_h.plstRad[i] = cur_h.plstRad[i];
    old_h.plstDfm[i] = cur_h.plstDfm[i];
    old_h.stage[i] = cur_h.stage[i];
    old_h.lqdBrg[i] = cur_h.lqdBrg[i];
    cur_h.dispt[i] = make_double3(0.0, 0.0, 0.0);
    cur_h.nDsp[i] = 0.0;
    cur_h.nDsp_mx[i] = 0.0;
    cur_h.plstRad[i] = 0.0;
    cur_h.plstDfm[i] = 0.0;
    cur_h.stage[i] = 0;
    cur_h.lqdBrg[i] = 0;
  }
}

__global__ void k_scan_small(const int* __restrict__ in, int* __restrict__ out, int n) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int acc = 0;
    for (int i = 0; i < n; i++) {
      acc += in[i];
      out[i] = acc;
    }
  }
}

int grid_for(long long n, int block) { return n <= 0 ? 1 : div_up(n, block); }

}  // namespace

size_t sort_scratch_bytes(int np, int ncells) {
  const size_t tiles = (size_t)div_up(ncells, kScanTile);
  return sizeof(int) * (2 * (size_t)np + tiles + 64);
}

dem_status cell_sort(const double3* pos, const int* plevel, const int* order_key, int n, LevelView lv,
                     const DevConsts& k, int ncells, int* sorted_hash, int* sorted_src, int* cell_start,
                     int* cell_end, void* scratch, int* err, cudaStream_t stream, int* cell_off) {
  if (n < 0 || ncells <= 0) return fail(DEM_ERR_ARG, "cell_sort: bad sizes");
  int* key = (int*)scratch;
  int* rank = key + n;
  int* tile = rank + n;
  const int ntiles = div_up(ncells, kScanTile);
  cudaError_t e = cudaMemsetAsync(cell_end, 0, sizeof(int) * (size_t)ncells, stream);
  if (e != cudaSuccess) return cuda_check(e, "cell_sort memset");
  if (n > 0)
    k_hash_count<<<grid_for(n, 256), 256, 0, stream>>>(pos, plevel, n, lv, k.prm.Origin, ncells, key, rank,
                                                      cell_end, err);
  k_tile_sums<<<ntiles, kScanThreads, 0, stream>>>(cell_end, ncells, tile);
  k_scan_tiles<<<1, kScanThreads, 0, stream>>>(tile, ntiles);
  k_cell_ranges<<<ntiles, kScanThreads, 0, stream>>>(cell_start, cell_end, ncells, tile, cell_off);
  if (n > 0) {
    k_scatter<<<grid_for(n, 256), 256, 0, stream>>>(key, rank, n, cell_start, sorted_hash, sorted_src);
    k_cell_order<<<grid_for(n, 256), 256, 0, stream>>>(sorted_hash, sorted_src, cell_start, cell_end,
                                                      order_key, n);
  }
  return cuda_check(cudaGetLastError(), "cell_sort launch");
}

dem_status neighbor_find(const double3* pos, const double* rad, const int* sorted_src,
                         const int* cell_start, const int* cell_end, const int* plevel, const int* nebor_idx,
                         LevelView lv, const DevConsts& k, int* nebor, int* num_nebor, int n, int* err,
                         cudaStream_t stream, Prefilter pre, const int* cell_off) {
  if (n <= 0) return DEM_OK;
  k_neighbor_find<<<grid_for(n, 128), 128, 0, stream>>>(pos, rad, sorted_src, cell_start, cell_end, cell_off, plevel,
                                                       nebor_idx, lv, k.prm.Origin, k.prm.SearchGap, nebor,
                                                       num_nebor, n, err, pre);
  return cuda_check(cudaGetLastError(), "neighbor_find launch");
}

dem_status wall_list(const double3* pos, const double* rad, const CylinderBC* cyl, int* wlist, size_t pitch,
                     int* nwall, int n, const DevConsts& k, cudaStream_t stream, const int* id,
                     const int* sys_of_id) {
  if (n <= 0) return DEM_OK;
  k_wall_list<<<grid_for(n, 128), 128, 0, stream>>>(pos, rad, cyl, wlist, pitch, nwall, n, k.prm.SearchGap, id,
                                                    sys_of_id);
  return cuda_check(cudaGetLastError(), "wall_list launch");
}

dem_status history_carry_pp(const int* nebor, const int* nebor_old, const int* plevel, const int* nebor_idx,
                            const int* nebor_idx_old, const int* level_npars, const int* level_nnebors,
                            HistSoA old_h, HistSoA cur_h, const int* num_nebor, const int* num_nebor_old,
                            const int* old_src, const int* old_to_new, int n, cudaStream_t stream) {
  if (n <= 0) return DEM_OK;
  k_carry_pp<<<grid_for(n, 256), 256, 0, stream>>>(nebor, nebor_old, plevel, nebor_idx, nebor_idx_old,
                                                  level_npars, level_nnebors, old_h, cur_h, num_nebor,
                                                  num_nebor_old, old_src, old_to_new, n);
  return cuda_check(cudaGetLastError(), "history_carry_pp launch");
}

dem_status history_carry_pw(const int* wlist, size_t pitch, const int* wlist_old, size_t pitch_old,
                            HistSoA old_h, HistSoA cur_h, const int* nwall, const int* nwall_old,
                            const int* old_src, int n, int np_new, int np_old, cudaStream_t stream) {
  if (n <= 0) return DEM_OK;
  k_carry_pw<<<grid_for(n, 128), 128, 0, stream>>>(wlist, pitch, wlist_old, pitch_old, old_h, cur_h, nwall,
                                                  nwall_old, old_src, n, np_new, np_old);
  return cuda_check(cudaGetLastError(), "history_carry_pw launch");
}

dem_status history_rotate(HistSoA old_h, HistSoA cur_h, long long count, cudaStream_t stream) {
  if (count <= 0) return DEM_OK;
  long long blocks = (count + 255) / 256;
  if (blocks > 152LL * 16) blocks = 152LL * 16;
  k_rotate<<<(int)blocks, 256, 0, stream>>>(old_h, cur_h, count);
  return cuda_check(cudaGetLastError(), "history_rotate launch");
}

dem_status inclusive_scan_small(const int* in, int* out, int n, cudaStream_t stream) {
  if (n <= 0) return DEM_OK;
  k_scan_small<<<1, 32, 0, stream>>>(in, out, n);
  return cuda_check(cudaGetLastError(), "scan launch");
}

}  // namespace dem
