/*
 * feed.cu -- the particle feed on the device.
 *
 * The reference feeds particles on the host (ParticleFeed.cpp:8-72, called
 * from main.cpp:439-448): it copies every position to the host, draws
 * positions in the feed band one at a time -- angle, a triangular radius
 * fold, a height -- rejects any that come closer than r_i + r_j + 0.002 to a
 * particle already there (a scan over all of them), gives up on a particle
 * after 500 rejections in a row, places at most 60000 per call, and copies
 * every position back.  Its generator is seeded from the clock.
 *
 * Here the same draws and the same acceptance test run on the device arrays,
 * in parallel rounds:
 *   - the particles already in the band's reach are bucketed once (uniform
 *     grid, cell = 2 r_max + 0.002, linked lists built with atomic exchanges);
 *   - every round, each unplaced new particle draws a candidate from a
 *     counter-based generator keyed by (seed, particle, try), and all new
 *     particles (placed ones and this round's candidates) are bucketed in a
 *     second grid;
 *   - a candidate is accepted when it clears every old particle, every new
 *     particle placed in an earlier round, and every lower-numbered candidate
 *     of this round (two candidates that clash cannot both be accepted: the
 *     higher-numbered one saw the other); otherwise its try count grows, and
 *     after 500 tries it has failed;
 *   - the batch keeps the particles below the first failure, in order, like
 *     the reference's stop at the particle that found no room.
 * No two kept particles overlap, and the outcome is independent of thread
 * scheduling (what a round sees is fixed when it starts): the same seed gives
 * the same positions.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

#include "dem_internal.h"

namespace {

constexpr int kFeedBatch = 60000; /* ParticleFeed.cpp:20 */
constexpr int kFeedTries = 500;   /* ParticleFeed.cpp:20, 54 */
constexpr double kClear = 0.002;  /* ParticleFeed.cpp:52 */
constexpr double kPiRef = 3.1415926;
constexpr long long kMaxCells = 64LL << 20;

inline int grid_for(long long n, int block) { return n <= 0 ? 1 : (int)((n + block - 1) / block); }

struct FeedGrid {
  double x0, y0, z0, cell;
  int gx, gy, gz;
  __device__ int cell_of(double3 p, int& ix, int& iy, int& iz) const {
    ix = min(max((int)floor((p.x - x0) / cell), 0), gx - 1);
    iy = min(max((int)floor((p.y - y0) / cell), 0), gy - 1);
    iz = min(max((int)floor((p.z - z0) / cell), 0), gz - 1);
    return (iz * gy + iy) * gx + ix;
  }
};

struct FeedBand {
  double zmin, zmax, R, cx, cy;
};

/* counter-based uniform in [0, 1]: SplitMix64 finaliser over a key of the
 * seed, the particle, the try and the draw */
__device__ __forceinline__ double feed_u01(unsigned long long seed, long long particle, int attempt, int draw) {
  unsigned long long z = seed ^ (0x9E3779B97F4A7C15ull * (unsigned long long)(particle + 1)) ^
                         (0xC2B2AE3D27D4EB4Full * (unsigned long long)(attempt * 4 + draw + 1));
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740991.0);
}

/* the draw of ParticleFeed.cpp:23-41 */
__device__ __forceinline__ double3 feed_draw(const FeedBand& b, double r, unsigned long long seed, long long particle,
                                             int attempt) {
  const double theta = 2.0 * kPiRef * feed_u01(seed, particle, attempt, 0);
  const double u = feed_u01(seed, particle, attempt, 1) + feed_u01(seed, particle, attempt, 2);
  const double mag = u > 1.0 ? 2.0 - u : u;
  double3 p;
  p.x = mag * (b.R - r) * cos(theta) + b.cx;
  p.y = mag * (b.R - r) * sin(theta) + b.cy;
  p.z = feed_u01(seed, particle, attempt, 3) * (b.zmax - b.zmin) + b.zmin;
  return p;
}

__global__ void k_max_radius(const double* __restrict__ rad, int n, unsigned long long* out) {
  double m = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmax(m, rad[i]);
  /* radii are positive: their bit patterns order like the values */
  atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

__global__ void k_fill(int* __restrict__ a, long long n, int v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = v;
}

/* the old particles within reach of the band, bucketed */
__global__ void k_bucket_old(const double3* __restrict__ pos, int n_old, double zlo, double zhi, FeedGrid g,
                             int* __restrict__ head, int* __restrict__ next) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_old) return;
  const double3 p = pos[i];
  if (p.z < zlo || p.z > zhi) return;
  int ix, iy, iz;
  next[i] = atomicExch(&head[g.cell_of(p, ix, iy, iz)], i);
}

/* this round's candidates drawn, then every new particle still in play
 * (placed, or a candidate) bucketed, with whether it was placed when the
 * round started */
__global__ void k_propose(const double* __restrict__ rad, int n_old, int B, FeedBand band, unsigned long long seed,
                          const int* __restrict__ status, const int* __restrict__ tries, double3* __restrict__ npos,
                          int* __restrict__ placed, const int* __restrict__ first_fail, FeedGrid g,
                          int* __restrict__ head, int* __restrict__ next) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B || i >= *first_fail) return;
  const int st = status[i];
  if (st == 0) npos[i] = feed_draw(band, rad[n_old + i], seed, (long long)n_old + i, tries[i]);
  placed[i] = st == 1;
  int ix, iy, iz;
  next[i] = atomicExch(&head[g.cell_of(npos[i], ix, iy, iz)], i);
}

/* ParticleFeed.cpp:45-58 for every candidate: clear of the old particles, of
 * the new ones placed before this round and of the lower-numbered candidates */
__global__ void k_check(const double3* __restrict__ pos, const double* __restrict__ rad, int n_old, int B,
                        const int* __restrict__ head_old, const int* __restrict__ next_old,
                        const int* __restrict__ head_new, const int* __restrict__ next_new,
                        const double3* __restrict__ npos, const int* __restrict__ placed, FeedGrid g,
                        int* __restrict__ status, int* __restrict__ tries, int* __restrict__ first_fail,
                        int* __restrict__ pending) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B || i >= *first_fail || status[i] != 0) return;
  const double3 p = npos[i];
  const double r = rad[n_old + i];
  int cx, cy, cz;
  g.cell_of(p, cx, cy, cz);
  bool clear = true;
  for (int dz = -1; dz <= 1 && clear; dz++)
    for (int dy = -1; dy <= 1 && clear; dy++)
      for (int dx = -1; dx <= 1 && clear; dx++) {
        const int x = cx + dx, y = cy + dy, z = cz + dz;
        if (x < 0 || y < 0 || z < 0 || x >= g.gx || y >= g.gy || z >= g.gz) continue;
        const int c = (z * g.gy + y) * g.gx + x;
        for (int j = head_old[c]; j >= 0 && clear; j = next_old[j]) {
          const double3 q = pos[j];
          const double ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
          if (sqrt(ex * ex + ey * ey + ez * ez) < rad[j] + r + kClear) clear = false;
        }
        for (int k = head_new[c]; k >= 0 && clear; k = next_new[k]) {
          if (k == i || (k > i && !placed[k])) continue;
          const double3 q = npos[k];
          const double ex = p.x - q.x, ey = p.y - q.y, ez = p.z - q.z;
          if (sqrt(ex * ex + ey * ey + ez * ez) < rad[n_old + k] + r + kClear) clear = false;
        }
      }
  if (clear) {
    status[i] = 1;
    return;
  }
  if (++tries[i] >= kFeedTries) {
    status[i] = 2;
    atomicMin(first_fail, i);
  } else {
    atomicAdd(pending, 1);
  }
}

__global__ void k_write(double3* __restrict__ pos, int n_old, int cut, const double3* __restrict__ npos) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cut) pos[n_old + i] = npos[i];
}

}  // namespace

extern "C" int ParticleFeedDevice(FeedZone* Feedcube, CylinderBC* h_Cir, double InitParSize, double3* dPos,
                                  double* dRad, int numParticle, int NP, unsigned long long seed) {
  (void)InitParSize; /* unused by the reference's feed as well */
  if (!Feedcube || !h_Cir || !dPos || !dRad || numParticle < 0 || NP < 0) {
    dem::set_error("ParticleFeedDevice: bad argument");
    return -1;
  }
  const int B = std::min(kFeedBatch, NP - numParticle);
  if (B <= 0) return numParticle;
  FeedBand band{Feedcube->Lmin, Feedcube->Lmax, h_Cir->R, h_Cir->cir.x, h_Cir->cir.y};
  if (!(band.zmax >= band.zmin) || !(band.R > 0.0)) {
    dem::set_error("ParticleFeedDevice: empty feed band or cylinder");
    return -1;
  }
  /* device scratch: counters, two grids, the new particles' state */
  unsigned long long* d_rmax = nullptr;
  int *ctr = nullptr, *head_old = nullptr, *next_old = nullptr, *head_new = nullptr, *next_new = nullptr;
  int *status = nullptr, *tries = nullptr, *placed = nullptr;
  double3* npos = nullptr;
  auto release = [&]() {
    cudaFree(d_rmax);
    cudaFree(ctr);
    cudaFree(head_old);
    cudaFree(next_old);
    cudaFree(head_new);
    cudaFree(next_new);
    cudaFree(status);
    cudaFree(tries);
    cudaFree(placed);
    cudaFree(npos);
  };
  auto fail = [&](cudaError_t e, const char* what) {
    cudaGetLastError();
    release();
    dem::set_error(std::string("ParticleFeedDevice: ") + what + ": " + cudaGetErrorString(e));
    return -1;
  };
  cudaError_t e = cudaMalloc(&d_rmax, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&ctr, 2 * sizeof(int));
  if (e != cudaSuccess) return fail(e, "allocation");
  e = cudaMemset(d_rmax, 0, sizeof(unsigned long long));
  if (e != cudaSuccess) return fail(e, "memset");
  k_max_radius<<<grid_for(NP, 256) < 1024 ? grid_for(NP, 256) : 1024, 256>>>(dRad, NP, d_rmax);
  unsigned long long rbits = 0;
  e = cudaMemcpy(&rbits, d_rmax, sizeof(rbits), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(e, "radius reduction");
  double rmax;
  std::memcpy(&rmax, &rbits, sizeof(rmax));
  FeedGrid g;
  g.cell = 2.0 * rmax + kClear;
  g.x0 = band.cx - band.R - g.cell;
  g.y0 = band.cy - band.R - g.cell;
  g.z0 = band.zmin - g.cell;
  g.gx = g.gy = (int)std::ceil((2.0 * band.R + 2.0 * g.cell) / g.cell) + 1;
  g.gz = (int)std::ceil((band.zmax - band.zmin + 2.0 * g.cell) / g.cell) + 1;
  const long long C = (long long)g.gx * g.gy * g.gz;
  if (C > kMaxCells) {
    release();
    dem::set_error("ParticleFeedDevice: feed band too large for the bucket grid (" + std::to_string(C) + " cells)");
    return -1;
  }
  e = cudaMalloc(&head_old, sizeof(int) * C);
  if (e == cudaSuccess) e = cudaMalloc(&head_new, sizeof(int) * C);
  if (e == cudaSuccess) e = cudaMalloc(&next_old, sizeof(int) * (numParticle > 0 ? numParticle : 1));
  if (e == cudaSuccess) e = cudaMalloc(&next_new, sizeof(int) * B);
  if (e == cudaSuccess) e = cudaMalloc(&status, sizeof(int) * B);
  if (e == cudaSuccess) e = cudaMalloc(&tries, sizeof(int) * B);
  if (e == cudaSuccess) e = cudaMalloc(&placed, sizeof(int) * B);
  if (e == cudaSuccess) e = cudaMalloc(&npos, sizeof(double3) * B);
  if (e != cudaSuccess) return fail(e, "allocation");
  const int fill_grid = (int)std::min<long long>(grid_for(C, 256), 4096);
  k_fill<<<fill_grid, 256>>>(head_old, C, -1);
  k_fill<<<grid_for(B, 256), 256>>>(status, B, 0);
  k_fill<<<grid_for(B, 256), 256>>>(tries, B, 0);
  /* the old particles that could touch a particle in the band */
  const double reach = g.cell;
  if (numParticle > 0)
    k_bucket_old<<<grid_for(numParticle, 256), 256>>>(dPos, numParticle, band.zmin - reach, band.zmax + reach, g,
                                                      head_old, next_old);
  int first_fail = B;
  e = cudaMemcpy(ctr, &first_fail, sizeof(int), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return fail(e, "counter upload");
  /* rounds: every round decides or advances every candidate below the first
   * failure, so kFeedTries rounds always suffice */
  for (int round = 0; round < kFeedTries + 1; round++) {
    k_fill<<<fill_grid, 256>>>(head_new, C, -1);
    e = cudaMemset(ctr + 1, 0, sizeof(int));
    if (e != cudaSuccess) return fail(e, "counter reset");
    k_propose<<<grid_for(B, 256), 256>>>(dRad, numParticle, B, band, seed, status, tries, npos, placed, ctr, g,
                                         head_new, next_new);
    k_check<<<grid_for(B, 256), 256>>>(dPos, dRad, numParticle, B, head_old, next_old, head_new, next_new, npos,
                                       placed, g, status, tries, ctr, ctr + 1);
    int h[2];
    e = cudaMemcpy(h, ctr, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(e, "feed round");
    first_fail = h[0];
    if (h[1] == 0) break; /* nothing below the first failure is still pending */
  }
  k_write<<<grid_for(first_fail, 256), 256>>>(dPos, numParticle, first_fail, npos);
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return fail(e, "write-back");
  release();
  return numParticle + first_fail;
}
