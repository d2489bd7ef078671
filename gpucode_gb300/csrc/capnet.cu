/*
 * capnet.cu -- the learned capillary closure: training samples from a running
 * wet bed, hand-written training kernels, inference kernels, and the host API
 * (dem_capnet_*, dem_set_capnet).  Definitions of the network's inputs,
 * outputs and layout: capnet.cuh.
 *
 * Samples: every bridged pair of the current state, features and the plain
 * formula's outputs in FP64 (kernel.cu:65-81, :518), written in particle /
 * slot order (deterministic).
 *
 * Training (FP32): one block of 128 threads takes 128 samples, one sample per
 * thread for the forward pass and the per-sample backward pass, with the
 * activations in shared memory; the weight gradients are reduced over the
 * block's samples in shared memory and written as one partial per block; a
 * second kernel sums the partials in block order (so a run is reproducible)
 * and applies Adam.  Loss: mean over samples of the squared error of the two
 * standardised outputs.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <string>
#include <vector>

#include "capnet.cuh"
#include "dem_device.cuh"
#include "engine.h"

struct dem_capnet {
  float* params;   /* device, kCapParams FP32 */
  float* adam_m;   /* device */
  float* adam_v;   /* device */
  float* partial;  /* device, per-block gradient partials */
  int partial_blocks;
  long long step;  /* Adam steps taken */
  float norm[20];  /* x_mean[4] x_std[4] y_mean[2] y_std[2] hull_lo[4] hull_hi[4] */
  bool has_norm;
  dem::CapNetSmem* packed; /* device, BF16 network as the step kernel stages it */
  bool packed_valid;
};

namespace dem {
namespace {

constexpr int kTB = 128;           /* samples per training block */
constexpr int kHS = kCapH + 1;     /* padded row of per-sample activations */
constexpr int kWPad = 4612;        /* parameters in shared memory, 16-byte multiple */
constexpr size_t kTrainSmem = sizeof(float) * (kWPad + kTB * 4 + 3 * kTB * kHS + kTB * 2 + 32);

inline int blocks_for(long long n, int b) { return n <= 0 ? 1 : (int)((n + b - 1) / b); }

struct Norm {
  float xm[4], xs[4], ym[2], ys[2]; /* means and standard deviations */
};
Norm norm_of(const dem_capnet* net) {
  Norm z;
  for (int i = 0; i < 4; i++) { z.xm[i] = net->norm[i]; z.xs[i] = net->norm[4 + i]; }
  for (int i = 0; i < 2; i++) { z.ym[i] = net->norm[8 + i]; z.ys[i] = net->norm[10 + i]; }
  return z;
}

__device__ __forceinline__ float silu_acc(float z) { return z / (1.0f + expf(-z)); }
__device__ __forceinline__ float dsilu_acc(float z) {
  const float s = 1.0f / (1.0f + expf(-z));
  return s * (1.0f + z * (1.0f - s));
}
__device__ __forceinline__ void std_inputs(const float* raw, const Norm& nz, float x[4]) {
  x[0] = (logf(raw[0]) - nz.xm[0]) / nz.xs[0];
  x[1] = (logf(raw[1]) - nz.xm[1]) / nz.xs[1];
  x[2] = (raw[2] - nz.xm[2]) / nz.xs[2];
  x[3] = (raw[3] - nz.xm[3]) / nz.xs[3];
}

/* ---------------- samples ---------------- */

struct SampleArgs {
  const double3* pos;
  const double* rad;
  const int *nebor, *num_nebor, *plevel, *nidx, *npars, *nneb, *lqd, *id;
  const unsigned char* brg;
  int n;
  double vol, gapmn, layer, stension;
  float theta_max;
  unsigned long long theta_seed;
  LiquidModel lm; /* mode 1: per-contact volumes and angles (liquid.cuh) */
};

__global__ void k_sample_count(SampleArgs a, int* cnt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.n) return;
  const int L = a.plevel[q];
  const long long stride = a.npars[L];
  const long long base = slot_base(L, a.npars, a.nneb) + a.nidx[q];
  int c = 0;
  for (int k = 0; k < a.num_nebor[q]; k++) c += a.brg[base + k * stride] ? 1 : 0;
  cnt[q] = c;
}

/* exclusive scan of n ints in one block of 1024 threads (each a contiguous chunk) */
__global__ void k_scan_chunks(const int* in, long long* out, int n, long long* total) {
  __shared__ long long part[1024];
  const int t = threadIdx.x, T = blockDim.x;
  const int per = (n + T - 1) / T, lo = min(n, t * per), hi = min(n, lo + per);
  long long s = 0;
  for (int i = lo; i < hi; i++) s += in[i];
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    long long acc = 0;
    for (int i = 0; i < T; i++) { const long long v = part[i]; part[i] = acc; acc += v; }
    *total = acc;
  }
  __syncthreads();
  long long acc = part[t];
  for (int i = lo; i < hi; i++) { out[i] = acc; acc += in[i]; }
}

__global__ void k_sample_write(SampleArgs a, const long long* off, long long capacity, float* x, float* y) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= a.n) return;
  const int L = a.plevel[q];
  const long long stride = a.npars[L];
  const long long base = slot_base(L, a.npars, a.nneb) + a.nidx[q];
  long long o = off[q];
  const double3 pi = a.pos[q];
  const double ri = a.rad[q];
  const int inl = max(12, a.lqd[q]);
  const double iVol = a.vol * (8.0 * ri * ri * ri) / inl; /* kernel.cu:434 */
  const float thi = cap_theta(a.id[q], a.theta_seed, a.theta_max);
  LIQUID lq;
  lq.stension = a.stension; lq.vol = a.vol; lq.gapmn = a.gapmn; lq.layer = a.layer; lq.brknmx = 0.0;
  for (int k = 0; k < a.num_nebor[q]; k++) {
    const long long s = base + k * stride;
    if (!a.brg[s]) continue;
    if (o >= capacity) return;
    const int j = a.nebor[s];
    const double3 pj = a.pos[j];
    const double rj = a.rad[j];
    const double dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
    const double gap = sqrt(dx * dx + dy * dy + dz * dz) - (ri + rj);
    const double Splus = gap < 0.0 ? 0.0 : gap;
    const double effR = 2.0 * ri * rj / (ri + rj);
    const double thj = cap_theta(a.id[j], a.theta_seed, a.theta_max);
    x[4 * o + 3] = (float)(fmin(ri, rj) / fmax(ri, rj));
    if (a.lm.mode == 0) {
      const int jnl = max(12, a.lqd[j]);
      const double jVol = a.vol * (8.0 * rj * rj * rj) / jnl;
      const double ijVol = iVol + jVol;
      const double F = fcap64(Splus, 8.0 * ijVol, effR, lq); /* kernel.cu:538-544 */
      x[4 * o + 0] = (float)fmax(a.gapmn, Splus);
      x[4 * o + 1] = (float)(8.0 * ijVol);
      x[4 * o + 2] = 0.5f * (thi + (float)thj);
      y[2 * o + 0] = (float)(F / (2.0 * kPiRef * effR * a.stension));
      y[2 * o + 1] = (float)(0.99 * pow(ijVol, 0.33)); /* kernel.cu:518 */
    } else {
      /* the per-contact model: the network learns the contact-angle terms too */
      const double th = 0.5 * ((double)thi + thj);
      const double V = pair_bridge_volume(a.lm, a.id[q], a.id[j], fmin(ri, rj));
      x[4 * o + 0] = (float)fmax(a.gapmn, Splus);
      x[4 * o + 1] = (float)(8.0 * V);
      x[4 * o + 2] = (float)th;
      y[2 * o + 0] = (float)willett64(fmax(a.gapmn, Splus), 8.0 * V, th);
      y[2 * o + 1] = (float)rupture64(V, th);
    }
    o++;
  }
}

/* ---------------- training ---------------- */

__global__ void __launch_bounds__(kTB) k_train(const float* __restrict__ P, const float* __restrict__ xr,
                                               const float* __restrict__ yr, const int* __restrict__ idx, int nb,
                                               float inv_total, Norm nz, float* __restrict__ partial) {
  extern __shared__ float sm[];
  float* W = sm;
  float* X = W + kWPad;
  float* H1 = X + kTB * 4;
  float* Z2 = H1 + kTB * kHS; /* pre-activations, then their gradients */
  float* H2 = Z2 + kTB * kHS; /* activations, then the layer-1 gradients */
  float* DY = H2 + kTB * kHS;
  float* red = DY + kTB * 2;
  const int tid = threadIdx.x;
  for (int i = tid; i < kCapParams; i += kTB) W[i] = P[i];
  const int gi = blockIdx.x * kTB + tid;
  const bool valid = gi < nb;
  float x[4] = {0.f, 0.f, 0.f, 0.f}, t[2] = {0.f, 0.f};
  if (valid) {
    const long long si = idx ? (long long)idx[gi] : (long long)gi;
    std_inputs(xr + 4 * si, nz, x);
    t[0] = (yr[2 * si] - nz.ym[0]) / nz.ys[0];
    t[1] = (yr[2 * si + 1] - nz.ym[1]) / nz.ys[1];
  }
  for (int i = 0; i < 4; i++) X[tid * 4 + i] = x[i];
  __syncthreads();
  const float* W1 = W + kCapW1;
  const float* B1 = W + kCapB1;
  const float* W2 = W + kCapW2;
  const float* B2 = W + kCapB2;
  const float* W3 = W + kCapW3;
  const float* B3 = W + kCapB3;
  float* h1 = H1 + tid * kHS;
  float* z2 = Z2 + tid * kHS;
  float* h2 = H2 + tid * kHS;
  /* forward */
  for (int m = 0; m < kCapH; m++) {
    float z = B1[m];
    for (int i = 0; i < 4; i++) z += W1[m * 4 + i] * x[i];
    h1[m] = silu_acc(z);
  }
  float y0 = B3[0], y1 = B3[1];
  for (int n = 0; n < kCapH; n++) {
    float z = B2[n];
    for (int m = 0; m < kCapH; m++) z += W2[n * kCapH + m] * h1[m];
    z2[n] = z;
    const float a = silu_acc(z);
    h2[n] = a;
    y0 += W3[n] * a;
    y1 += W3[kCapH + n] * a;
  }
  const float e0 = y0 - t[0], e1 = y1 - t[1];
  const float dy0 = valid ? 2.0f * e0 * inv_total : 0.f, dy1 = valid ? 2.0f * e1 * inv_total : 0.f;
  DY[tid * 2] = dy0;
  DY[tid * 2 + 1] = dy1;
  for (int n = 0; n < kCapH; n++) z2[n] = (W3[n] * dy0 + W3[kCapH + n] * dy1) * dsilu_acc(z2[n]);
  __syncthreads();
  float* out = partial + (size_t)blockIdx.x * (kCapParams + 1);
  /* layer 2 and 3 weight gradients, reduced over the block's samples */
  for (int p = tid; p < kCapH * kCapH + kCapH + kCapOut * kCapH + kCapOut; p += kTB) {
    float acc = 0.f;
    if (p < kCapH * kCapH) {
      const int n = p / kCapH, m = p % kCapH;
      for (int s = 0; s < kTB; s++) acc += Z2[s * kHS + n] * H1[s * kHS + m];
      out[kCapW2 + p] = acc;
    } else if (p < kCapH * kCapH + kCapH) {
      const int n = p - kCapH * kCapH;
      for (int s = 0; s < kTB; s++) acc += Z2[s * kHS + n];
      out[kCapB2 + n] = acc;
    } else if (p < kCapH * kCapH + kCapH + kCapOut * kCapH) {
      const int q = p - kCapH * kCapH - kCapH, o = q / kCapH, n = q % kCapH;
      for (int s = 0; s < kTB; s++) acc += DY[s * 2 + o] * H2[s * kHS + n];
      out[kCapW3 + q] = acc;
    } else {
      const int o = p - kCapH * kCapH - kCapH - kCapOut * kCapH;
      for (int s = 0; s < kTB; s++) acc += DY[s * 2 + o];
      out[kCapB3 + o] = acc;
    }
  }
  __syncthreads();
  /* layer-1 gradients of this sample (into the H2 rows) */
  for (int m = 0; m < kCapH; m++) {
    float g = 0.f;
    for (int n = 0; n < kCapH; n++) g += W2[n * kCapH + m] * z2[n];
    float z = B1[m];
    for (int i = 0; i < 4; i++) z += W1[m * 4 + i] * x[i];
    h2[m] = g * dsilu_acc(z);
  }
  __syncthreads();
  for (int p = tid; p < kCapH * 4 + kCapH; p += kTB) {
    float acc = 0.f;
    if (p < kCapH * 4) {
      const int m = p / 4, i = p % 4;
      for (int s = 0; s < kTB; s++) acc += H2[s * kHS + m] * X[s * 4 + i];
      out[kCapW1 + p] = acc;
    } else {
      const int m = p - kCapH * 4;
      for (int s = 0; s < kTB; s++) acc += H2[s * kHS + m];
      out[kCapB1 + m] = acc;
    }
  }
  /* loss partial */
  float l = valid ? (e0 * e0 + e1 * e1) * inv_total : 0.f;
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((tid & 31) == 0) red[tid >> 5] = l;
  __syncthreads();
  if (tid == 0) {
    float s = 0.f;
    for (int w = 0; w < kTB / 32; w++) s += red[w];
    out[kCapParams] = s;
  }
}

/* sum the block partials in order; then an Adam step (lr > 0) and/or a copy of the gradient */
__global__ void k_reduce_adam(float* P, float* M, float* V, const float* partial, int nblocks, float lr, float bc1,
                              float bc2, float* grad_out, float* loss_out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kCapParams) return;
  float g = 0.f;
  for (int b = 0; b < nblocks; b++) g += partial[(size_t)b * (kCapParams + 1) + p];
  if (p == kCapParams) {
    if (loss_out) *loss_out = g;
    return;
  }
  if (grad_out) grad_out[p] = g;
  if (lr > 0.f) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float m = b1 * M[p] + (1.f - b1) * g;
    const float v = b2 * V[p] + (1.f - b2) * g * g;
    M[p] = m;
    V[p] = v;
    P[p] -= lr * (m / bc1) / (sqrtf(v / bc2) + eps);
  }
}

/* FP32 forward (the training precision) on raw features -> raw outputs */
__global__ void k_infer32(const float* __restrict__ P, const float* __restrict__ xr, long long n, Norm nz,
                          float* __restrict__ y) {
  __shared__ float W[kWPad];
  for (int i = threadIdx.x; i < kCapParams; i += blockDim.x) W[i] = P[i];
  __syncthreads();
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  float x[4], h1[kCapH];
  std_inputs(xr + 4 * q, nz, x);
  for (int m = 0; m < kCapH; m++) {
    float z = W[kCapB1 + m];
    for (int i = 0; i < 4; i++) z += W[kCapW1 + m * 4 + i] * x[i];
    h1[m] = silu_acc(z);
  }
  float y0 = W[kCapB3], y1 = W[kCapB3 + 1];
  for (int nn = 0; nn < kCapH; nn++) {
    float z = W[kCapB2 + nn];
    for (int m = 0; m < kCapH; m++) z += W[kCapW2 + nn * kCapH + m] * h1[m];
    const float a = silu_acc(z);
    y0 += W[kCapW3 + nn] * a;
    y1 += W[kCapW3 + kCapH + nn] * a;
  }
  y[2 * q] = y0 * nz.ys[0] + nz.ym[0];
  y[2 * q + 1] = y1 * nz.ys[1] + nz.ym[1];
}

/* BF16 tensor-core tiles, exactly as the fused step kernel evaluates them */
__global__ void __launch_bounds__(128) k_infer_tc(const CapNetSmem* __restrict__ wsrc, const float* __restrict__ xr,
                                                  long long n, float* __restrict__ y) {
  __shared__ __align__(16) unsigned char wbuf[sizeof(CapNetSmem)];
  CapNetSmem& w = *reinterpret_cast<CapNetSmem*>(wbuf);
  cap_stage(wsrc, &w);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long tile = warp; tile * 16 < n; tile += nwarps) {
    uint32_t xa = 0u, xb = 0u;
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    if (t < 2) {
      if (r0 < n) {
        const float* f = xr + 4 * r0;
        xa = cap_pair(w, f[0], f[1], f[2], f[3], t);
      }
      if (r1 < n) {
        const float* f = xr + 4 * r1;
        xb = cap_pair(w, f[0], f[1], f[2], f[3], t);
      }
    }
    float o[4];
    cap_tile16(w, xa, xb, o);
    if (t == 0) {
      if (r0 < n) {
        y[2 * r0] = o[0] * w.y_std[0] + w.y_mean[0];
        y[2 * r0 + 1] = o[1] * w.y_std[1] + w.y_mean[1];
      }
      if (r1 < n) {
        y[2 * r1] = o[2] * w.y_std[0] + w.y_mean[0];
        y[2 * r1 + 1] = o[3] * w.y_std[1] + w.y_mean[1];
      }
    }
  }
}

/* ---------------- the network on the 5th-generation tensor cores ----------------
 * One CTA of 128 threads takes 128 bridges (one row each) at a time and runs
 * layers 1 and 2 as tcgen05.mma (kind::f16: BF16 operands from shared memory,
 * FP32 accumulators in tensor memory), M = 128 rows, N = 64 hidden units:
 *   layer 1: D1[128 x 64] = X[128 x 16] W1^T   (K = 4 inputs padded to 16: one MMA)
 *   layer 2: D2[128 x 64] = S1[128 x 64] W2^T  (K = 64: four MMAs of K = 16)
 * Each thread reads its row of D1 / D2 back with tcgen05.ld (warp w owns
 * tensor-memory lanes 32w..32w+31), adds the bias, applies SiLU (the same
 * hardware-tanh form as the warp tiles), writes layer 2's BF16 operand row,
 * and evaluates layer 3 (2 outputs) on the CUDA cores.  One thread issues the
 * MMAs; their completion arrives on an mbarrier through tcgen05.commit.
 *
 * Operands are in the canonical no-swizzle K-major layout: 8-row x 16-byte
 * core matrices, 128 bytes each; the core matrices of one 8-row group are
 * adjacent along K (leading-dimension offset 128 B), 8-row groups follow
 * each other (stride-dimension offset = 128 B x cores along K). */
constexpr int kTcRows = 128;
constexpr uint32_t kTcCols = 128;  /* tensor-memory columns: D1 at 0, D2 at 64 */
constexpr unsigned long long kTcWaitNs = 1000000000ull; /* give up on an MMA completion after 1 s */

struct __align__(128) TcSmem {
  __nv_bfloat16 a1[kTcRows * 16];   /* X, 16 row groups x 2 K cores */
  __nv_bfloat16 a2[kTcRows * kCapH]; /* SiLU(layer 1), 16 row groups x 8 K cores */
  __nv_bfloat16 b1[kCapH * 16];     /* W1 [n][k], 8 n groups x 2 K cores */
  __nv_bfloat16 b2[kCapH * kCapH];  /* W2 [n][k], 8 n groups x 8 K cores */
  float bias1[kCapH], bias2[kCapH], w3[2][kCapH], b3[2];
  float xm[4], xis[4], ym[2], ys[2];
  unsigned long long mbar;
  uint32_t tmem_base;
};

/* byte offset of element (row, k) of a K-major operand with `kcores` core
 * matrices along K */
__device__ __forceinline__ uint32_t tc_off(int row, int k, int kcores) {
  return (uint32_t)((row >> 3) * (kcores * 128) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

/* shared-memory matrix descriptor: start, leading (K) and stride (8-row)
 * byte offsets, version 1, no swizzle */
__device__ __forceinline__ unsigned long long tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (unsigned long long)((saddr >> 4) & 0x3FFFu) | ((unsigned long long)((lbo >> 4) & 0x3FFFu) << 16) |
         ((unsigned long long)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
 * K-major, N = 64, M = 128 */
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kCapH >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, unsigned long long a, unsigned long long b, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kTcIdesc), "r"(acc));
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
/* wait for the mbarrier's phase `parity` to complete; false after kTcWaitNs */
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity) {
  const unsigned long long t0 = global_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > kTcWaitNs) return false;
  }
}
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

/* raw features -> raw outputs; err gets 1 if an MMA completion was not seen
 * within kTcWaitNs (the kernel then stops; tensor memory is freed on every
 * path) */
__global__ void __launch_bounds__(kTcRows, 1) k_infer_tc5(const CapNetSmem* __restrict__ wsrc,
                                                          const float* __restrict__ xr, long long n,
                                                          float* __restrict__ y, int* __restrict__ err) {
  __shared__ TcSmem sm;
  const int tid = threadIdx.x, warp = tid >> 5;
  /* weights into the canonical layout, biases and the last layer as FP32 */
  for (int e = tid; e < kCapH * 16; e += kTcRows) {
    const int nn = e >> 4, k = e & 15;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(sm.b1) + tc_off(nn, k, 2)) = wsrc->w1[nn * kCapS1 + k];
  }
  for (int e = tid; e < kCapH * kCapH; e += kTcRows) {
    const int nn = e >> 6, k = e & 63;
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(sm.b2) + tc_off(nn, k, 8)) = wsrc->w2[nn * kCapS2 + k];
  }
  for (int e = tid; e < kTcRows * 16; e += kTcRows) sm.a1[e] = __float2bfloat16(0.f);
  if (tid < kCapH) {
    sm.bias1[tid] = wsrc->b1[tid];
    sm.bias2[tid] = wsrc->b2[tid];
    sm.w3[0][tid] = __bfloat162float(wsrc->w3[tid]);
    sm.w3[1][tid] = __bfloat162float(wsrc->w3[kCapS2 + tid]);
  }
  if (tid < 4) {
    sm.xm[tid] = wsrc->x_mean[tid];
    sm.xis[tid] = wsrc->x_inv_std[tid];
  }
  if (tid < 2) {
    sm.b3[tid] = wsrc->b3[tid];
    sm.ym[tid] = wsrc->y_mean[tid];
    sm.ys[tid] = wsrc->y_std[tid];
  }
  const uint32_t mbar = smem_u32(&sm.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                 "r"(kTcCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  tc_sync();
  const uint32_t tmem = sm.tmem_base;
  const uint32_t d1 = tmem, d2 = tmem + (uint32_t)kCapH;
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16; /* this warp's tensor-memory lanes */
  const unsigned long long da1 = tc_desc(smem_u32(sm.a1), 128, 2 * 128);
  const unsigned long long db1 = tc_desc(smem_u32(sm.b1), 128, 2 * 128);
  uint32_t parity = 0;
  bool ok = true;
  const long long tiles = (n + kTcRows - 1) / kTcRows;
  for (long long tile = blockIdx.x; tile < tiles && ok; tile += gridDim.x) {
    const long long row = tile * kTcRows + tid;
    /* layer 1 operand: this row's standardised inputs (k 0..3; k 4..15 stay 0) */
    float x0 = 0.f, x1 = 0.f, x2 = 0.f, x3 = 0.f;
    if (row < n) {
      const float4 f = *reinterpret_cast<const float4*>(xr + 4 * row);
      x0 = (__logf(f.x) - sm.xm[0]) * sm.xis[0];
      x1 = (__logf(f.y) - sm.xm[1]) * sm.xis[1];
      x2 = (f.z - sm.xm[2]) * sm.xis[2];
      x3 = (f.w - sm.xm[3]) * sm.xis[3];
    }
    {
      uint2 v;
      v.x = pack_bf16(x0, x1);
      v.y = pack_bf16(x2, x3);
      *reinterpret_cast<uint2*>(reinterpret_cast<char*>(sm.a1) + tc_off(tid, 0, 2)) = v;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_sync();
    if (tid == 0) {
      tc_mma(d1, da1, db1, 0);
      tc_commit(mbar);
    }
    /* every thread polls with a bound; the block decides together */
    ok = __syncthreads_and(tc_wait(mbar, parity)) != 0;
    if (!ok) break;
    parity ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    /* layer 1 out: bias, SiLU, BF16 into layer 2's operand row */
#pragma unroll
    for (int c = 0; c < kCapH; c += 16) {
      float v[16];
      tc_ld16(d1 + lane_base + (uint32_t)c, v);
      uint4 lo, hi;
      lo.x = pack_bf16(cap_silu(v[0] + sm.bias1[c + 0]), cap_silu(v[1] + sm.bias1[c + 1]));
      lo.y = pack_bf16(cap_silu(v[2] + sm.bias1[c + 2]), cap_silu(v[3] + sm.bias1[c + 3]));
      lo.z = pack_bf16(cap_silu(v[4] + sm.bias1[c + 4]), cap_silu(v[5] + sm.bias1[c + 5]));
      lo.w = pack_bf16(cap_silu(v[6] + sm.bias1[c + 6]), cap_silu(v[7] + sm.bias1[c + 7]));
      hi.x = pack_bf16(cap_silu(v[8] + sm.bias1[c + 8]), cap_silu(v[9] + sm.bias1[c + 9]));
      hi.y = pack_bf16(cap_silu(v[10] + sm.bias1[c + 10]), cap_silu(v[11] + sm.bias1[c + 11]));
      hi.z = pack_bf16(cap_silu(v[12] + sm.bias1[c + 12]), cap_silu(v[13] + sm.bias1[c + 13]));
      hi.w = pack_bf16(cap_silu(v[14] + sm.bias1[c + 14]), cap_silu(v[15] + sm.bias1[c + 15]));
      *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.a2) + tc_off(tid, c, 8)) = lo;
      *reinterpret_cast<uint4*>(reinterpret_cast<char*>(sm.a2) + tc_off(tid, c + 8, 8)) = hi;
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc_sync();
    if (tid == 0) {
#pragma unroll
      for (int k = 0; k < kCapH / 16; k++) {
        const unsigned long long da = tc_desc(smem_u32(sm.a2) + 256u * k, 128, 8 * 128);
        const unsigned long long db = tc_desc(smem_u32(sm.b2) + 256u * k, 128, 8 * 128);
        tc_mma(d2, da, db, k > 0);
      }
      tc_commit(mbar);
    }
    ok = __syncthreads_and(tc_wait(mbar, parity)) != 0;
    if (!ok) break;
    parity ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    /* layer 2 out: bias, SiLU, and layer 3 on the CUDA cores */
    float o0 = sm.b3[0], o1 = sm.b3[1];
#pragma unroll
    for (int c = 0; c < kCapH; c += 16) {
      float v[16];
      tc_ld16(d2 + lane_base + (uint32_t)c, v);
#pragma unroll
      for (int i = 0; i < 16; i++) {
        /* the same BF16 rounding of the activations as the warp tiles */
        const float a = __bfloat162float(__float2bfloat16(cap_silu(v[i] + sm.bias2[c + i])));
        o0 = fmaf(sm.w3[0][c + i], a, o0);
        o1 = fmaf(sm.w3[1][c + i], a, o1);
      }
    }
    if (row < n) {
      y[2 * row] = o0 * sm.ys[0] + sm.ym[0];
      y[2 * row + 1] = o1 * sm.ys[1] + sm.ym[1];
    }
    tc_sync(); /* every row read before the next tile's MMAs overwrite D1 / D2 */
  }
  if (!ok) {
    if (tid == 0) atomicOr(err, 1);
    /* the phase that was not seen: whatever was issued completes (bounded)
     * before the memory is freed */
    tc_wait(mbar, parity);
  }
  tc_sync();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcCols) : "memory");
  }
}

/* the plain closure on raw features: FP64 as the reference evaluates it
 * (kernel.cu:65-81 with pow/log/exp, :518), or the step kernel's FP32 form */
__global__ void k_formula64(const float* __restrict__ xr, long long n, float* __restrict__ y, int angle) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const double v = xr[4 * q + 1];
  if (angle) { /* the per-contact model's regression with the contact-angle terms */
    const double t = xr[4 * q + 2];
    y[2 * q] = (float)willett64((double)xr[4 * q], v, t);
    y[2 * q + 1] = (float)rupture64(v / 8.0, t);
    return;
  }
  LIQUID unit;
  unit.stension = 1.0; unit.vol = 0.0; unit.gapmn = 0.0; unit.layer = 0.0; unit.brknmx = 0.0;
  y[2 * q] = (float)(fcap64((double)xr[4 * q], v, 1.0, unit) / (2.0 * kPiRef));
  y[2 * q + 1] = (float)(0.99 * pow(v / 8.0, 0.33));
}
__global__ void k_formula32(const float* __restrict__ xr, long long n, float* __restrict__ y, int angle) {
  const long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float v = xr[4 * q + 1];
  if (angle) {
    const float t = xr[4 * q + 2];
    y[2 * q] = willett32(xr[4 * q], v, t);
    y[2 * q + 1] = rupture32(0.125f * v, t);
    return;
  }
  y[2 * q] = cap_formula32(xr[4 * q], v);
  y[2 * q + 1] = 0.99f * exp2f(0.33f * __log2f(0.125f * v));
}

/* per-block sums for the standardisation and the hull: columns ln x0, ln x1,
 * x2, x3, y0, y1 -> sum, sum of squares (FP64), min, max of the raw x */
__global__ void k_moments(const float* xr, const float* yr, const int* idx, long long n, double* part,
                          float* mn, float* mx) {
  __shared__ double s1[6][256], s2[6][256];
  __shared__ float lo[4][256], hi[4][256];
  const int t = threadIdx.x;
  double a[6] = {0, 0, 0, 0, 0, 0}, b[6] = {0, 0, 0, 0, 0, 0};
  float l[4] = {3.4e38f, 3.4e38f, 3.4e38f, 3.4e38f}, h[4] = {-3.4e38f, -3.4e38f, -3.4e38f, -3.4e38f};
  for (long long i = blockIdx.x * (long long)blockDim.x + t; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long si = idx[i];
    const float* f = xr + 4 * si;
    const double v[6] = {log((double)f[0]), log((double)f[1]), f[2], f[3], yr[2 * si], yr[2 * si + 1]};
    for (int c = 0; c < 6; c++) { a[c] += v[c]; b[c] += v[c] * v[c]; }
    for (int c = 0; c < 4; c++) { l[c] = fminf(l[c], f[c]); h[c] = fmaxf(h[c], f[c]); }
  }
  for (int c = 0; c < 6; c++) { s1[c][t] = a[c]; s2[c][t] = b[c]; }
  for (int c = 0; c < 4; c++) { lo[c][t] = l[c]; hi[c][t] = h[c]; }
  __syncthreads();
  if (t == 0) {
    for (int c = 0; c < 6; c++) {
      double u = 0, w = 0;
      for (int k = 0; k < (int)blockDim.x; k++) { u += s1[c][k]; w += s2[c][k]; }
      part[blockIdx.x * 12 + c] = u;
      part[blockIdx.x * 12 + 6 + c] = w;
    }
    for (int c = 0; c < 4; c++) {
      float u = 3.4e38f, w = -3.4e38f;
      for (int k = 0; k < (int)blockDim.x; k++) { u = fminf(u, lo[c][k]); w = fmaxf(w, hi[c][k]); }
      mn[blockIdx.x * 4 + c] = u;
      mx[blockIdx.x * 4 + c] = w;
    }
  }
}

dem_status ck(cudaError_t e, const char* what) { return e == cudaSuccess ? DEM_OK : cuda_check(e, what); }

/* host: FP32 parameters + standardisation -> the BF16 staged layout */
void pack_net(const float* P, const float* norm, CapNetSmem* w) {
  std::memset(w, 0, sizeof(*w));
  for (int n = 0; n < kCapH; n++)
    for (int i = 0; i < kCapIn; i++) w->w1[n * kCapS1 + i] = __float2bfloat16(P[kCapW1 + n * kCapIn + i]);
  for (int n = 0; n < kCapH; n++)
    for (int m = 0; m < kCapH; m++) w->w2[n * kCapS2 + m] = __float2bfloat16(P[kCapW2 + n * kCapH + m]);
  for (int o = 0; o < kCapOut; o++)
    for (int m = 0; m < kCapH; m++) w->w3[o * kCapS2 + m] = __float2bfloat16(P[kCapW3 + o * kCapH + m]);
  for (int n = 0; n < kCapH; n++) { w->b1[n] = P[kCapB1 + n]; w->b2[n] = P[kCapB2 + n]; }
  w->b3[0] = P[kCapB3];
  w->b3[1] = P[kCapB3 + 1];
  for (int i = 0; i < 4; i++) {
    w->x_mean[i] = norm[i];
    w->x_inv_std[i] = 1.0f / norm[4 + i];
    w->hull_lo[i] = norm[12 + i];
    w->hull_hi[i] = norm[16 + i];
  }
  for (int o = 0; o < 2; o++) { w->y_mean[o] = norm[8 + o]; w->y_std[o] = norm[10 + o]; }
}

dem_status ensure_packed(dem_capnet* net) {
  if (net->packed_valid) return DEM_OK;
  if (!net->has_norm) return fail(DEM_ERR_STATE, "capnet: no standardisation yet (fit or set it first)");
  std::vector<float> P(kCapParams);
  dem_status st = ck(cudaMemcpy(P.data(), net->params, sizeof(float) * kCapParams, cudaMemcpyDeviceToHost),
                     "capnet params download");
  if (st != DEM_OK) return st;
  CapNetSmem h;
  pack_net(P.data(), net->norm, &h);
  st = ck(cudaMemcpy(net->packed, &h, sizeof(h), cudaMemcpyHostToDevice), "capnet pack upload");
  if (st == DEM_OK) net->packed_valid = true;
  return st;
}

dem_status ensure_partials(dem_capnet* net, int blocks) {
  if (blocks <= net->partial_blocks) return DEM_OK;
  if (net->partial) cudaFree(net->partial);
  net->partial = nullptr;
  net->partial_blocks = 0;
  dem_status st = cuda_alloc((void**)&net->partial, sizeof(float) * (size_t)blocks * (kCapParams + 1));
  if (st == DEM_OK) net->partial_blocks = blocks;
  return st;
}

/* one gradient (and optionally Adam) step over `nb` samples given by idx (device) */
dem_status train_step(dem_capnet* net, const float* x, const float* y, const int* idx, int nb, float lr,
                      float* grad_dev, float* loss_dev, cudaStream_t s) {
  const int blocks = blocks_for(nb, kTB);
  dem_status st = ensure_partials(net, blocks);
  if (st != DEM_OK) return st;
  const Norm nz = norm_of(net);
  k_train<<<blocks, kTB, kTrainSmem, s>>>(net->params, x, y, idx, nb, 1.0f / (float)nb, nz, net->partial);
  float bc1 = 1.f, bc2 = 1.f;
  if (lr > 0.f) {
    net->step++;
    bc1 = 1.f - (float)std::pow(0.9, (double)net->step);
    bc2 = 1.f - (float)std::pow(0.999, (double)net->step);
  }
  k_reduce_adam<<<blocks_for(kCapParams + 1, 256), 256, 0, s>>>(net->params, net->adam_m, net->adam_v, net->partial,
                                                                 blocks, lr, bc1, bc2, grad_dev, loss_dev);
  return ck(cudaGetLastError(), "capnet train launch");
}

}  // namespace
}  // namespace dem

using namespace dem;

extern "C" {

dem_status dem_capnet_create(unsigned long long seed, dem_capnet** out) {
  if (!out) return fail(DEM_ERR_ARG, "dem_capnet_create: null out");
  *out = nullptr;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem);
    if (e != cudaSuccess) return cuda_check(e, "capnet: shared-memory attribute");
    attr = true;
  }
  dem_capnet* net = new dem_capnet();
  std::memset(net, 0, sizeof(*net));
  dem_status st = cuda_alloc((void**)&net->params, sizeof(float) * kCapParams);
  if (st == DEM_OK) st = cuda_alloc((void**)&net->adam_m, sizeof(float) * kCapParams);
  if (st == DEM_OK) st = cuda_alloc((void**)&net->adam_v, sizeof(float) * kCapParams);
  if (st == DEM_OK) st = cuda_alloc((void**)&net->packed, sizeof(CapNetSmem));
  if (st != DEM_OK) {
    dem_capnet_destroy(net);
    return st;
  }
  /* uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, seeded */
  std::vector<float> P(kCapParams);
  std::mt19937_64 rng(seed);
  auto fill = [&](int off, int count, int fan_in) {
    std::uniform_real_distribution<float> u(-1.0f / std::sqrt((float)fan_in), 1.0f / std::sqrt((float)fan_in));
    for (int i = 0; i < count; i++) P[off + i] = u(rng);
  };
  fill(kCapW1, kCapH * kCapIn, kCapIn);
  fill(kCapB1, kCapH, kCapIn);
  fill(kCapW2, kCapH * kCapH, kCapH);
  fill(kCapB2, kCapH, kCapH);
  fill(kCapW3, kCapOut * kCapH, kCapH);
  fill(kCapB3, kCapOut, kCapH);
  st = ck(cudaMemcpy(net->params, P.data(), sizeof(float) * kCapParams, cudaMemcpyHostToDevice), "capnet init");
  if (st == DEM_OK) st = ck(cudaMemset(net->adam_m, 0, sizeof(float) * kCapParams), "capnet init");
  if (st == DEM_OK) st = ck(cudaMemset(net->adam_v, 0, sizeof(float) * kCapParams), "capnet init");
  if (st != DEM_OK) {
    dem_capnet_destroy(net);
    return st;
  }
  *out = net;
  return DEM_OK;
}

void dem_capnet_destroy(dem_capnet* net) {
  if (!net) return;
  cudaFree(net->params);
  cudaFree(net->adam_m);
  cudaFree(net->adam_v);
  cudaFree(net->partial);
  cudaFree(net->packed);
  delete net;
}

dem_status dem_capnet_get(const dem_capnet* net, float* params, float* norm) {
  if (!net) return fail(DEM_ERR_ARG, "dem_capnet_get: null net");
  if (params) {
    dem_status st = ck(cudaMemcpy(params, net->params, sizeof(float) * kCapParams, cudaMemcpyDeviceToHost),
                       "dem_capnet_get");
    if (st != DEM_OK) return st;
  }
  if (norm) std::memcpy(norm, net->norm, sizeof(net->norm));
  return DEM_OK;
}

dem_status dem_capnet_set(dem_capnet* net, const float* params, const float* norm) {
  if (!net) return fail(DEM_ERR_ARG, "dem_capnet_set: null net");
  if (params) {
    dem_status st = ck(cudaMemcpy(net->params, params, sizeof(float) * kCapParams, cudaMemcpyHostToDevice),
                       "dem_capnet_set");
    if (st != DEM_OK) return st;
  }
  if (norm) {
    for (int i = 0; i < 4; i++)
      if (!(norm[4 + i] > 0.f)) return fail(DEM_ERR_ARG, "dem_capnet_set: input deviations must be > 0");
    for (int i = 0; i < 2; i++)
      if (!(norm[10 + i] > 0.f)) return fail(DEM_ERR_ARG, "dem_capnet_set: output deviations must be > 0");
    std::memcpy(net->norm, norm, sizeof(net->norm));
    net->has_norm = true;
  }
  net->packed_valid = false;
  return DEM_OK;
}

dem_status dem_capnet_grad(dem_capnet* net, const float* x_dev, const float* y_dev, int n, float* grad,
                           float* loss) {
  if (!net || !x_dev || !y_dev || n <= 0) return fail(DEM_ERR_ARG, "dem_capnet_grad: bad arguments");
  if (!net->has_norm) return fail(DEM_ERR_STATE, "dem_capnet_grad: set the standardisation first");
  float* buf = nullptr;
  dem_status st = cuda_alloc((void**)&buf, sizeof(float) * (kCapParams + 1));
  if (st != DEM_OK) return st;
  st = train_step(net, x_dev, y_dev, nullptr, n, 0.f, buf, buf + kCapParams, 0);
  if (st == DEM_OK) st = ck(cudaDeviceSynchronize(), "dem_capnet_grad");
  if (st == DEM_OK && grad)
    st = ck(cudaMemcpy(grad, buf, sizeof(float) * kCapParams, cudaMemcpyDeviceToHost), "dem_capnet_grad");
  if (st == DEM_OK && loss)
    st = ck(cudaMemcpy(loss, buf + kCapParams, sizeof(float), cudaMemcpyDeviceToHost), "dem_capnet_grad");
  cudaFree(buf);
  return st;
}

dem_status dem_capnet_infer(dem_capnet* net, const float* x_dev, long long n, int tensor_cores, float* y_dev) {
  if (!net || !x_dev || !y_dev || n < 0) return fail(DEM_ERR_ARG, "dem_capnet_infer: bad arguments");
  if (!net->has_norm) return fail(DEM_ERR_STATE, "dem_capnet_infer: no standardisation");
  if (n == 0) return DEM_OK;
  if (tensor_cores == 2) {
    /* the 5th-generation tensor cores: 128-row tiles, tcgen05.mma into tensor memory */
    dem_status st = ensure_packed(net);
    if (st != DEM_OK) return st;
    int* err = nullptr;
    st = cuda_alloc((void**)&err, sizeof(int));
    if (st != DEM_OK) return st;
    st = ck(cudaMemset(err, 0, sizeof(int)), "dem_capnet_infer");
    const long long tiles = (n + kTcRows - 1) / kTcRows;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int blocks = (int)std::min<long long>(tiles, (long long)std::max(1, sms) * 4);
    if (st == DEM_OK) k_infer_tc5<<<blocks, kTcRows>>>(net->packed, x_dev, n, y_dev, err);
    if (st == DEM_OK) st = ck(cudaGetLastError(), "dem_capnet_infer launch");
    if (st == DEM_OK) st = ck(cudaDeviceSynchronize(), "dem_capnet_infer");
    int h = 0;
    if (st == DEM_OK) st = ck(cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost), "dem_capnet_infer");
    cudaFree(err);
    if (st == DEM_OK && h) st = fail(DEM_ERR_CUDA, "dem_capnet_infer: tensor-core completion not seen in time");
    return st;
  } else if (tensor_cores) {
    dem_status st = ensure_packed(net);
    if (st != DEM_OK) return st;
    const long long tiles = (n + 15) / 16;
    const int blocks = (int)std::min<long long>((tiles + 3) / 4, 152LL * 16);
    k_infer_tc<<<blocks, 128>>>(net->packed, x_dev, n, y_dev);
  } else {
    k_infer32<<<blocks_for(n, 128), 128>>>(net->params, x_dev, n, norm_of(net), y_dev);
  }
  dem_status st = ck(cudaGetLastError(), "dem_capnet_infer launch");
  if (st == DEM_OK) st = ck(cudaDeviceSynchronize(), "dem_capnet_infer");
  return st;
}

dem_status dem_capnet_formula(const float* x_dev, long long n, int fp64, float* y_dev) {
  if (!x_dev || !y_dev || n < 0) return fail(DEM_ERR_ARG, "dem_capnet_formula: bad arguments");
  if (n == 0) return DEM_OK;
  const int angle = (fp64 & 2) != 0;
  if (fp64 & 1) k_formula64<<<blocks_for(n, 256), 256>>>(x_dev, n, y_dev, angle);
  else k_formula32<<<blocks_for(n, 256), 256>>>(x_dev, n, y_dev, angle);
  dem_status st = ck(cudaGetLastError(), "dem_capnet_formula launch");
  if (st == DEM_OK) st = ck(cudaDeviceSynchronize(), "dem_capnet_formula");
  return st;
}

dem_status dem_capnet_fit(dem_capnet* net, const float* x_dev, const float* y_dev, long long n,
                          const dem_capnet_fit_opts* opt, dem_capnet_report* rep) {
  if (!net || !x_dev || !y_dev || n < 16 || !opt) return fail(DEM_ERR_ARG, "dem_capnet_fit: bad arguments");
  if (opt->epochs <= 0 || opt->batch <= 0 || !(opt->lr > 0.f) || opt->val_frac < 0.f || opt->val_frac >= 1.f)
    return fail(DEM_ERR_ARG, "dem_capnet_fit: bad options");
  const auto t0 = std::chrono::steady_clock::now();
  dem_capnet_report r;
  std::memset(&r, 0, sizeof(r));
  /* seeded split */
  std::vector<int> perm((size_t)n);
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937_64 rng(opt->seed);
  std::shuffle(perm.begin(), perm.end(), rng);
  const long long n_val = (long long)std::floor((double)n * opt->val_frac);
  const long long n_tr = n - n_val;
  r.n_train = (int)n_tr;
  r.n_val = (int)n_val;
  int* idx = nullptr;
  dem_status st = cuda_alloc((void**)&idx, sizeof(int) * (size_t)n);
  if (st != DEM_OK) return st;
  std::vector<void*> tmp{idx};
  auto cleanup = [&]() { for (void* p : tmp) cudaFree(p); };
  /* standardisation and hull from the training split */
  {
    const int B = 256, G = 304;
    double* part = nullptr;
    float *mn = nullptr, *mx = nullptr;
    if (st == DEM_OK) st = cuda_alloc((void**)&part, sizeof(double) * G * 12);
    if (part) tmp.push_back(part);
    if (st == DEM_OK) st = cuda_alloc((void**)&mn, sizeof(float) * G * 4);
    if (mn) tmp.push_back(mn);
    if (st == DEM_OK) st = cuda_alloc((void**)&mx, sizeof(float) * G * 4);
    if (mx) tmp.push_back(mx);
    if (st == DEM_OK)
      st = ck(cudaMemcpy(idx, perm.data() + n_val, sizeof(int) * (size_t)n_tr, cudaMemcpyHostToDevice), "fit idx");
    if (st == DEM_OK) {
      k_moments<<<G, B>>>(x_dev, y_dev, idx, n_tr, part, mn, mx);
      st = ck(cudaGetLastError(), "fit moments");
    }
    std::vector<double> hp((size_t)G * 12);
    std::vector<float> hmn((size_t)G * 4), hmx((size_t)G * 4);
    if (st == DEM_OK) st = ck(cudaMemcpy(hp.data(), part, sizeof(double) * G * 12, cudaMemcpyDeviceToHost), "fit");
    if (st == DEM_OK) st = ck(cudaMemcpy(hmn.data(), mn, sizeof(float) * G * 4, cudaMemcpyDeviceToHost), "fit");
    if (st == DEM_OK) st = ck(cudaMemcpy(hmx.data(), mx, sizeof(float) * G * 4, cudaMemcpyDeviceToHost), "fit");
    if (st != DEM_OK) {
      cleanup();
      return st;
    }
    float nrm[20];
    for (int c = 0; c < 6; c++) {
      double u = 0, w = 0;
      for (int b = 0; b < G; b++) { u += hp[b * 12 + c]; w += hp[b * 12 + 6 + c]; }
      const double mean = u / (double)n_tr;
      const double var = std::max(w / (double)n_tr - mean * mean, 0.0);
      const double sd = std::max(std::sqrt(var), 1e-6 * std::max(1.0, std::fabs(mean)));
      if (c < 4) { nrm[c] = (float)mean; nrm[4 + c] = (float)sd; }
      else { nrm[8 + c - 4] = (float)mean; nrm[10 + c - 4] = (float)sd; }
    }
    for (int c = 0; c < 4; c++) {
      float lo = 3.4e38f, hi = -3.4e38f;
      for (int b = 0; b < G; b++) { lo = std::min(lo, hmn[b * 4 + c]); hi = std::max(hi, hmx[b * 4 + c]); }
      nrm[12 + c] = lo;
      nrm[16 + c] = hi;
    }
    std::memcpy(net->norm, nrm, sizeof(nrm));
    net->has_norm = true;
    net->packed_valid = false;
  }
  /* epochs over seeded permutations of the training split */
  std::vector<int> tr(perm.begin() + n_val, perm.end());
  float* loss_dev = nullptr;
  if (st == DEM_OK) st = cuda_alloc((void**)&loss_dev, sizeof(float) * 2);
  if (loss_dev) tmp.push_back(loss_dev);
  for (int ep = 0; ep < opt->epochs && st == DEM_OK; ep++) {
    std::shuffle(tr.begin(), tr.end(), rng);
    st = ck(cudaMemcpy(idx, tr.data(), sizeof(int) * (size_t)n_tr, cudaMemcpyHostToDevice), "fit epoch idx");
    double ep_loss = 0.0;
    long long nsteps = 0;
    for (long long b0 = 0; b0 < n_tr && st == DEM_OK; b0 += opt->batch) {
      const int nb = (int)std::min<long long>(opt->batch, n_tr - b0);
      st = train_step(net, x_dev, y_dev, idx + b0, nb, opt->lr, nullptr, loss_dev, 0);
      if (st == DEM_OK && (b0 / opt->batch) % 64 == 0) {
        float l = 0.f;
        st = ck(cudaMemcpy(&l, loss_dev, sizeof(float), cudaMemcpyDeviceToHost), "fit loss");
        ep_loss += l;
        nsteps++;
      }
    }
    if (ep < 64) r.train_mse[ep] = nsteps ? (float)(ep_loss / (double)nsteps) : 0.f;
    r.epochs = ep + 1;
  }
  net->packed_valid = false;
  /* validation: standardised MSE of the FP32 network, relative errors of the
   * BF16 tensor-core network against the formula's outputs */
  if (st == DEM_OK && n_val > 0) {
    float *xv = nullptr, *yv = nullptr, *yp = nullptr;
    st = cuda_alloc((void**)&xv, sizeof(float) * 4 * (size_t)n_val);
    if (xv) tmp.push_back(xv);
    if (st == DEM_OK) st = cuda_alloc((void**)&yv, sizeof(float) * 2 * (size_t)n_val);
    if (yv) tmp.push_back(yv);
    if (st == DEM_OK) st = cuda_alloc((void**)&yp, sizeof(float) * 2 * (size_t)n_val);
    if (yp) tmp.push_back(yp);
    /* gather the validation rows on the host (deterministic order) */
    std::vector<float> hx((size_t)n * 4), hy((size_t)n * 2), vx((size_t)n_val * 4), vy((size_t)n_val * 2);
    if (st == DEM_OK) st = ck(cudaMemcpy(hx.data(), x_dev, sizeof(float) * 4 * n, cudaMemcpyDeviceToHost), "val");
    if (st == DEM_OK) st = ck(cudaMemcpy(hy.data(), y_dev, sizeof(float) * 2 * n, cudaMemcpyDeviceToHost), "val");
    if (st == DEM_OK) {
      for (long long i = 0; i < n_val; i++) {
        const long long s = perm[(size_t)i];
        for (int c = 0; c < 4; c++) vx[(size_t)i * 4 + c] = hx[(size_t)s * 4 + c];
        for (int c = 0; c < 2; c++) vy[(size_t)i * 2 + c] = hy[(size_t)s * 2 + c];
      }
      st = ck(cudaMemcpy(xv, vx.data(), sizeof(float) * 4 * n_val, cudaMemcpyHostToDevice), "val");
    }
    std::vector<float> p32((size_t)n_val * 2), ptc((size_t)n_val * 2);
    if (st == DEM_OK) st = dem_capnet_infer(net, xv, n_val, 0, yp);
    if (st == DEM_OK) st = ck(cudaMemcpy(p32.data(), yp, sizeof(float) * 2 * n_val, cudaMemcpyDeviceToHost), "val");
    if (st == DEM_OK) st = dem_capnet_infer(net, xv, n_val, 1, yp);
    if (st == DEM_OK) st = ck(cudaMemcpy(ptc.data(), yp, sizeof(float) * 2 * n_val, cudaMemcpyDeviceToHost), "val");
    if (st == DEM_OK) {
      double mse = 0, fm = 0, fx = 0, rx = 0;
      for (long long i = 0; i < n_val; i++) {
        for (int c = 0; c < 2; c++) {
          const double e = (p32[(size_t)i * 2 + c] - vy[(size_t)i * 2 + c]) / net->norm[10 + c];
          mse += e * e;
        }
        const double f = vy[(size_t)i * 2], rf = std::fabs(ptc[(size_t)i * 2] - f) / std::max(std::fabs(f), 1e-30);
        const double rr = std::fabs(ptc[(size_t)i * 2 + 1] - vy[(size_t)i * 2 + 1]) /
                          std::max(std::fabs((double)vy[(size_t)i * 2 + 1]), 1e-30);
        fm += rf;
        fx = std::max(fx, rf);
        rx = std::max(rx, rr);
      }
      r.val_mse = (float)(mse / (double)n_val);
      r.val_force_rel_mean = (float)(fm / (double)n_val);
      r.val_force_rel_max = (float)fx;
      r.val_rupture_rel_max = (float)rx;
    }
  }
  cleanup();
  r.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rep) *rep = r;
  return st;
}

dem_status dem_capnet_samples(dem_ctx* c, float* x_dev, float* y_dev, long long capacity, long long* count) {
  if (!c || !x_dev || !y_dev || capacity < 0 || !count) return fail(DEM_ERR_ARG, "dem_capnet_samples: bad arguments");
  if (c->s.force_cap != 1) return fail(DEM_ERR_STATE, "dem_capnet_samples: the bed has no capillary bridges");
  cudaStream_t s = c->stream;
  dem_status st = DEM_OK;
  if (c->opt.precision == DEM_PREC_MIXED) st = mixed_pre_rebuild(c, c->parity, s); /* bridge counts -> lqd */
  if (st != DEM_OK) return st;
  int* cnt = nullptr;
  long long *off = nullptr, *total = nullptr;
  st = cuda_alloc((void**)&cnt, sizeof(int) * (size_t)c->n);
  if (st == DEM_OK) st = cuda_alloc((void**)&off, sizeof(long long) * (size_t)c->n);
  if (st == DEM_OK) st = cuda_alloc((void**)&total, sizeof(long long));
  SampleArgs a;
  a.pos = c->b.pos; a.rad = c->b.rad; a.nebor = c->b.nebor; a.num_nebor = c->b.num_nebor; a.plevel = c->b.plevel;
  a.nidx = c->b.nidx; a.npars = c->b.npars; a.nneb = c->b.nneb; a.lqd = c->b.lqd; a.id = c->b.id;
  a.brg = c->b.brg; a.n = c->n;
  a.vol = c->s.lqd.vol; a.gapmn = c->s.lqd.gapmn; a.layer = c->s.lqd.layer; a.stension = c->s.lqd.stension;
  a.theta_max = c->theta_max;
  a.theta_seed = c->theta_seed;
  a.lm = c->lm;
  if (st == DEM_OK) {
    k_sample_count<<<blocks_for(c->n, 256), 256, 0, s>>>(a, cnt);
    k_scan_chunks<<<1, 1024, 0, s>>>(cnt, off, c->n, total);
    k_sample_write<<<blocks_for(c->n, 128), 128, 0, s>>>(a, off, capacity, x_dev, y_dev);
    st = ck(cudaGetLastError(), "dem_capnet_samples launch");
  }
  long long tot = 0;
  if (st == DEM_OK) st = ck(cudaMemcpyAsync(&tot, total, sizeof(long long), cudaMemcpyDeviceToHost, s), "samples");
  if (st == DEM_OK) st = ck(cudaStreamSynchronize(s), "dem_capnet_samples");
  cudaFree(cnt);
  cudaFree(off);
  cudaFree(total);
  if (st == DEM_OK) *count = std::min(tot, capacity);
  return st;
}

dem_status dem_set_contact_angles(dem_ctx* c, float theta_max, unsigned long long seed) {
  if (!c || !(theta_max >= 0.f)) return fail(DEM_ERR_ARG, "dem_set_contact_angles: bad arguments");
  c->theta_max = theta_max;
  c->theta_seed = seed;
  /* the captured step kernels hold the old angles: recapture */
  for (int p = 0; p < 2; p++) {
    if (c->graph_exec[p]) { cudaGraphExecDestroy(c->graph_exec[p]); c->graph_exec[p] = nullptr; }
    if (c->graph_one[p]) { cudaGraphExecDestroy(c->graph_one[p]); c->graph_one[p] = nullptr; }
  }
  return DEM_OK;
}

dem_status dem_set_capnet(dem_ctx* c, dem_capnet* net) {
  if (!c || !net) return fail(DEM_ERR_ARG, "dem_set_capnet: null argument");
  if (c->opt.precision != DEM_PREC_MIXED || c->opt.capillary != DEM_CAP_MLP)
    return fail(DEM_ERR_STATE, "dem_set_capnet: the context was not created with mixed precision and DEM_CAP_MLP");
  dem_status st = ensure_packed(net);
  if (st != DEM_OK) return st;
  if (!c->cap_w) {
    st = cuda_alloc(&c->cap_w, sizeof(CapNetSmem));
    if (st != DEM_OK) return st;
    c->allocs.push_back(c->cap_w);
  }
  st = ck(cudaMemcpyAsync(c->cap_w, net->packed, sizeof(CapNetSmem), cudaMemcpyDeviceToDevice, c->stream),
          "dem_set_capnet");
  if (st == DEM_OK) st = ck(cudaStreamSynchronize(c->stream), "dem_set_capnet");
  return st;
}

}  // extern "C"
