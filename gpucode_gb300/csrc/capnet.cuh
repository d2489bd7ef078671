/*
 * capnet.cuh -- the learned capillary closure: device-side definitions shared
 * by the training / sampling kernels (capnet.cu) and the fused step kernel
 * (mixed.cu).
 *
 * The network stands in for the reference's capillary routine fCap
 * (kernel.cu:65-81) and its rupture distance (kernel.cu:518):
 *
 *   inputs   x0 = ln(S+)      S+ = max(gapmn, gap): the separation fCap sees
 *            x1 = ln(V)       V  = 8 (Vi + Vj): the bridge volume fCap sees
 *            x2 = theta       contact angle of the pair (mean of the two
 *                             particles' angles) [rad]
 *            x3 = r_min/r_max radius ratio
 *   outputs  y0 = F / (2 pi R_eff gamma)   the normalised capillary force
 *            y1 = 0.99 (V / 8)^0.33         the rupture distance
 *
 * Lengths are in the reduced unit the reference's kernels work in (the largest
 * diameter), the unit fCap's regression is written in, so R* = 1 and the
 * separation and volume enter as S+/R* and V/R*^3.  The reference's formula
 * does not depend on the contact angle or the radius ratio; the network gets
 * them as inputs all the same.
 *
 * Architecture 4 -> 64 -> 64 -> 2, SiLU, inputs and outputs standardised with
 * the training set's mean and deviation.  Parameters (FP32 master copy):
 *   W1[64][4] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]   (4610 floats)
 * Inference in the step kernel: BF16 weights and activations, FP32
 * accumulation, on the tensor cores one 16-row tile of bridges per warp
 * (mma.sync m16n8k16).
 */
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "liquid.cuh"

namespace dem {

constexpr int kCapIn = 4, kCapH = 64, kCapOut = 2;
constexpr int kCapW1 = 0, kCapB1 = kCapW1 + kCapH * kCapIn, kCapW2 = kCapB1 + kCapH,
              kCapB2 = kCapW2 + kCapH * kCapH, kCapW3 = kCapB2 + kCapH, kCapB3 = kCapW3 + kCapOut * kCapH,
              kCapParams = kCapB3 + kCapOut;
static_assert(kCapParams == 4610, "parameter count");

/* Standardisation, training hull and the network's BF16 weights as the step
 * kernel stages them in shared memory (row strides padded so that the eight
 * rows a fragment load touches fall in distinct banks). */
constexpr int kCapS1 = 24; /* W1 row stride (bf16): k padded 4 -> 16, +8 */
constexpr int kCapS2 = 72; /* W2 / W3 row stride (bf16): 64 + 8 */
struct CapNetSmem {
  __nv_bfloat16 w1[kCapH * kCapS1];
  __nv_bfloat16 w2[kCapH * kCapS2];
  __nv_bfloat16 w3[8 * kCapS2]; /* rows 2..7 zero */
  float b1[kCapH], b2[kCapH], b3[8];
  float x_mean[kCapIn], x_inv_std[kCapIn], y_mean[kCapOut], y_std[kCapOut];
  float hull_lo[kCapIn], hull_hi[kCapIn]; /* raw-feature box of the training set */
};

/* what the engine keeps on the device for DEM_CAP_MLP */
struct CapNetDev {
  const CapNetSmem* w; /* device copy, staged into shared memory per block */
  unsigned long long theta_seed;
  float theta_max;
};

/* is a raw feature vector inside the network's training box? */
__device__ __forceinline__ bool cap_in_hull(const CapNetSmem& w, float sep, float vol, float theta, float ratio) {
  return sep >= w.hull_lo[0] && sep <= w.hull_hi[0] && vol >= w.hull_lo[1] && vol <= w.hull_hi[1] &&
         theta >= w.hull_lo[2] && theta <= w.hull_hi[2] && ratio >= w.hull_lo[3] && ratio <= w.hull_hi[3];
}

/* The plain closure in FP32, normalised: fCap (kernel.cu:65-81) divided by
 * 2 pi R_eff gamma, for sep = max(gapmn, gap) and the volume V it takes.  The
 * hardware approximations of log and exp are used: their errors (a few ulp,
 * relative) stay far below the FP32 force tolerance, and the regression they
 * feed is itself a fit. */
__device__ __forceinline__ float cap_formula32(float sep, float vol) {
  const float sp = sep * rsqrtf(vol);
  const float L = __logf(vol), L2 = L * L, L3 = L2 * L;
  const float f1 = -0.44507f - 0.1119f * L - 0.012101f * L2 - 0.0005f * L3;
  const float f2 = 1.9222f - 0.0668f * L - 0.0013375f * L2;
  const float f3 = 1.268f + 0.198f * L + 0.02232f * L2 + 0.0008585f * L3;
  const float f4 = -0.010703f + 0.03345f * L + 0.0018574f * L2;
  const float ls = __logf(sp);
  return __expf(f1 - f2 * __expf(f3 * ls + f4 * ls * ls));
}

/* SiLU for the BF16 tiles: z sigmoid(z) = h + h tanh(h) with h = z / 2, one
 * hardware tanh (relative error ~2^-11, below the BF16 rounding that follows) */
__device__ __forceinline__ float cap_silu(float z) {
  const float h = 0.5f * z;
  float th;
  asm("tanh.approx.f32 %0, %1;" : "=f"(th) : "f"(h));
  return fmaf(h, th, h);
}

/* ldmatrix: lane l addresses row (l % 8) of 8x8 BF16 matrix (l / 8); each
 * lane receives, per matrix, row (l / 4) elements 2 (l % 4) and +1 -- the
 * B-fragment layout of mma.m16n8k16 for a [n][k] (k contiguous) matrix */
__device__ __forceinline__ void ldsm_x4(uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3, const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(a));
}
__device__ __forceinline__ void ldsm_x2(uint32_t& r0, uint32_t& r1, const void* p) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r0), "=r"(r1) : "r"(a));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

/* the two standardised inputs tile column t (0: ln S+, ln V; 1: angle, ratio)
 * of a row, packed as BF16 */
__device__ __forceinline__ uint32_t cap_pair(const CapNetSmem& w, float sep, float vol, float theta, float ratio,
                                             int t) {
  if (t == 0)
    return pack_bf16((__logf(sep) - w.x_mean[0]) * w.x_inv_std[0], (__logf(vol) - w.x_mean[1]) * w.x_inv_std[1]);
  return pack_bf16((theta - w.x_mean[2]) * w.x_inv_std[2], (ratio - w.x_mean[3]) * w.x_inv_std[3]);
}

/* D += A(16x16, row) * B(16x8, col), BF16 in, FP32 accumulate */
__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

/* One 16-row tile through the network on the tensor cores; all 32 lanes of
 * the warp call it together.  Lane l (g = l / 4, t = l % 4) supplies inputs
 * packed as BF16 pairs: xg = (x0, x1) or (x2, x3) of row g for t = 0 or 1, and
 * xg8 the same of row g + 8 (zero for t >= 2).  On return lanes with t == 0
 * hold the two standardised outputs of rows g (o[0], o[1]) and g + 8 (o[2],
 * o[3]). */
__device__ __forceinline__ void cap_tile16(const CapNetSmem& w, uint32_t xg, uint32_t xg8, float (&o)[4]) {
  const int lane = threadIdx.x & 31, t = lane & 3;
  const int mr = lane & 7, mi = lane >> 3; /* the ldmatrix row this lane addresses */
  /* layer 1 (K = 4 padded to 16) + SiLU, repacked as layer 2's A fragments */
  uint32_t h1[4][4];
#pragma unroll
  for (int c = 0; c < 4; c++) {
    uint32_t bw[2]; /* B fragments (k 0..7) of n-tiles 2c and 2c + 1 */
    ldsm_x2(bw[0], bw[1], w.w1 + (16 * c + (mi & 1) * 8 + mr) * kCapS1);
    float acc[2][4];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int n0 = (2 * c + h) * 8;
      const float bb0 = w.b1[n0 + 2 * t], bb1 = w.b1[n0 + 2 * t + 1];
      acc[h][0] = bb0; acc[h][1] = bb1; acc[h][2] = bb0; acc[h][3] = bb1;
      mma_bf16(acc[h], xg, xg8, 0u, 0u, bw[h], 0u);
    }
    h1[c][0] = pack_bf16(cap_silu(acc[0][0]), cap_silu(acc[0][1]));
    h1[c][1] = pack_bf16(cap_silu(acc[0][2]), cap_silu(acc[0][3]));
    h1[c][2] = pack_bf16(cap_silu(acc[1][0]), cap_silu(acc[1][1]));
    h1[c][3] = pack_bf16(cap_silu(acc[1][2]), cap_silu(acc[1][3]));
  }
  /* layers 2 and 3: 16 hidden units of layer 2 at a time, each chunk fed
   * straight into layer 3 */
  const float ob0 = t == 0 ? w.b3[0] : 0.f, ob1 = t == 0 ? w.b3[1] : 0.f;
  o[0] = ob0; o[1] = ob1; o[2] = ob0; o[3] = ob1;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    float acc[2][4];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int n0 = (2 * c + h) * 8;
      const float bb0 = w.b2[n0 + 2 * t], bb1 = w.b2[n0 + 2 * t + 1];
      acc[h][0] = bb0; acc[h][1] = bb1; acc[h][2] = bb0; acc[h][3] = bb1;
    }
    /* matrices: rows 16c..+7 / 16c+8..+15 of W2 x columns 16kk..+7 / 16kk+8..+15 */
    const __nv_bfloat16* wrow = w.w2 + (16 * c + (mi >> 1) * 8 + mr) * kCapS2 + (mi & 1) * 8;
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      uint32_t q0, q1, q2, q3;
      ldsm_x4(q0, q1, q2, q3, wrow + 16 * kk);
      mma_bf16(acc[0], h1[kk][0], h1[kk][1], h1[kk][2], h1[kk][3], q0, q1);
      mma_bf16(acc[1], h1[kk][0], h1[kk][1], h1[kk][2], h1[kk][3], q2, q3);
    }
    const uint32_t a0 = pack_bf16(cap_silu(acc[0][0]), cap_silu(acc[0][1]));
    const uint32_t a1 = pack_bf16(cap_silu(acc[0][2]), cap_silu(acc[0][3]));
    const uint32_t a2 = pack_bf16(cap_silu(acc[1][0]), cap_silu(acc[1][1]));
    const uint32_t a3 = pack_bf16(cap_silu(acc[1][2]), cap_silu(acc[1][3]));
    uint32_t c0, c1;
    ldsm_x2(c0, c1, w.w3 + mr * kCapS2 + 16 * c + (mi & 1) * 8);
    mma_bf16(o, a0, a1, a2, a3, c0, c1);
  }
}

/* stage the network from global into shared memory (all threads of the block) */
__device__ __forceinline__ void cap_stage(const CapNetSmem* src, CapNetSmem* dst) {
  const int4* s = reinterpret_cast<const int4*>(src);
  int4* d = reinterpret_cast<int4*>(dst);
  constexpr int n16 = (int)(sizeof(CapNetSmem) / 16);
  for (int i = threadIdx.x; i < n16; i += blockDim.x) d[i] = s[i];
}
static_assert(sizeof(CapNetSmem) % 16 == 0, "CapNetSmem is copied in 16-byte words");

}  // namespace dem
