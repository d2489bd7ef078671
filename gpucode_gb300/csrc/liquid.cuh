/*
 * liquid.cuh -- the per-contact liquid-bridge model (host and device).
 *
 * The reference splits one liquid fraction per particle over its bridges
 * (LIQUID.vol (2r)^3 / max(12, bridges), kernel.cu:429-434, :511-515) and
 * evaluates the capillary regression at zero contact angle (fCap,
 * kernel.cu:65-81).  That regression is the closed-form fit of Willett,
 * Adams, Johnson and Seville (2000, "Capillary bridges between two spherical
 * bodies", Langmuir 16:9396) with its contact-angle terms set to zero: each of
 * its four functions f1..f4 of ln V* has coefficients quadratic in the
 * contact angle theta (radians), and the reference keeps the constant ones.
 *
 * DEM_LIQUID_PER_CONTACT (no counterpart in the reference) evaluates the same
 * fit with its theta terms:
 *   - every particle has a contact angle, uniform in [0, theta_max] from a
 *     hash of its id and a seed; a pair takes the mean of its two;
 *   - every unordered pair has a bridge volume, a fraction uniform in
 *     [vol_min, vol_max] (a hash of the two ids and the seed, so both
 *     directions of the pair agree) of the smaller sphere's volume
 *     (pi/6 (2 r_min)^3, reduced units);
 *   - the force is 2 pi R_eff gamma F*(S+, V*, theta) with the fit's
 *     F* = exp(f1 - f2 exp(f3 ln S+ + f4 ln^2 S+)), S+ = max(gapmn, S) /
 *     sqrt(V*), V* = 8 V -- the reference's scaling of fCap's arguments;
 *   - the bridge ruptures beyond (1 + theta / 2) 0.99 V^0.33: the reference's
 *     rupture distance (kernel.cu:518) with the contact-angle factor of Lian,
 *     Thornton and Adams (1993), S_c = (1 + theta / 2) V^(1/3).
 * Formation (gap below 2 layer (r_i + r_j)) and the bridge flags are the
 * reference's.  At theta = 0 the fit's coefficients are exactly fCap's.
 */
#pragma once

#include <cuda_runtime.h>

namespace dem {

/* per-contact liquid model as the kernels take it (mode 0: the reference's) */
struct LiquidModel {
  int mode;
  float theta_max;
  double vol_min, vol_max;
  unsigned long long seed;
};

__host__ __device__ inline unsigned long long liquid_mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* contact angles: uniform in [0, theta_max] per particle, from a hash of its id */
__host__ __device__ inline float cap_theta(int id, unsigned long long seed, float theta_max) {
  const unsigned long long z = liquid_mix64(seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(id + 1));
  return theta_max * (float)((double)(z >> 11) * (1.0 / 9007199254740992.0));
}

/* uniform in [0, 1) for the unordered pair {a, b} */
__host__ __device__ inline double pair_uniform(int a, int b, unsigned long long seed) {
  const unsigned long long lo = (unsigned long long)(a < b ? a : b), hi = (unsigned long long)(a < b ? b : a);
  const unsigned long long z =
      liquid_mix64(liquid_mix64(seed ^ (0xD1B54A32D192ED03ull * (lo + 1))) + 0x9E3779B97F4A7C15ull * (hi + 1));
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

/* the bridge volume of pair {ida, idb} (reduced units): a fraction of the
 * smaller sphere's volume, pi/6 (2 r_min)^3 with the reference's pi */
__host__ __device__ inline double pair_bridge_volume(const LiquidModel& m, int ida, int idb, double r_min) {
  const double f = m.vol_min + (m.vol_max - m.vol_min) * pair_uniform(ida, idb, m.seed);
  const double d = 2.0 * r_min;
  return f * (3.1415926 / 6.0) * (d * d * d);
}

#ifdef __CUDACC__
/* FP32 forms for the mixed-precision step (no FP64 operations): the same
 * hashes with 24-bit uniforms, within 2^-24 of the FP64 forms' */
__device__ __forceinline__ float cap_theta32(int id, unsigned long long seed, float theta_max) {
  const unsigned long long z = liquid_mix64(seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(id + 1));
  return theta_max * ((float)(unsigned)(z >> 40) * 5.9604644775390625e-8f);
}
__device__ __forceinline__ float pair_bridge_volume32(int a, int b, unsigned long long seed, float vmin, float vspan,
                                                      float r_min) {
  const unsigned long long lo = (unsigned long long)(a < b ? a : b), hi = (unsigned long long)(a < b ? b : a);
  const unsigned long long z =
      liquid_mix64(liquid_mix64(seed ^ (0xD1B54A32D192ED03ull * (lo + 1))) + 0x9E3779B97F4A7C15ull * (hi + 1));
  const float f = vmin + vspan * ((float)(unsigned)(z >> 40) * 5.9604644775390625e-8f);
  const float d = 2.0f * r_min;
  return f * (3.1415926f / 6.0f) * (d * d * d);
}

/* F*(S+, V*, theta) of the fit, FP64: s = max(gapmn, S) (not yet divided by
 * sqrt(V*)), v = V* = 8 V, t = theta */
__device__ __forceinline__ double willett64(double s, double v, double t) {
  const double t2 = t * t;
  const double L = log(v), L2 = L * L, L3 = L2 * L;
  const double f1 = (-0.44507 + 0.050832 * t - 1.1466 * t2) + (-0.1119 - 0.000411 * t - 0.1490 * t2) * L +
                    (-0.012101 - 0.0036456 * t - 0.01255 * t2) * L2 +
                    (-0.0005 - 0.0003505 * t - 0.00029076 * t2) * L3;
  const double f2 = (1.9222 - 0.57473 * t - 1.2918 * t2) + (-0.0668 - 0.1201 * t - 0.22574 * t2) * L +
                    (-0.0013375 - 0.0068988 * t - 0.01137 * t2) * L2;
  const double f3 = (1.268 - 0.01396 * t - 0.23566 * t2) + (0.198 + 0.092 * t - 0.06418 * t2) * L +
                    (0.02232 + 0.02238 * t - 0.009853 * t2) * L2 + (0.0008585 + 0.001318 * t - 0.00053 * t2) * L3;
  const double f4 = (-0.010703 + 0.073776 * t - 0.34742 * t2) + (0.03345 + 0.04543 * t - 0.09056 * t2) * L +
                    (0.0018574 + 0.004456 * t - 0.006257 * t2) * L2;
  const double ls = log(s / sqrt(v));
  return exp(f1 - f2 * exp(f3 * ls + f4 * ls * ls));
}

/* the same in FP32 with the hardware log / exp (a few ulp relative, far below
 * the FP32 force tolerance) */
__device__ __forceinline__ float willett32(float s, float v, float t) {
  const float t2 = t * t;
  const float L = __logf(v), L2 = L * L, L3 = L2 * L;
  const float f1 = (-0.44507f + 0.050832f * t - 1.1466f * t2) + (-0.1119f - 0.000411f * t - 0.1490f * t2) * L +
                   (-0.012101f - 0.0036456f * t - 0.01255f * t2) * L2 +
                   (-0.0005f - 0.0003505f * t - 0.00029076f * t2) * L3;
  const float f2 = (1.9222f - 0.57473f * t - 1.2918f * t2) + (-0.0668f - 0.1201f * t - 0.22574f * t2) * L +
                   (-0.0013375f - 0.0068988f * t - 0.01137f * t2) * L2;
  const float f3 = (1.268f - 0.01396f * t - 0.23566f * t2) + (0.198f + 0.092f * t - 0.06418f * t2) * L +
                   (0.02232f + 0.02238f * t - 0.009853f * t2) * L2 +
                   (0.0008585f + 0.001318f * t - 0.00053f * t2) * L3;
  const float f4 = (-0.010703f + 0.073776f * t - 0.34742f * t2) + (0.03345f + 0.04543f * t - 0.09056f * t2) * L +
                   (0.0018574f + 0.004456f * t - 0.006257f * t2) * L2;
  const float ls = __logf(s * rsqrtf(v));
  return __expf(f1 - f2 * __expf(f3 * ls + f4 * ls * ls));
}

/* rupture distance of a bridge of volume V (reduced, unscaled) and contact angle t */
__device__ __forceinline__ double rupture64(double V, double t) { return (1.0 + 0.5 * t) * (0.99 * pow(V, 0.33)); }
__device__ __forceinline__ float rupture32(float V, float t) {
  return (1.0f + 0.5f * t) * (0.99f * exp2f(0.33f * __log2f(V)));
}
#endif /* __CUDACC__ */

}  // namespace dem
