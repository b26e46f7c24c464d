// Compositing helpers shared by the compositing kernels (render_kernels.cu) and the fused
// field + compositing render of fixed-count rays (fused_impl.cuh): the degree-2 SH colour head
// (models/sh.py:34-64 composed with a sigmoid), a sample's density and alpha (basis2density
// models/FactorFields.py:639-643, raw2alpha :82-88) and the warp-wide transmittance scan.
#pragma once

#include <cstdint>

#include "ff_common.cuh"

namespace ffgb {

constexpr float kSH_C0 = 0.28209479177387814f;
constexpr float kSH_C1 = 0.4886025119029199f;
constexpr float kSH_C2_0 = 1.0925484305920792f;
constexpr float kSH_C2_1 = -1.0925484305920792f;
constexpr float kSH_C2_2 = 0.31539156525252005f;
constexpr float kSH_C2_3 = -1.0925484305920792f;
constexpr float kSH_C2_4 = 0.5462742152960396f;

// The nine real SH basis values of degree <= 2 with the reference's signs (models/sh.py:49-64).
__device__ __forceinline__ void sh2_basis(const float* d, float* y) {
  const float x = d[0], yy_ = d[1], z = d[2];
  const float xx = x * x, yy = yy_ * yy_, zz = z * z;
  y[0] = kSH_C0;
  y[1] = -kSH_C1 * yy_;
  y[2] = kSH_C1 * z;
  y[3] = -kSH_C1 * x;
  y[4] = kSH_C2_0 * (x * yy_);
  y[5] = kSH_C2_1 * (yy_ * z);
  y[6] = kSH_C2_2 * (2.f * zz - xx - yy);
  y[7] = kSH_C2_3 * (x * z);
  y[8] = kSH_C2_4 * (xx - yy);
}

struct SampleVals {
  float z, delta, f0, sigma, alpha, fac;
};

// A sample's density and alpha (basis2density :639-643 with raw2alpha :82-88) from its first
// feature f0 and its distance to the next sample.
__device__ __forceinline__ SampleVals sample_vals_at(const FFRender& r, float z, float dist, float f0) {
  SampleVals s;
  s.z = z;
  s.delta = __fmul_rn(dist, r.distance_scale);
  s.f0 = f0;
  const float x = s.f0 + r.density_shift;
  if (r.density_act == 0)
    s.sigma = (x > 20.f) ? x : log1pf(expf(x));  // softplus, threshold 20
  else
    s.sigma = fmaxf(x, 0.f);
  s.alpha = 1.f - expf(-s.sigma * s.delta);
  s.fac = 1.f - s.alpha + 1e-10f;
  return s;
}

// Per-chunk exclusive transmittance: T_j = carry * prod_{lanes < j} fac; returns the chunk product.
__device__ __forceinline__ float excl_trans(float fac, int lane, float& excl) {
  float incl = fac;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl *= v;
  }
  excl = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) excl = 1.f;
  return __shfl_sync(0xffffffffu, incl, 31);
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float sigmoidf(float x) { return 1.f / (1.f + expf(-x)); }

// The 28 values of a sample's feature row (density + 27 SH coefficients) in registers. Lane j
// of a warp reads row j, 112 bytes from its neighbour's, so each scalar load instruction touches
// ~28 cache lines: with 16-byte-aligned rows (vec: feat_stride % 4 == 0, aligned base) seven
// float4 loads replace the 28 scalar ones.
constexpr int kRow = 28;

__device__ __forceinline__ void load_row(const float* __restrict__ row, bool vec, float* v) {
  if (vec) {
#pragma unroll
    for (int q = 0; q < kRow / 4; ++q) {
      const float4 t = reinterpret_cast<const float4*>(row)[q];
      v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kRow; ++k) v[k] = row[k];
  }
}

__device__ __forceinline__ void store_row(float* __restrict__ row, bool vec, const float* v) {
  if (vec) {
#pragma unroll
    for (int q = 0; q < kRow / 4; ++q)
      reinterpret_cast<float4*>(row)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
  } else {
#pragma unroll
    for (int k = 0; k < kRow; ++k) row[k] = v[k];
  }
}

__device__ __forceinline__ bool rows_vec(const void* feat, int feat_stride) {
  return (feat_stride % 4) == 0 && (reinterpret_cast<uintptr_t>(feat) & 15) == 0;
}

// Colour of one sample: sigmoid(SH2(dir) . sh[c]) (models/sh.py:34 composed with a sigmoid).
__device__ __forceinline__ void sample_rgb(const float* feat_row, const float* ybasis, float* rgb, float* lin) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float* sh = feat_row + 1 + c * 9;
    float v = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) v += ybasis[k] * sh[k];
    lin[c] = v;
    rgb[c] = sigmoidf(v);
  }
}

}  // namespace ffgb
