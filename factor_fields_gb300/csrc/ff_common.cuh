// Shared device helpers for the Factor Fields sm_103a kernels.
//
// Arithmetic that decides which grid cell, sample or occupancy bit is used is written with
// explicitly rounded intrinsics (__fadd_rn, __fmul_rn, __fdiv_rn ...) in the same operation
// order as the reference's PyTorch ops, so that the compiler cannot contract it into FMAs and
// indices / interpolation weights come out bit-identical to the reference's float32 values.
#pragma once
#include <utility>

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ff_native.h"

namespace ffgb {

constexpr int kMapSawtooth = FF_MAP_SAWTOOTH;
constexpr int kMapTriangle = FF_MAP_TRIANGLE;

// ---------------------------------------------------------------------------------------
// float32 arithmetic with Python / ATen semantics
// ---------------------------------------------------------------------------------------

// torch.remainder for floats: fmod (exact) shifted into the divisor's sign.
__device__ __forceinline__ float py_rem(float a, float b) {
  float m = fmodf(a, b);
  if (m != 0.f && ((b < 0.f) != (m < 0.f))) m = __fadd_rn(m, b);
  return m;
}

// torch.floor_divide for floats (c10::div_floor_floating).
__device__ __forceinline__ float py_floordiv(float a, float b) {
  float mod = fmodf(a, b);
  float div = __fdiv_rn(__fsub_rn(a, mod), b);
  if (mod != 0.f && ((b < 0.f) != (mod < 0.f))) div = __fsub_rn(div, 1.f);
  float fl;
  if (div != 0.f) {
    fl = floorf(div);
    if (__fsub_rn(div, fl) > 0.5f) fl = __fadd_rn(fl, 1.f);
  } else {
    fl = copysignf(0.f, __fdiv_rn(a, b));
  }
  return fl;
}

// grid_mapping (models/FactorFields.py:11-22) for one coordinate and one level.
__device__ __forceinline__ float map_coord(float p, float origin, float scale, int mapping) {
  const float rel = __fsub_rn(p, origin);
  const float half = __fmul_rn(scale, 0.5f);  // scale / 2, exact
  const float m = py_rem(rel, scale);
  float loc = __fsub_rn(__fdiv_rn(m, half), 1.f);
  if (mapping == kMapTriangle) {
    const float odd = py_rem(py_floordiv(rel, scale), 2.f);
    if (odd == 1.f) loc = -loc;
  } else {
    loc = fminf(fmaxf(loc, -1.f), 1.f);
  }
  return loc;
}

// Division-free grid_mapping for the fused kernels: q = floor(rel / scale) from a reciprocal,
// m = rel - q*scale corrected into [0, scale), loc = m * (2/scale) - 1. Within a few ulp of
// map_coord; both mappings are continuous at the period boundaries where it matters (the
// triangle wave is continuous there, the sawtooth jump is at m = 0 which both compute exactly).
__device__ __forceinline__ float map_coord_fast(float p, float origin, float scale, float inv_scale,
                                                float inv_half, int mapping) {
  const float rel = p - origin;
  float q = floorf(rel * inv_scale);
  float m = fmaf(-q, scale, rel);
  if (m < 0.f) {
    m += scale;
    q -= 1.f;
  } else if (m >= scale) {
    m -= scale;
    q += 1.f;
  }
  float loc = fmaf(m, inv_half, -1.f);
  if (mapping == kMapTriangle) {
    if (((int)q) & 1) loc = -loc;
  } else {
    loc = fminf(fmaxf(loc, -1.f), 1.f);
  }
  return loc;
}

// ATen grid_sampler_unnormalize + border clip (grid_sampler_compute_source_index).
__device__ __forceinline__ float unnorm_align(float c, int size) {  // align_corners=True
  return __fmul_rn(__fmul_rn(__fadd_rn(c, 1.f), 0.5f), (float)(size - 1));
}
__device__ __forceinline__ float unnorm_noalign_border(float c, int size) {  // False + border
  float ix = __fmul_rn(__fsub_rn(__fmul_rn(__fadd_rn(c, 1.f), (float)size), 1.f), 0.5f);
  return fminf((float)(size - 1), fmaxf(ix, 0.f));
}

// normalize_coord (models/FactorFields.py:635-637).
__device__ __forceinline__ float normalize_coord(float x, float origin, float inv) {
  return __fsub_rn(__fmul_rn(__fsub_rn(x, origin), inv), 1.f);
}

// ---------------------------------------------------------------------------------------
// interpolation corners
// ---------------------------------------------------------------------------------------

// Corner set of one bi/trilinear (or nearest) lookup. idx < 0 marks an out-of-bounds corner
// (zero padding): it is neither read nor scattered to. Order: x fastest, then y, then z
// (ATen's nw, ne, sw, se, [bnw ... bse]).
template <int D>
struct Corners {
  static constexpr int K = 1 << D;
  int32_t idx[K];
  float w[K];
};

// Linear corners for coordinates already unnormalised to grid units (ix[k] along axis k,
// size[k] cells). Weights: low corner (x0 + 1) - ix, high corner ix - x0 (both exact), and
// the product is formed x*y*z in that order like ATen.
template <int D>
__device__ __forceinline__ void linear_corners(const float* ix, const int* size, Corners<D>& c) {
  static_assert(D == 2 || D == 3, "bi- or trilinear corners");
  int lo[D], step[D];
  float wl[D], wh[D];
  bool ok_lo[D], ok_hi[D];  // the low / high corner along axis k is inside the grid
  int base = 0;
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float f = floorf(ix[k]);
    lo[k] = (int)f;
    wl[k] = __fsub_rn(__fadd_rn(f, 1.f), ix[k]);
    wh[k] = __fsub_rn(ix[k], f);
    ok_lo[k] = lo[k] >= 0 && lo[k] < size[k];
    ok_hi[k] = lo[k] >= -1 && lo[k] + 1 < size[k];
    step[k] = k == 0 ? 1 : step[k - 1] * size[k - 1];
    base += lo[k] * step[k];
  }
  // weight products in the order x * y (* z), shared by the corners that differ only in z
  float wxy[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) wxy[b] = __fmul_rn((b & 1) ? wh[0] : wl[0], ((b >> 1) & 1) ? wh[1] : wl[1]);
#pragma unroll
  for (int b = 0; b < (1 << D); ++b) {
    int flat = base;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const bool hi = (b >> k) & 1;
      if (hi) flat += step[k];
      ok = ok && (hi ? ok_hi[k] : ok_lo[k]);
    }
    float w = wxy[b & 3];
    if (D == 3) w = __fmul_rn(w, ((b >> 2) & 1) ? wh[D - 1] : wl[D - 1]);
    c.idx[b] = ok ? flat : -1;
    c.w[b] = ok ? w : 0.f;
  }
}

// Linear corners for lookups whose coordinates lie inside the grid on every axis, 0 <= ix <= size-1:
// basis lookups (align_corners=True after grid_mapping, |loc| <= 1) and coefficient lookups
// (border padding clamps). No corner is ever out of bounds, so there are no per-corner checks: the
// low corner is clamped to size-2, and at ix == size-1 the high corner takes weight 1 and the low
// one weight 0, the same nonzero terms as ATen's single in-bounds corner (an axis of size 1 aliases
// both corners onto cell 0, the high one with weight 0). ix is clamped into the grid first, which
// leaves in-range values unchanged and keeps any input (even NaN) inside the buffer. Weights and
// their products are formed exactly as in linear_corners.
template <int D>
__device__ __forceinline__ void linear_corners_inside(const float* ix_in, const int* size, Corners<D>& c) {
  static_assert(D == 2 || D == 3, "bi- or trilinear corners");
  int base = 0, step[D], pitch = 1;
  float wl[D], wh[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    const float ix = fminf(fmaxf(ix_in[k], 0.f), (float)(size[k] - 1));
    const int lo = max(0, min((int)floorf(ix), size[k] - 2));
    const float f = (float)lo;
    wl[k] = __fsub_rn(__fadd_rn(f, 1.f), ix);
    wh[k] = __fsub_rn(ix, f);
    step[k] = size[k] > 1 ? pitch : 0;
    base += lo * pitch;
    pitch *= size[k];
  }
  float wxy[4];
#pragma unroll
  for (int b = 0; b < 4; ++b) wxy[b] = __fmul_rn((b & 1) ? wh[0] : wl[0], ((b >> 1) & 1) ? wh[1] : wl[1]);
#pragma unroll
  for (int b = 0; b < (1 << D); ++b) {
    int flat = base;
#pragma unroll
    for (int k = 0; k < D; ++k)
      if ((b >> k) & 1) flat += step[k];
    float w = wxy[b & 3];
    if (D == 3) w = __fmul_rn(w, ((b >> 2) & 1) ? wh[D - 1] : wl[D - 1]);
    c.idx[b] = flat;
    c.w[b] = w;
  }
}

// Nearest corner (nearbyint = round half to even), stored in slot 0 with weight 1. Outside the
// grid (zero padding; also a NaN coordinate) slot 0 keeps an in-range index, clamped, with weight
// 0, so that gathers which read slot 0 unconditionally stay inside the buffer; the checked
// gather / scatter skip it by its zero weight.
template <int D>
__device__ __forceinline__ void nearest_corner(const float* ix, const int* size, Corners<D>& c) {
  int flat = 0;
  bool ok = true;
#pragma unroll
  for (int k = D - 1; k >= 0; --k) {
    const float r = rintf(ix[k]);
    ok = ok && (r >= 0.f) && (r < (float)size[k]);
    const int ri = min(max((int)fminf(fmaxf(r, 0.f), (float)(size[k] - 1)), 0), size[k] - 1);
    flat = flat * size[k] + ri;
  }
  c.idx[0] = flat;
  c.w[0] = ok ? 1.f : 0.f;
#pragma unroll
  for (int b = 1; b < (1 << D); ++b) {
    c.idx[b] = -1;
    c.w[b] = 0.f;
  }
}

// ---------------------------------------------------------------------------------------
// vector loads (float32 / bf16 storage -> float32 registers) and vector atomics
// ---------------------------------------------------------------------------------------

template <int V>
__device__ __forceinline__ void load_vec(const float* __restrict__ p, float* v) {
  if constexpr (V == 4) {
    const float4 t = __ldg(reinterpret_cast<const float4*>(p));
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  } else if constexpr (V == 2) {
    const float2 t = __ldg(reinterpret_cast<const float2*>(p));
    v[0] = t.x; v[1] = t.y;
  } else {
    v[0] = __ldg(p);
  }
}

template <int V>
__device__ __forceinline__ void load_vec(const __nv_bfloat16* __restrict__ p, float* v) {
  if constexpr (V == 4) {
    const uint2 t = __ldg(reinterpret_cast<const uint2*>(p));
    v[0] = __uint_as_float(t.x << 16); v[1] = __uint_as_float(t.x & 0xffff0000u);
    v[2] = __uint_as_float(t.y << 16); v[3] = __uint_as_float(t.y & 0xffff0000u);
  } else if constexpr (V == 2) {
    const uint32_t t = __ldg(reinterpret_cast<const unsigned int*>(p));
    v[0] = __uint_as_float(t << 16); v[1] = __uint_as_float(t & 0xffff0000u);
  } else {
    const unsigned short t = __ldg(reinterpret_cast<const unsigned short*>(p));
    v[0] = __uint_as_float(((uint32_t)t) << 16);
  }
}

template <int V>
__device__ __forceinline__ void atomic_add_vec(float* p, const float* v) {
  if constexpr (V == 4) {
    atomicAdd(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
  } else if constexpr (V == 2) {
    atomicAdd(reinterpret_cast<float2*>(p), make_float2(v[0], v[1]));
  } else {
    atomicAdd(p, v[0]);
  }
}

// ---------------------------------------------------------------------------------------
// per-point corner sets of the coefficient grid and of one basis level; gather / scatter
// ---------------------------------------------------------------------------------------

// kInside: linear corners without per-corner bounds checks (border padding keeps every lookup
// inside the grid); the fused kernels' gathers then read every corner unconditionally.
template <int CD, bool kInside = false>
__device__ __forceinline__ void coeff_corners(const FFField& f, const float* p, Corners<CD>& cc) {
  float ix[CD];
  int sz[CD];
#pragma unroll
  for (int k = 0; k < CD; ++k) {
    sz[k] = f.coeff_reso[k];
    ix[k] = unnorm_noalign_border(normalize_coord(p[k], f.coeff_origin[k], f.coeff_inv_size[k]), sz[k]);
  }
  if (f.coeff_interp == FF_INTERP_NEAREST)
    nearest_corner<CD>(ix, sz, cc);
  else if constexpr (kInside)
    linear_corners_inside<CD>(ix, sz, cc);
  else
    linear_corners<CD>(ix, sz, cc);
}

template <int BD>
__device__ __forceinline__ void basis_corners(const FFField& f, int l, const float* p, Corners<BD>& bc) {
  float ix[BD];
  int sz[BD];
  const int r = f.level_reso[l];
#pragma unroll
  for (int k = 0; k < BD; ++k) {
    sz[k] = r;
    ix[k] = unnorm_align(map_coord(p[k], f.map_origin[k], f.level_scale[l], f.mapping), r);
  }
  if (f.basis_interp == FF_INTERP_NEAREST)
    nearest_corner<BD>(ix, sz, bc);
  else
    linear_corners<BD>(ix, sz, bc);
}

// Gather V channels at channel offset c of every valid corner (ATen corner order). Offsets are
// 32-bit: every grid (one basis level, one coefficient volume) has fewer than 2^31 elements.
template <int V, int D, typename T>
__device__ __forceinline__ void gather(const T* __restrict__ grid, int stride, int c, const Corners<D>& cn,
                                       float* acc) {
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = 0.f;
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if (cn.idx[k] >= 0 && cn.w[k] != 0.f) {
      float t[V];
      load_vec<V>(grid + (cn.idx[k] * stride + c), t);
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] += t[v] * cn.w[k];
    }
  }
}

template <int V, int D>
__device__ __forceinline__ void scatter(float* __restrict__ grad, int stride, int c, const Corners<D>& cn,
                                        const float* g) {
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if (cn.idx[k] >= 0 && cn.w[k] != 0.f) {
      float t[V];
#pragma unroll
      for (int v = 0; v < V; ++v) t[v] = g[v] * cn.w[k];
      atomic_add_vec<V>(grad + (cn.idx[k] * stride + c), t);
    }
  }
}

// Basis corners with the division-free mapping (fused kernels). The mapped coordinate lies in
// [-1, 1], so every linear lookup is inside the grid (linear_corners_inside).
template <int BD>
__device__ __forceinline__ void basis_corners_fast(const FFField& f, int l, const float* p, Corners<BD>& bc) {
  float ix[BD];
  int sz[BD];
  const int r = f.level_reso[l];
#pragma unroll
  for (int k = 0; k < BD; ++k) {
    sz[k] = r;
    ix[k] = unnorm_align(
        map_coord_fast(p[k], f.map_origin[k], f.level_scale[l], f.level_inv_scale[l], f.level_inv_half[l], f.mapping),
        r);
  }
  if (f.basis_interp == FF_INTERP_NEAREST)
    nearest_corner<BD>(ix, sz, bc);
  else
    linear_corners_inside<BD>(ix, sz, bc);
}

// Gather / scatter over corner sets whose corners are all inside the grid (linear_corners_inside),
// or, with all == false, over slot 0 alone (nearest_corner; the slot is inside the grid for the
// lookups that use these helpers). No index checks: every read is unconditional.
template <int V, int D, typename T>
__device__ __forceinline__ void gather_inside(const T* __restrict__ grid, int stride, const Corners<D>& cn, bool all,
                                              float* acc) {
#pragma unroll
  for (int v = 0; v < V; ++v) acc[v] = 0.f;
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if (k == 0 || all) {
      float t[V];
      load_vec<V>(grid + cn.idx[k] * stride, t);
#pragma unroll
      for (int v = 0; v < V; ++v) acc[v] += t[v] * cn.w[k];
    }
  }
}

// Zero-weight corners (nearest's unused slots, the weight-0 corner at the grid's far edge) are
// skipped: they would add zeros. Two channels per corner, packed (stride 2, 16-byte-aligned
// level): the x-adjacent corners k, k + 1 of a lookup are neighbouring 8-byte entries, and when
// the low one has an even index they share one 16-byte chunk: one float4 atomic covers both.
template <int V, int D>
__device__ __forceinline__ void scatter_inside(float* __restrict__ grad, int stride, const Corners<D>& cn,
                                               const float* g) {
  if constexpr (V == 2) {
    const bool packed = stride == 2 && (reinterpret_cast<uintptr_t>(grad) & 15) == 0;
#pragma unroll
    for (int k = 0; k < Corners<D>::K; k += 2) {
      const int i0 = cn.idx[k];
      const float w0 = cn.w[k], w1 = cn.w[k + 1];
      if (packed && (i0 & 1) == 0 && cn.idx[k + 1] == i0 + 1) {
        atomicAdd(reinterpret_cast<float4*>(grad + i0 * 2), make_float4(g[0] * w0, g[1] * w0, g[0] * w1, g[1] * w1));
      } else {
        if (w0 != 0.f) atomicAdd(reinterpret_cast<float2*>(grad + i0 * stride), make_float2(g[0] * w0, g[1] * w0));
        if (w1 != 0.f)
          atomicAdd(reinterpret_cast<float2*>(grad + cn.idx[k + 1] * stride), make_float2(g[0] * w1, g[1] * w1));
      }
    }
  } else {
#pragma unroll
    for (int k = 0; k < Corners<D>::K; ++k) {
      if (cn.w[k] != 0.f) {
        float t[V];
#pragma unroll
        for (int v = 0; v < V; ++v) t[v] = g[v] * cn.w[k];
        atomic_add_vec<V>(grad + cn.idx[k] * stride, t);
      }
    }
  }
}

// All 18 coefficient channels of every valid corner with 16-byte loads (channels 0..15) and
// one 4- (BF16) or 8-byte (float32) load for channels 16, 17. Needs coeff_stride % 8 == 0.
// Corner sets as in gather_inside (all: every corner; else slot 0 only).
// kSkipZero: corners of zero weight are not loaded. For image-set lookups (a 2-D basis with a 3-D
// coefficient volume over (x, y, image)) the image coordinate sits on a voxel centre, so half of
// the 8 corners carry weight 0; elsewhere zero weights are rare and the test costs more than it
// saves.
template <int D, bool kSkipZero = false>
__device__ __forceinline__ void gather_coeff18(const __nv_bfloat16* __restrict__ grid, int stride, const Corners<D>& cn,
                                               bool all, float* acc) {
#pragma unroll
  for (int v = 0; v < 18; ++v) acc[v] = 0.f;
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if ((k == 0 || all) && (!kSkipZero || cn.w[k] != 0.f)) {
      const __nv_bfloat16* p = grid + (int64_t)cn.idx[k] * stride;
      const uint4 a = __ldg(reinterpret_cast<const uint4*>(p));
      const uint4 b = __ldg(reinterpret_cast<const uint4*>(p + 8));
      const uint32_t c = __ldg(reinterpret_cast<const unsigned int*>(p + 16));
      const uint32_t w[9] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c};
      const float wk = cn.w[k];
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        acc[2 * j] += __uint_as_float(w[j] << 16) * wk;
        acc[2 * j + 1] += __uint_as_float(w[j] & 0xffff0000u) * wk;
      }
    }
  }
}

template <int D, bool kSkipZero = false>
__device__ __forceinline__ void gather_coeff18(const float* __restrict__ grid, int stride, const Corners<D>& cn,
                                               bool all, float* acc) {
#pragma unroll
  for (int v = 0; v < 18; ++v) acc[v] = 0.f;
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if ((k == 0 || all) && (!kSkipZero || cn.w[k] != 0.f)) {
      const float* p = grid + (int64_t)cn.idx[k] * stride;
      const float wk = cn.w[k];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(p) + j);
        acc[4 * j] += t.x * wk; acc[4 * j + 1] += t.y * wk; acc[4 * j + 2] += t.z * wk; acc[4 * j + 3] += t.w * wk;
      }
      const float2 t = __ldg(reinterpret_cast<const float2*>(p + 16));
      acc[16] += t.x * wk;
      acc[17] += t.y * wk;
    }
  }
}

// Scatter 18 coefficient-channel gradients (float32 grid, stride % 4 == 0): four float4 and
// one float2 atomic per corner of nonzero weight (corner sets as in gather_inside).
template <int D>
__device__ __forceinline__ void scatter_coeff18(float* __restrict__ grad, int stride, const Corners<D>& cn,
                                                const float* g) {
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if (cn.w[k] != 0.f) {
      float* p = grad + (int64_t)cn.idx[k] * stride;
      const float wk = cn.w[k];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        atomicAdd(reinterpret_cast<float4*>(p) + j,
                  make_float4(g[4 * j] * wk, g[4 * j + 1] * wk, g[4 * j + 2] * wk, g[4 * j + 3] * wk));
      atomicAdd(reinterpret_cast<float2*>(p + 16), make_float2(g[16] * wk, g[17] * wk));
    }
  }
}

// ---------------------------------------------------------------------------------------
// misc
// ---------------------------------------------------------------------------------------

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Trilinear value of the 0/1 occupancy volume at p (AlphaGridMask.sample_alpha,
// models/FactorFields.py:103-107): float32 sum of the weights of the occupied corners in ATen's corner order, zero padding.
__device__ __forceinline__ float occupancy_value(const FFRender& r, const float* p) {
  float ix[3];
  int sz[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    sz[k] = r.occ_reso[k];
    const float u = __fsub_rn(__fmul_rn(__fsub_rn(p[k], r.occ_origin[k]), r.occ_inv[k]), 1.f);
    ix[k] = unnorm_align(u, sz[k]);
  }
  Corners<3> c;
  linear_corners<3>(ix, sz, c);
  float val = 0.f;
#pragma unroll
  for (int b = 0; b < 8; ++b) {
    if (c.idx[b] >= 0) {
      const uint32_t word = __ldg(r.occ_bits + (c.idx[b] >> 5));
      if ((word >> (c.idx[b] & 31)) & 1u) val = __fadd_rn(val, c.w[b]);
    }
  }
  return val;
}

// The alpha-mask test of FactorFields.forward (models/FactorFields.py:866): sample_alpha > 0.5.
__device__ __forceinline__ bool occupied(const FFRender& r, const float* p) { return occupancy_value(r, p) > 0.5f; }

// Programmatic dependent launch (the binned fit step's chain: bin -> alloc -> permute -> fit). A
// kernel launched with launch_pdl may start while the kernel before it in the stream still runs,
// once that kernel has executed pdl_launch_dependents (or ended); it does its independent prologue,
// then pdl_wait() returns when the kernel before it has completed and its memory is visible.
// Without a programmatic launch both are no-ops.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace ffgb
