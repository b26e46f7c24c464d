// Ray marching, compaction and alpha compositing for bounded scenes.
//
// Replaces FactorFields.forward's sampling and compositing (models/FactorFields.py:843-898):
//   sample_point         :586-602  slab entry t_min, z_i = t_min + step * (i + u), in-box mask
//   AlphaGridMask        :91-110, :865-867  trilinear lookup of the 0/1 volume > 0.5
//   boolean compaction   :863-885  xyz_sampled[ray_valid], row-major order
//   raw2alpha + composite :82-88, :876-896  softplus density, alpha, cumprod transmittance,
//                         weights, colour head on w > thres, acc / rgb / white bg / clamp / depth
// with the colour head = degree-2 SH (models/sh.py:34-64) + sigmoid.
//
// Everything that decides WHICH sample is live (positions, in-box test, occupancy) uses
// explicitly rounded float32 ops in the reference's order, so the live set and its order are
// bit-identical to the reference. The occupancy volume is a bitfield: the reference's rule
// (trilinear interpolation of 0/1 values, > 0.5) is evaluated exactly from the 8 corner bits.
//
// Warp per ray throughout: marching tests 32 samples per step and compacts them with a
// ballot + popc prefix; compositing runs a 32-wide multiplicative scan per chunk with the
// running transmittance carried between chunks; the backward runs the forward again, then a
// reverse affine scan for sum_{k>j} dL/dw_k * alpha_k * prod_{j<m<k} (1 - alpha_m + 1e-10).
#include <mutex>

#include "composite_common.cuh"
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kRayWarps = 8;  // warps (rays) per block
// The compositing kernels: blocks of 4 rays, registers capped so that 7 blocks fit per SM (1,064
// resident rays): a 4,096-ray batch runs in one wave, so the kernel lasts about as long as its
// longest ray instead of two block generations.
constexpr int kCompWarps = 4;
constexpr int kCompBlocksPerSM = 7;

struct RayGeo {
  float o[3], d[3], t_min, u;
};

__device__ __forceinline__ RayGeo ray_setup(const FFRender& r, const float* rays, const float* jitter, int64_t ray) {
  RayGeo g;
  float tm = -INFINITY;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    g.o[k] = rays[ray * 6 + k];
    g.d[k] = rays[ray * 6 + 3 + k];
    const float vec = (g.d[k] == 0.f) ? 1e-6f : g.d[k];
    const float ra = __fdiv_rn(__fsub_rn(r.aabb_max[k], g.o[k]), vec);
    const float rb = __fdiv_rn(__fsub_rn(r.aabb_min[k], g.o[k]), vec);
    tm = fmaxf(tm, fminf(ra, rb));
  }
  g.t_min = fminf(fmaxf(tm, 0.05f), 1e3f);
  g.u = jitter ? jitter[ray] : 0.f;
  return g;
}

// z of sample i: t_min + step * (i + u)  (float32, reference order)
__device__ __forceinline__ float sample_z(const FFRender& r, const RayGeo& g, int i) {
  const float rng = (g.u != 0.f) ? __fadd_rn((float)i, g.u) : (float)i;
  return __fadd_rn(g.t_min, __fmul_rn(r.step, rng));
}

// Sample i of the ray: live (in the box and, with a mask, occupied) and its position.
__device__ __forceinline__ bool sample_live(const FFRender& r, const RayGeo& g, int i, float* p) {
  const float z = sample_z(r, g, i);
  bool in = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p[k] = __fadd_rn(g.o[k], __fmul_rn(g.d[k], z));
    in = in && !(r.aabb_min[k] > p[k] || p[k] > r.aabb_max[k]);
  }
  if (in && r.occ_bits) in = occupied(r, p);
  return in;
}

// filtering_rays (:825-841), warp per ray. bbox_only: the ray meets the aabb (t_max > t_min of
// the slab test, no clamping). Else: some sample z_i = t_min + step * i, i < n_samples (no
// jitter, all samples, in the box or not) has sample_alpha > 0.
__global__ void __launch_bounds__(kRayWarps * 32) filter_rays_kernel(const FFRender r, const float* __restrict__ rays,
                                                                    int64_t n_rays, int n_samples, int bbox_only,
                                                                    uint8_t* __restrict__ keep) {
  const int lane = threadIdx.x & 31;
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    bool hit = false;
    if (bbox_only) {
      float tmin = -INFINITY, tmax = INFINITY;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float o = rays[ray * 6 + k], d = rays[ray * 6 + 3 + k];
        const float vec = (d == 0.f) ? 1e-6f : d;
        const float ra = __fdiv_rn(__fsub_rn(r.aabb_max[k], o), vec);
        const float rb = __fdiv_rn(__fsub_rn(r.aabb_min[k], o), vec);
        tmin = fmaxf(tmin, fminf(ra, rb));
        tmax = fminf(tmax, fmaxf(ra, rb));
      }
      hit = tmax > tmin;
    } else {
      const RayGeo g = ray_setup(r, rays, nullptr, ray);
      for (int i0 = 0; i0 < n_samples && !hit; i0 += 32) {
        const int i = i0 + lane;
        bool h = false;
        if (i < n_samples) {
          const float z = sample_z(r, g, i);
          float p[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) p[k] = __fadd_rn(g.o[k], __fmul_rn(g.d[k], z));
          h = occupancy_value(r, p) > 0.f;
        }
        hit = __any_sync(0xffffffffu, h);
      }
    }
    if (lane == 0) keep[ray] = hit ? 1 : 0;
  }
}

__global__ void __launch_bounds__(kRayWarps * 32) march_count_kernel(const FFRender r, const float* __restrict__ rays,
                                                                    const float* __restrict__ jitter, int64_t n_rays,
                                                                    int32_t* __restrict__ counts,
                                                                    float* __restrict__ t_min) {
  const int lane = threadIdx.x & 31;
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const RayGeo g = ray_setup(r, rays, jitter, ray);
    int cnt = 0;
    for (int i0 = 0; i0 < r.n_samples; i0 += 32) {
      const int i = i0 + lane;
      float p[3];
      const bool live = (i < r.n_samples) && sample_live(r, g, i, p);
      cnt += __popc(__ballot_sync(0xffffffffu, live));
    }
    if (lane == 0) {
      counts[ray] = cnt;
      if (t_min) t_min[ray] = g.t_min;
    }
  }
}

__global__ void __launch_bounds__(kRayWarps * 32) march_emit_kernel(const FFRender r, const float* __restrict__ rays,
                                                                   const float* __restrict__ jitter, int64_t n_rays,
                                                                   const int64_t* __restrict__ offsets,
                                                                   float* __restrict__ xyz,
                                                                   int32_t* __restrict__ sample_idx) {
  const int lane = threadIdx.x & 31;
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const RayGeo g = ray_setup(r, rays, jitter, ray);
    int64_t pos = offsets[ray];
    for (int i0 = 0; i0 < r.n_samples; i0 += 32) {
      const int i = i0 + lane;
      float p[3];
      const bool live = (i < r.n_samples) && sample_live(r, g, i, p);
      const uint32_t m = __ballot_sync(0xffffffffu, live);
      if (live) {
        const int64_t j = pos + __popc(m & ((1u << lane) - 1u));
        xyz[j * 3 + 0] = p[0];
        xyz[j * 3 + 1] = p[1];
        xyz[j * 3 + 2] = p[2];
        sample_idx[j] = i;
      }
      pos += __popc(m);
    }
  }
}

// ---- exclusive scan of per-ray counts (two levels through a caller workspace) ----------

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ int64_t block_excl_scan(int64_t v, int64_t* warp_sums, int64_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int64_t s = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    warp_sums[lane] = s;
  }
  __syncthreads();
  total = warp_sums[(blockDim.x >> 5) - 1];
  const int64_t before = warp > 0 ? warp_sums[warp - 1] : 0;
  __syncthreads();
  return before + x - v;
}

__global__ void __launch_bounds__(kScanThreads) scan_blocks_kernel(const int32_t* __restrict__ counts, int64_t n,
                                                                   int64_t* __restrict__ block_sums) {
  __shared__ int64_t ws[32];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  int64_t v = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < n) v += counts[base + k];
  int64_t total;
  block_excl_scan(v, ws, total);
  if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Scans the block sums in place (one block, looping over chunks of the sums array).
__global__ void __launch_bounds__(kScanThreads) scan_sums_kernel(int64_t* __restrict__ block_sums, int64_t nb) {
  __shared__ int64_t ws[32];
  int64_t carry = 0;
  for (int64_t c = 0; c < nb; c += kScanThreads) {
    const int64_t i = c + threadIdx.x;
    const int64_t v = i < nb ? block_sums[i] : 0;
    int64_t total;
    const int64_t ex = block_excl_scan(v, ws, total);
    if (i < nb) block_sums[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const int32_t* __restrict__ counts, int64_t n,
                                                                  const int64_t* __restrict__ block_prefix,
                                                                  int64_t* __restrict__ offsets) {
  __shared__ int64_t ws[32];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
  int64_t vals[kScanItems];
  int64_t v = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    vals[k] = (base + k < n) ? counts[base + k] : 0;
    v += vals[k];
  }
  int64_t total;
  int64_t run = block_prefix[blockIdx.x] + block_excl_scan(v, ws, total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) offsets[base + k] = run;
    run += vals[k];
  }
  if (base + kScanItems >= n && base < n) offsets[n] = run;  // the thread holding the last element
}

// ---- compositing --------------------------------------------------------------------

// zd (optional): explicit (z, dist) of the sample, for samplers other than the uniform one.
__device__ __forceinline__ SampleVals sample_vals(const FFRender& r, const RayGeo& g, int i, const float* feat_row,
                                                  const float* zd = nullptr) {
  if (zd) return sample_vals_at(r, zd[0], zd[1], feat_row[0]);
  const float z = sample_z(r, g, i);
  const float dist = (i + 1 < r.n_samples) ? __fsub_rn(sample_z(r, g, i + 1), z) : 0.f;  // :861
  return sample_vals_at(r, z, dist, feat_row[0]);
}

// Colour source of the compositing kernels: the SH-2 head evaluated from the feature row
// (kColSH), or per-sample colours computed beforehand by another head (kColExt: rgb_sample
// [M, 3], read for the samples whose weight passes the threshold; MLPRender_Fea, :884-885).
enum { kColSH = 0, kColExt = 1 };

template <int kCol>
__global__ void __launch_bounds__(kCompWarps * 32, kCompBlocksPerSM) composite_forward_kernel(
    const FFRender r, const float* __restrict__ rays, const float* __restrict__ jitter, int64_t n_rays,
    const int64_t* __restrict__ offsets, const int32_t* __restrict__ sample_idx, const float* __restrict__ feat,
    int feat_stride, const int32_t* __restrict__ white_bg, float* __restrict__ rgb_out, float* __restrict__ depth_out,
    float* __restrict__ acc_out, const float* __restrict__ zd, float* __restrict__ w_out,
    const float* __restrict__ rgb_sample) {
  const int lane = threadIdx.x & 31;
  const bool vec = kCol == kColSH && rows_vec(feat, feat_stride);
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const RayGeo g = ray_setup(r, rays, jitter, ray);
    float yb[9];
    sh2_basis(g.d, yb);
    const int64_t beg = offsets[ray], end = offsets[ray + 1];
    float T = 1.f, acc = 0.f, depth = 0.f, col[3] = {0.f, 0.f, 0.f};
    for (int64_t c0 = beg; c0 < end; c0 += 32) {
      const int64_t j = c0 + lane;
      const bool active = j < end;
      SampleVals s = {0.f, 0.f, 0.f, 0.f, 0.f, 1.f};
      float row[kRow];
      if (active) {
        if constexpr (kCol == kColSH)
          load_row(feat + j * feat_stride, vec, row);
        else
          row[0] = feat[j * feat_stride];
        s = sample_vals(r, g, zd ? 0 : sample_idx[j], row, zd ? zd + 2 * j : nullptr);
      }
      float excl;
      const float prod = excl_trans(s.fac, lane, excl);
      const float w = active ? s.alpha * (T * excl) : 0.f;
      if (active && w_out) w_out[j] = w;
      acc += w;
      depth += w * s.z;
      if (active && w > r.weight_thres) {
        float c[3];
        if constexpr (kCol == kColSH) {
          float lin[3];
          sample_rgb(row, yb, c, lin);
        } else {
          c[0] = rgb_sample[j * 3]; c[1] = rgb_sample[j * 3 + 1]; c[2] = rgb_sample[j * 3 + 2];
        }
        col[0] += w * c[0]; col[1] += w * c[1]; col[2] += w * c[2];
      }
      T *= prod;
    }
    acc = warp_sum(acc);
    depth = warp_sum(depth);
    col[0] = warp_sum(col[0]); col[1] = warp_sum(col[1]); col[2] = warp_sum(col[2]);
    if (lane == 0) {
      const bool wb = white_bg ? (*white_bg != 0) : (r.white_bg != 0);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float v = col[c];
        if (wb) v = v + (1.f - acc);
        rgb_out[ray * 3 + c] = fminf(fmaxf(v, 0.f), 1.f);
      }
      if (depth_out) depth_out[ray] = depth;
      if (acc_out) acc_out[ray] = acc;
    }
  }
}

// Values of one live sample that the reverse pass needs, parked by the forward pass in the
// sample's gradient row (which the reverse pass overwrites) when the row has >= 8 floats:
// exclusive transmittance T, alpha, fac = 1 - alpha + 1e-10, exp(-sigma delta) delta (d alpha /
// d sigma), d sigma / d f0, and the colour (zero below the weight threshold).
constexpr int kPark = 8;

struct Parked {
  float T, alpha, fac, ed, dsig, c[3];
};

__device__ __forceinline__ float dsigma_df0(const FFRender& r, float f0) {
  const float x = f0 + r.density_shift;
  if (r.density_act == 0) return (x > 20.f) ? 1.f : sigmoidf(x);  // softplus, threshold 20
  return x > 0.f ? 1.f : 0.f;
}

__device__ __forceinline__ void park_store(float* row, bool vec, const Parked& p) {
  if (vec) {
    reinterpret_cast<float4*>(row)[0] = make_float4(p.T, p.alpha, p.fac, p.ed);
    reinterpret_cast<float4*>(row)[1] = make_float4(p.dsig, p.c[0], p.c[1], p.c[2]);
  } else {
    row[0] = p.T; row[1] = p.alpha; row[2] = p.fac; row[3] = p.ed;
    row[4] = p.dsig; row[5] = p.c[0]; row[6] = p.c[1]; row[7] = p.c[2];
  }
}

__device__ __forceinline__ Parked park_load(const float* row, bool vec) {
  Parked p;
  if (vec) {
    const float4 u = reinterpret_cast<const float4*>(row)[0], v = reinterpret_cast<const float4*>(row)[1];
    p.T = u.x; p.alpha = u.y; p.fac = u.z; p.ed = u.w;
    p.dsig = v.x; p.c[0] = v.y; p.c[1] = v.z; p.c[2] = v.w;
  } else {
    p.T = row[0]; p.alpha = row[1]; p.fac = row[2]; p.ed = row[3];
    p.dsig = row[4]; p.c[0] = row[5]; p.c[1] = row[6]; p.c[2] = row[7];
  }
  return p;
}

// kColExt: grad_feat rows get dL/dfeat0 in channel 0 and zeros in channels 1 .. feat_stride - 1
// (the colour head's backward fills the channels of its samples afterwards), and
// grad_rgb_sample [M, 3] receives dL/dcolour = w * dL/drgb (zero below the weight threshold).
//
// Two passes per ray (warp per ray, 32-sample chunks): the forward again (the colour before the
// clamp decides which channels pass gradient), then the reverse scan. With rows of >= 8 floats the
// forward pass parks what the reverse pass needs in the gradient row (struct Parked), so the
// reverse pass reads 32 bytes per sample (the next chunk's prefetched) instead of the feature row,
// and recomputes neither the density nor the colours; narrower rows park T alone and recompute.
template <int kCol>
__global__ void __launch_bounds__(kCompWarps * 32, kCompBlocksPerSM) composite_backward_kernel(
    const FFRender r, const float* __restrict__ rays, const float* __restrict__ jitter, int64_t n_rays,
    const int64_t* __restrict__ offsets, const int32_t* __restrict__ sample_idx, const float* __restrict__ feat,
    int feat_stride, const int32_t* __restrict__ white_bg, const float* __restrict__ grad_rgb,
    float* __restrict__ grad_feat, const float* __restrict__ zd, const float* __restrict__ rgb_sample,
    float* __restrict__ grad_rgb_sample) {
  const int lane = threadIdx.x & 31;
  const bool vec = kCol == kColSH && rows_vec(feat, feat_stride) && rows_vec(grad_feat, feat_stride);
  const bool park = kCol == kColSH || feat_stride >= kPark;  // SH rows are >= 28 wide
  const bool pvec = park && rows_vec(grad_feat, feat_stride);
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const RayGeo g = ray_setup(r, rays, jitter, ray);
    float yb[9];
    sh2_basis(g.d, yb);
    const int64_t beg = offsets[ray], end = offsets[ray + 1];
    const bool wb = white_bg ? (*white_bg != 0) : (r.white_bg != 0);
    // pass 1: the forward again; each sample's values are parked in its gradient row. The SH
    // colour's three dot products are taken before the transmittance scan, so the 28-value row
    // is dead during it; the sigmoid follows for the samples above the weight threshold.
    float T = 1.f, acc = 0.f, col[3] = {0.f, 0.f, 0.f};
    for (int64_t c0 = beg; c0 < end; c0 += 32) {
      const int64_t j = c0 + lane;
      const bool active = j < end;
      SampleVals s = {0.f, 0.f, 0.f, 0.f, 0.f, 1.f};
      float lin[3] = {0.f, 0.f, 0.f};
      if (active) {
        float row[kRow];
        if constexpr (kCol == kColSH) {
          load_row(feat + j * feat_stride, vec, row);
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            float v = 0.f;
#pragma unroll
            for (int k = 0; k < 9; ++k) v += yb[k] * row[1 + q * 9 + k];
            lin[q] = v;
          }
        } else {
          row[0] = feat[j * feat_stride];
        }
        s = sample_vals(r, g, zd ? 0 : sample_idx[j], row, zd ? zd + 2 * j : nullptr);
      }
      float excl;
      const float prod = excl_trans(s.fac, lane, excl);
      const float Tj = T * excl;
      const float w = active ? s.alpha * Tj : 0.f;
      acc += w;
      if (active) {
        float c[3] = {0.f, 0.f, 0.f};
        if (w > r.weight_thres) {
          if constexpr (kCol == kColSH) {
            c[0] = sigmoidf(lin[0]); c[1] = sigmoidf(lin[1]); c[2] = sigmoidf(lin[2]);
          } else {
            c[0] = rgb_sample[j * 3]; c[1] = rgb_sample[j * 3 + 1]; c[2] = rgb_sample[j * 3 + 2];
          }
          col[0] += w * c[0]; col[1] += w * c[1]; col[2] += w * c[2];
        }
        if (park) {
          Parked p;
          p.T = Tj; p.alpha = s.alpha; p.fac = s.fac;
          p.ed = expf(-s.sigma * s.delta) * s.delta;
          p.dsig = dsigma_df0(r, s.f0);
          p.c[0] = c[0]; p.c[1] = c[1]; p.c[2] = c[2];
          park_store(grad_feat + j * feat_stride, pvec, p);
        } else {
          grad_feat[j * feat_stride] = Tj;
        }
      }
      T *= prod;
    }
    acc = warp_sum(acc);
    float G[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float v = warp_sum(col[c]);
      if (wb) v = v + (1.f - acc);
      G[c] = (v >= 0.f && v <= 1.f) ? grad_rgb[ray * 3 + c] : 0.f;  // clamp backward
    }
    // pass 2: reverse. E_j = A_j + F_j * E_{j+1} with A = dL/dw * alpha, F = fac; S_j = E_{j+1}.
    float carry = 0.f;
    const int64_t n = end - beg;
    const int64_t k_last = n > 0 ? ((n - 1) / 32) * 32 : -1;
    Parked nxt = {};
    if (park && k_last >= 0 && beg + k_last + lane < end) nxt = park_load(grad_feat + (beg + k_last + lane) * feat_stride, pvec);
    for (int64_t k0 = k_last; k0 >= 0; k0 -= 32) {
      const int64_t j = beg + k0 + lane;
      const bool active = j < end;
      Parked p = {};
      if (park) {
        p = nxt;  // the next (earlier) chunk's values are loaded while this one is scanned
        if (k0 >= 32) nxt = park_load(grad_feat + (j - 32) * feat_stride, pvec);
      } else if (active) {
        // narrow rows: recompute from the feature row and the parked T
        SampleVals s;
        float row[kRow];
        if constexpr (kCol == kColSH)
          load_row(feat + j * feat_stride, vec, row);
        else
          row[0] = feat[j * feat_stride];
        s = sample_vals(r, g, zd ? 0 : sample_idx[j], row, zd ? zd + 2 * j : nullptr);
        p.T = grad_feat[j * feat_stride];
        p.alpha = s.alpha; p.fac = s.fac;
        p.ed = expf(-s.sigma * s.delta) * s.delta;
        p.dsig = dsigma_df0(r, s.f0);
        if (s.alpha * p.T > r.weight_thres) {
          if constexpr (kCol == kColSH) {
            float lin[3];
            sample_rgb(row, yb, p.c, lin);
          } else {
            p.c[0] = rgb_sample[j * 3]; p.c[1] = rgb_sample[j * 3 + 1]; p.c[2] = rgb_sample[j * 3 + 2];
          }
        }
      }
      float w = 0.f, gw = 0.f;
      bool app = false;
      if (active) {
        w = p.alpha * p.T;
        app = w > r.weight_thres;
#pragma unroll
        for (int q = 0; q < 3; ++q) gw += G[q] * (p.c[q] - (wb ? 1.f : 0.f));
      }
      // reverse inclusive affine scan over lanes l..31: (a, f) o (a', f') = (a + f a', f f')
      float a = active ? gw * p.alpha : 0.f, f = active ? p.fac : 1.f;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float a2 = __shfl_down_sync(0xffffffffu, a, o);
        const float f2 = __shfl_down_sync(0xffffffffu, f, o);
        if (lane + o < 32) {
          a = a + f * a2;
          f = f * f2;
        }
      }
      const float e_incl = a + f * carry;                 // E_j
      float s_next = __shfl_down_sync(0xffffffffu, e_incl, 1);  // E_{j+1}
      if (lane == 31) s_next = carry;
      const float new_carry = __shfl_sync(0xffffffffu, e_incl, 0);
      if (active) {
        const float g_alpha = p.T * (gw - s_next);
        const float g_f0 = g_alpha * p.ed * p.dsig;
        if constexpr (kCol == kColSH) {
          float gl[3];
#pragma unroll
          for (int q = 0; q < 3; ++q) gl[q] = app ? G[q] * w * p.c[q] * (1.f - p.c[q]) : 0.f;
          // value m of the row: dL/dfeat0, then dL/dsh[q][k] = gl[q] * yb[k] (m = 1 + 9 q + k)
          auto val = [&](int m) { return m == 0 ? g_f0 : gl[(m - 1) / 9] * yb[(m - 1) % 9]; };
          float* gr = grad_feat + j * feat_stride;
          if (vec) {
#pragma unroll
            for (int q4 = 0; q4 < kRow / 4; ++q4)
              reinterpret_cast<float4*>(gr)[q4] = make_float4(val(4 * q4), val(4 * q4 + 1), val(4 * q4 + 2),
                                                              val(4 * q4 + 3));
          } else {
#pragma unroll
            for (int m = 0; m < kRow; ++m) gr[m] = val(m);
          }
        } else {
          float* gr = grad_feat + j * feat_stride;
          gr[0] = g_f0;
          for (int k = 1; k < feat_stride; ++k) gr[k] = 0.f;
#pragma unroll
          for (int q = 0; q < 3; ++q) grad_rgb_sample[j * 3 + q] = app ? G[q] * w : 0.f;
        }
      }
      carry = new_carry;
    }
  }
}

// The compositing weights alone (the forward's scan without colours): w_out [M] and, per ray,
// the number of samples whose weight passes the threshold (app_mask, :879-881).
__global__ void __launch_bounds__(kRayWarps * 32) composite_weights_kernel(
    const FFRender r, const float* __restrict__ rays, const float* __restrict__ jitter, int64_t n_rays,
    const int64_t* __restrict__ offsets, const int32_t* __restrict__ sample_idx, const float* __restrict__ feat,
    int feat_stride, float* __restrict__ w_out, int32_t* __restrict__ app_counts) {
  const int lane = threadIdx.x & 31;
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const RayGeo g = ray_setup(r, rays, jitter, ray);
    const int64_t beg = offsets[ray], end = offsets[ray + 1];
    float T = 1.f;
    int cnt = 0;
    for (int64_t c0 = beg; c0 < end; c0 += 32) {
      const int64_t j = c0 + lane;
      const bool active = j < end;
      SampleVals s = {0.f, 0.f, 0.f, 0.f, 0.f, 1.f};
      if (active) {
        const float f0 = feat[j * feat_stride];
        s = sample_vals(r, g, sample_idx[j], &f0);
      }
      float excl;
      const float prod = excl_trans(s.fac, lane, excl);
      const float w = active ? s.alpha * (T * excl) : 0.f;
      if (active) w_out[j] = w;
      cnt += __popc(__ballot_sync(0xffffffffu, active && w > r.weight_thres));
      T *= prod;
    }
    if (lane == 0) app_counts[ray] = cnt;
  }
}

// The samples whose weight passes the threshold, in ray-major order (feat[app_mask] of :884):
// app_idx = live-sample index, app_ray = its ray, from the scanned per-ray counts.
__global__ void __launch_bounds__(kRayWarps * 32) app_emit_kernel(int64_t n_rays, const int64_t* __restrict__ offsets,
                                                                 const float* __restrict__ w, float thres,
                                                                 const int64_t* __restrict__ app_offsets,
                                                                 int32_t* __restrict__ app_idx,
                                                                 int32_t* __restrict__ app_ray) {
  const int lane = threadIdx.x & 31;
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t beg = offsets[ray], end = offsets[ray + 1];
    int64_t pos = app_offsets[ray];
    for (int64_t c0 = beg; c0 < end; c0 += 32) {
      const int64_t j = c0 + lane;
      const bool app = j < end && w[j] > thres;
      const uint32_t m = __ballot_sync(0xffffffffu, app);
      if (app) {
        const int64_t k = pos + __popc(m & ((1u << lane) - 1u));
        app_idx[k] = (int32_t)j;
        app_ray[k] = (int32_t)ray;
      }
      pos += __popc(m);
    }
  }
}

int comp_blocks(int64_t n_rays) {
  const int64_t want = ceil_div(n_rays, kCompWarps);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * kCompBlocksPerSM * 4));
}

int ray_blocks(int64_t n_rays) {
  const int64_t want = ceil_div(n_rays, kRayWarps);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 16));
}

}  // namespace

int64_t scan_workspace_bytes(int64_t n) { return (ceil_div(n, kScanBlock) + 1) * (int64_t)sizeof(int64_t); }

// ---- the scan without a caller workspace ------------------------------------------------
// Some callers cannot allocate device memory at all (a host engine that owns every device
// buffer and hands this library only its inputs and outputs, or code that must not touch the
// device allocator). For them the per-block partial
// sums live in this fixed file-scope device array instead of a workspace. Every process that
// loads the library holds these 32 KiB on each GPU it uses until it exits; all calls share
// them, so calls that overlap on the GPU (different streams, no ordering) race on the array.
// Nothing in it needs to start at zero: the first kernel of the scan writes every partial sum
// it later reads.
constexpr int64_t kNoAllocScanBlocks = 4096;
static __device__ __align__(256) int64_t g_scan_scratch[kNoAllocScanBlocks];

int64_t scan_noalloc_max_counts() { return kNoAllocScanBlocks * kScanBlock; }

cudaError_t launch_scan_noalloc(const int32_t* counts, int64_t n, int64_t* offsets, cudaStream_t s) {
  // Host code cannot use g_scan_scratch directly (its name is a host-side stand-in); the
  // device address is looked up once per device, with that device current, on the first call,
  // in the device's primary context, and kept for the life of the process (a cudaDeviceReset
  // does not refresh it).
  static std::mutex mu;
  static void* addr[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  void* p = nullptr;
  {
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
      e = cudaGetSymbolAddress(&addr[dev], g_scan_scratch);
      if (e != cudaSuccess) {
        addr[dev] = nullptr;
        return e;
      }
    }
    p = addr[dev];
  }
  return launch_scan(counts, n, offsets, p, s);
}

cudaError_t launch_march_count(const FFRender& r, const float* rays, const float* jitter, int64_t n, int32_t* counts,
                               float* t_min, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  march_count_kernel<<<ray_blocks(n), kRayWarps * 32, 0, s>>>(r, rays, jitter, n, counts, t_min);
  return cudaGetLastError();
}

cudaError_t launch_scan(const int32_t* counts, int64_t n, int64_t* offsets, void* workspace, cudaStream_t s) {
  if (n == 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), s);
  const int64_t nb = ceil_div(n, kScanBlock);
  int64_t* sums = static_cast<int64_t*>(workspace);
  scan_blocks_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, n, sums);
  scan_sums_kernel<<<1, kScanThreads, 0, s>>>(sums, nb);
  scan_apply_kernel<<<(unsigned)nb, kScanThreads, 0, s>>>(counts, n, sums, offsets);
  return cudaGetLastError();
}

cudaError_t launch_filter_rays(const FFRender& r, const float* rays, int64_t n, int n_samples, int bbox_only,
                               uint8_t* keep, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  filter_rays_kernel<<<ray_blocks(n), kRayWarps * 32, 0, s>>>(r, rays, n, n_samples, bbox_only, keep);
  return cudaGetLastError();
}

cudaError_t launch_march_emit(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                              const int64_t* offsets, float* xyz, int32_t* sample_idx, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  march_emit_kernel<<<ray_blocks(n), kRayWarps * 32, 0, s>>>(r, rays, jitter, n, offsets, xyz, sample_idx);
  return cudaGetLastError();
}

cudaError_t launch_composite_forward(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                     const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                     int feat_stride, const int32_t* white_bg, float* rgb, float* depth, float* acc,
                                     const float* zd, float* w_out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  composite_forward_kernel<kColSH><<<comp_blocks(n), kCompWarps * 32, 0, s>>>(
      r, rays, jitter, n, offsets, sample_idx, feat, feat_stride, white_bg, rgb, depth, acc, zd, w_out, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_composite_forward_rgb(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                         const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                         int feat_stride, const float* rgb_sample, const int32_t* white_bg, float* rgb,
                                         float* depth, float* acc, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  composite_forward_kernel<kColExt><<<comp_blocks(n), kCompWarps * 32, 0, s>>>(
      r, rays, jitter, n, offsets, sample_idx, feat, feat_stride, white_bg, rgb, depth, acc, nullptr, nullptr,
      rgb_sample);
  return cudaGetLastError();
}

cudaError_t launch_composite_weights(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                     const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                     int feat_stride, float* w_out, int32_t* app_counts, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  composite_weights_kernel<<<ray_blocks(n), kRayWarps * 32, 0, s>>>(r, rays, jitter, n, offsets, sample_idx, feat,
                                                                     feat_stride, w_out, app_counts);
  return cudaGetLastError();
}

cudaError_t launch_app_emit(int64_t n, const int64_t* offsets, const float* w, float thres, const int64_t* app_offsets,
                            int32_t* app_idx, int32_t* app_ray, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  app_emit_kernel<<<ray_blocks(n), kRayWarps * 32, 0, s>>>(n, offsets, w, thres, app_offsets, app_idx, app_ray);
  return cudaGetLastError();
}

cudaError_t launch_composite_backward(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                      const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                      int feat_stride, const int32_t* white_bg, const float* grad_rgb,
                                      float* grad_feat, const float* zd, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  composite_backward_kernel<kColSH><<<comp_blocks(n), kCompWarps * 32, 0, s>>>(
      r, rays, jitter, n, offsets, sample_idx, feat, feat_stride, white_bg, grad_rgb, grad_feat, zd, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_composite_backward_rgb(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                          const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                          int feat_stride, const float* rgb_sample, const int32_t* white_bg,
                                          const float* grad_rgb, float* grad_feat, float* grad_rgb_sample,
                                          cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  composite_backward_kernel<kColExt><<<comp_blocks(n), kCompWarps * 32, 0, s>>>(
      r, rays, jitter, n, offsets, sample_idx, feat, feat_stride, white_bg, grad_rgb, grad_feat, nullptr, rgb_sample,
      grad_rgb_sample);
  return cudaGetLastError();
}

}  // namespace ffgb
