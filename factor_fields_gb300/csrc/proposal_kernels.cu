// Learned proposal sampler: a coarse density grid + small MLP that predicts, per ray, where the
// field's compositing weight is, and inverse-CDF resampling of a few samples per ray.
//
// The reference has no proposal network; its resampling semantics are those of sample_pdf
// (dataLoader/ray_utils.py:132-174): pdf = (w + 1e-5) / sum, cdf with a leading 0,
// searchsorted(cdf, u, right=True), linear interpolation inside the bin (denominator < 1e-5
// replaced by 1). The proposal loss restates the published Mip-NeRF 360 idea: the proposal's
// weight on each coarse bin should upper-bound the field's weight mass in that bin,
//     L = sum_k max(0, m_k - w_k)^2 / (w_k + eps),
// with gradients reaching only the proposal (the field's weights are inputs).
//
// Per ray: n_bins coarse bins of equal length over the ray's segment inside the aabb
// [t_in, t_out] (t_in clamped to >= 0.05 like sample_point, models/FactorFields.py:591), the
// proposal density sigma = softplus(o + shift) at the bin centres, alpha = 1 - exp(-sigma *
// bin_len * distance_scale), weights by an exclusive transmittance scan (raw2alpha :82-88).
//
// Kernels: encode (bin-centre positions + trilinear gather of the C-channel grid, thread per
// coarse sample), resample (warp per ray: weights, cdf, n_fine samples), loss (warp per ray:
// bin masses, loss, reverse scan to dL/do), scatter (thread per coarse sample).
#include "ff_common.cuh"
#include "ff_internal.h"
#include "mma_util.cuh"

namespace ffgb {

namespace {

constexpr float kPropEps = 1e-5f;  // loss denominator guard

struct Segment {
  float o[3], d[3], t_in, t_out, len;
};

__device__ __forceinline__ Segment segment(const FFProposal& p, const float* rays, int64_t ray) {
  Segment s;
  float tin = -INFINITY, tout = INFINITY;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s.o[k] = rays[ray * 6 + k];
    s.d[k] = rays[ray * 6 + 3 + k];
    const float vec = (s.d[k] == 0.f) ? 1e-6f : s.d[k];
    const float ra = (p.aabb_max[k] - s.o[k]) / vec, rb = (p.aabb_min[k] - s.o[k]) / vec;
    tin = fmaxf(tin, fminf(ra, rb));
    tout = fminf(tout, fmaxf(ra, rb));
  }
  s.t_in = fmaxf(tin, 0.05f);
  s.t_out = fmaxf(tout, s.t_in);
  s.len = (s.t_out - s.t_in) / (float)p.n_bins;
  return s;
}

// segment() for a warp whose 32 lanes share `ray` (all lanes call it): lane k < 3 computes axis
// k's two slab distances, the others read them by shuffles. The same float32 operations as
// segment() (min / max are exact), so the same Segment, with two divisions per warp instead of six.
__device__ __forceinline__ Segment segment_warp(const FFProposal& p, const float* rays, int64_t ray, int lane) {
  const int k = lane < 3 ? lane : 0;
  const float o = rays[ray * 6 + k], d = rays[ray * 6 + 3 + k];
  const float amax = k == 0 ? p.aabb_max[0] : (k == 1 ? p.aabb_max[1] : p.aabb_max[2]);
  const float amin = k == 0 ? p.aabb_min[0] : (k == 1 ? p.aabb_min[1] : p.aabb_min[2]);
  const float vec = (d == 0.f) ? 1e-6f : d;
  const float ra = (amax - o) / vec, rb = (amin - o) / vec;
  const float lo = fminf(ra, rb), hi = fmaxf(ra, rb);
  Segment s;
  float tin = -INFINITY, tout = INFINITY;
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    s.o[q] = __shfl_sync(0xffffffffu, o, q);
    s.d[q] = __shfl_sync(0xffffffffu, d, q);
    tin = fmaxf(tin, __shfl_sync(0xffffffffu, lo, q));
    tout = fminf(tout, __shfl_sync(0xffffffffu, hi, q));
  }
  s.t_in = fmaxf(tin, 0.05f);
  s.t_out = fmaxf(tout, s.t_in);
  s.len = (s.t_out - s.t_in) / (float)p.n_bins;
  return s;
}

// Coarse sample e = ray * nb + bin (shifts when nb is a power of two).
__device__ __forceinline__ void ray_bin(int64_t e, int nb, int64_t& ray, int& bin) {
  if ((nb & (nb - 1)) == 0) {
    const int sh = __ffs(nb) - 1;
    ray = e >> sh;
    bin = (int)(e & (nb - 1));
  } else {
    ray = e / nb;
    bin = (int)(e - ray * nb);
  }
}

// Trilinear corners of x in the proposal grid (align_corners over the aabb, zero padding).
__device__ __forceinline__ void grid_corners(const FFProposal& p, const float* x, Corners<3>& c) {
  float ix[3];
  int sz[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    sz[k] = p.reso;
    ix[k] = (x[k] - p.aabb_min[k]) * p.inv_cell[k];
  }
  linear_corners<3>(ix, sz, c);
}

template <typename T>
__device__ __forceinline__ void load8(const T* g, float* v);

template <>
__device__ __forceinline__ void load8<__nv_bfloat16>(const __nv_bfloat16* g, float* v) {
  const uint4 t = __ldg(reinterpret_cast<const uint4*>(g));
  const uint32_t w[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    v[2 * j] = __uint_as_float(w[j] << 16);
    v[2 * j + 1] = __uint_as_float(w[j] & 0xffff0000u);
  }
}

template <>
__device__ __forceinline__ void load8<float>(const float* g, float* v) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(g));
  const float4 b = __ldg(reinterpret_cast<const float4*>(g) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

template <typename T>
__global__ void __launch_bounds__(256) proposal_encode_kernel(const FFProposal p, const T* __restrict__ grid,
                                                              const float* __restrict__ rays, int64_t n_rays,
                                                              float* __restrict__ feat) {
  const int64_t total = n_rays * p.n_bins;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ray = e / p.n_bins;
    const int k = (int)(e % p.n_bins);
    const Segment s = segment(p, rays, ray);
    const float t = s.t_in + ((float)k + 0.5f) * s.len;
    float x[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) x[q] = s.o[q] + s.d[q] * t;
    Corners<3> c;
    grid_corners(p, x, c);
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      if (c.idx[b] >= 0 && c.w[b] != 0.f) {
        float v[8];
        load8<T>(grid + (int64_t)c.idx[b] * 8, v);
#pragma unroll
        for (int q = 0; q < 8; ++q) acc[q] += v[q] * c.w[b];
      }
    }
    float4* out = reinterpret_cast<float4*>(feat + e * 8);
    out[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    out[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
  }
}

__global__ void __launch_bounds__(256) proposal_scatter_kernel(const FFProposal p, const float* __restrict__ rays,
                                                               int64_t n_rays, const float* __restrict__ grad_feat,
                                                               float* __restrict__ grad_grid) {
  const int64_t total = n_rays * p.n_bins;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ray = e / p.n_bins;
    const int k = (int)(e % p.n_bins);
    const Segment s = segment(p, rays, ray);
    const float t = s.t_in + ((float)k + 0.5f) * s.len;
    float x[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) x[q] = s.o[q] + s.d[q] * t;
    Corners<3> c;
    grid_corners(p, x, c);
    const float4 g0 = reinterpret_cast<const float4*>(grad_feat + e * 8)[0];
    const float4 g1 = reinterpret_cast<const float4*>(grad_feat + e * 8)[1];
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      if (c.idx[b] >= 0 && c.w[b] != 0.f) {
        const float w = c.w[b];
        float4* dst = reinterpret_cast<float4*>(grad_grid + (int64_t)c.idx[b] * 8);
        atomicAdd(dst, make_float4(g0.x * w, g0.y * w, g0.z * w, g0.w * w));
        atomicAdd(dst + 1, make_float4(g1.x * w, g1.y * w, g1.z * w, g1.w * w));
      }
    }
  }
}

constexpr int kMaxBinsPerLane = 4;  // n_bins <= 128
constexpr int kMaxFine = 128;

// Proposal densities, alphas, exclusive transmittances and weights of this lane's bins
// (bins lane*B .. lane*B + B - 1). Returns the warp's total weight.
struct BinState {
  float o[kMaxBinsPerLane], sigma[kMaxBinsPerLane], alpha[kMaxBinsPerLane], fac[kMaxBinsPerLane],
      T[kMaxBinsPerLane], w[kMaxBinsPerLane];
};

__device__ __forceinline__ void bin_weights(const FFProposal& p, const float* o_row, float len, int lane, int B,
                                            BinState& st) {
  const float delta = len * p.distance_scale;
  float prod = 1.f;
#pragma unroll
  for (int b = 0; b < kMaxBinsPerLane; ++b) {
    if (b < B) {
      const float o = o_row ? o_row[lane * B + b] : -60.f;  // NULL: a flat histogram
      const float x = o + p.density_shift;
      st.o[b] = o;
      st.sigma[b] = (x > 20.f) ? x : log1pf(expf(x));
      st.alpha[b] = 1.f - expf(-st.sigma[b] * delta);
      st.fac[b] = 1.f - st.alpha[b] + 1e-10f;
      st.T[b] = prod;  // lane-local exclusive prefix, completed below
      prod *= st.fac[b];
    }
  }
  // exclusive product scan of the lane products across the warp
  float incl = prod;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const float v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl *= v;
  }
  float excl = __shfl_up_sync(0xffffffffu, incl, 1);
  if (lane == 0) excl = 1.f;
#pragma unroll
  for (int b = 0; b < kMaxBinsPerLane; ++b) {
    if (b < B) {
      st.T[b] *= excl;
      st.w[b] = st.alpha[b] * st.T[b];
    }
  }
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Position of the sample at distance t along the segment's ray (one rounding per coordinate, the
// same in every resampling mode so that the occupied rows equal the unculled ones bit for bit).
__device__ __forceinline__ void sample_pos(const Segment& s, float t, float* x) {
#pragma unroll
  for (int q = 0; q < 3; ++q) x[q] = fmaf(s.d[q], t, s.o[q]);
}

// Resampling modes: every sample with its bin and the proposal weights (training and the
// unculled render), or, for rendering through an occupancy volume, the occupied samples alone:
// a counting pass (counts[ray]) and, after the scan of the counts, an emitting pass that writes
// each ray's occupied samples in sample order from offsets[ray].
enum { kResampleAll = 0, kResampleCount = 1, kResampleEmit = 2 };

template <int MODE>
__global__ void __launch_bounds__(256) proposal_resample_kernel(
    const FFProposal p, const FFRender occ, const float* __restrict__ rays, int64_t n_rays,
    const float* __restrict__ o_prop, const float* __restrict__ jitter, const float* __restrict__ u_given,
    float* __restrict__ w_prop, float* __restrict__ xyz, float* __restrict__ zd, int32_t* __restrict__ bin_of,
    int32_t* __restrict__ counts, const int64_t* __restrict__ offsets) {
  __shared__ float cdf_s[8][kMaxBinsPerLane * 32 + 1];
  __shared__ float t_s[8][kMaxFine];
  __shared__ float e_s[8][kMaxFine + 1];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nb = p.n_bins, nf = p.n_fine, B = nb / 32;
  float* cdf = cdf_s[wib];
  float* ts = t_s[wib];
  float* es = e_s[wib];
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const Segment s = segment_warp(p, rays, ray, lane);
    BinState st;
    bin_weights(p, o_prop ? o_prop + ray * nb : nullptr, s.len, lane, B, st);
    // pdf = (w + 1e-5) / sum, cdf with a leading zero (sample_pdf, ray_utils.py:135-138)
    float lsum = 0.f;
#pragma unroll
    for (int b = 0; b < kMaxBinsPerLane; ++b)
      if (b < B) {
        if (MODE == kResampleAll && w_prop) w_prop[ray * nb + lane * B + b] = st.w[b];
        lsum += st.w[b] + 1e-5f;
      }
    const float tot = warp_sum_f(lsum);
    float incl = lsum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const float v = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += v;
    }
    const float keep = 1.f - p.uniform_mix, flat = p.uniform_mix / (float)nb;
    float run = keep * (incl - lsum) / tot + flat * (float)(lane * B);
#pragma unroll
    for (int b = 0; b < kMaxBinsPerLane; ++b)
      if (b < B) {
        run += keep * (st.w[b] + 1e-5f) / tot + flat;
        cdf[lane * B + b + 1] = run;
      }
    if (lane == 0) cdf[0] = 0.f;
    __syncwarp();
    // inverse CDF: searchsorted(cdf, u, right=True) and linear interpolation inside the bin
    auto inv_cdf = [&](float u, int& bin) {
      int lo = 0, hi = nb + 1;  // first index with cdf > u
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid] > u) hi = mid; else lo = mid + 1;
      }
      const int below = max(0, lo - 1), above = min(nb, lo);
      const float cb = cdf[below], ca = cdf[above];
      float denom = ca - cb;
      if (denom < 1e-5f) denom = 1.f;
      const float tt = (u - cb) / denom;
      const float eb = s.t_in + (float)below * s.len, ea = s.t_in + (float)above * s.len;
      bin = min(below, nb - 1);
      return eb + tt * (ea - eb);
    };
    for (int i = lane; i < nf; i += 32) {
      float u;
      if (u_given)
        u = u_given[ray * nf + i];
      else
        u = ((float)i + (jitter ? jitter[ray] : 0.5f)) / (float)nf;
      int bin;
      const float t = inv_cdf(u, bin);
      ts[i] = t;
      if constexpr (MODE == kResampleAll) {
        if (bin_of) bin_of[ray * nf + i] = bin;
        float x[3];
        sample_pos(s, t, x);
#pragma unroll
        for (int q = 0; q < 3; ++q) xyz[(ray * nf + i) * 3 + q] = x[q];
      }
    }
    // Stratified samples (u = (i + jitter) / n_fine, or given u with p.u_stratified): sample i
    // stands for its CDF stratum [F^-1(i / n), F^-1((i + 1) / n)]; the strata tile
    // [t_in, t_out]. Other given u: the distance to the next sample (the last one to t_out).
    const bool strata = !u_given || p.u_stratified;
    if (strata && MODE != kResampleCount) {  // the counting pass needs positions only
      for (int i = lane; i <= nf; i += 32) {
        int bin;
        es[i] = i == 0 ? s.t_in : (i == nf ? s.t_out : inv_cdf((float)i / (float)nf, bin));
      }
    }
    __syncwarp();
    if constexpr (MODE == kResampleAll) {
      for (int i = lane; i < nf; i += 32) {
        const float t = ts[i];
        float d;
        if (!strata) {
          const float nxt = (i + 1 < nf) ? ts[i + 1] : s.t_out;
          d = nxt - t;
        } else {
          d = es[i + 1] - es[i];
        }
        zd[(ray * nf + i) * 2 + 0] = t;
        zd[(ray * nf + i) * 2 + 1] = fmaxf(d, 0.f);
      }
    } else {
      // occupied samples only (AlphaGridMask's test, models/FactorFields.py:865-867): the others
      // would have zero density, alpha 0 and weight 0, and leave the transmittance unchanged
      int64_t pos = (MODE == kResampleEmit) ? offsets[ray] : 0;
      int cnt = 0;
      for (int i0 = 0; i0 < nf; i0 += 32) {
        const int i = i0 + lane;
        float x[3] = {0.f, 0.f, 0.f}, t = 0.f, d = 0.f;
        bool live = false;
        if (i < nf) {
          t = ts[i];
          if constexpr (MODE == kResampleEmit) {
            if (!strata) {
              const float nxt = (i + 1 < nf) ? ts[i + 1] : s.t_out;
              d = nxt - t;
            } else {
              d = es[i + 1] - es[i];
            }
          }
          sample_pos(s, t, x);
          live = occupied(occ, x);
        }
        const uint32_t m = __ballot_sync(0xffffffffu, live);
        if constexpr (MODE == kResampleEmit) {
          if (live) {
            const int64_t j = pos + __popc(m & ((1u << lane) - 1u));
#pragma unroll
            for (int q = 0; q < 3; ++q) xyz[j * 3 + q] = x[q];
            zd[j * 2 + 0] = t;
            zd[j * 2 + 1] = fmaxf(d, 0.f);
          }
          pos += __popc(m);
        } else {
          cnt += __popc(m);
        }
      }
      if constexpr (MODE == kResampleCount) {
        if (lane == 0) counts[ray] = cnt;
      }
    }
    __syncwarp();
  }
}

__global__ void __launch_bounds__(256) proposal_loss_kernel(const FFProposal p, const float* __restrict__ rays,
                                                            int64_t n_rays, const float* __restrict__ o_prop,
                                                            const float* __restrict__ w_field,
                                                            const int32_t* __restrict__ bin_of, float loss_scale,
                                                            float* __restrict__ loss_sum,
                                                            float* __restrict__ grad_o) {
  __shared__ float mass_s[8][kMaxBinsPerLane * 32];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nb = p.n_bins, nf = p.n_fine, B = nb / 32;
  float* mass = mass_s[wib];
  float loss_acc = 0.f;
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const Segment s = segment(p, rays, ray);
    BinState st;
    bin_weights(p, o_prop + ray * nb, s.len, lane, B, st);
    for (int k = lane; k < nb; k += 32) mass[k] = 0.f;
    __syncwarp();
    for (int i = lane; i < nf; i += 32) {
      const int b = bin_of[ray * nf + i];
      if (b >= 0 && b < nb) atomicAdd(&mass[b], w_field[ray * nf + i]);  // bins outside the histogram add nothing
    }
    __syncwarp();
    // loss and dL/dw per bin
    float gw[kMaxBinsPerLane];
#pragma unroll
    for (int b = 0; b < kMaxBinsPerLane; ++b) {
      gw[b] = 0.f;
      if (b < B) {
        const float m = mass[lane * B + b], w = st.w[b];
        const float r = fmaxf(m - w, 0.f), den = w + kPropEps;
        loss_acc += r * r / den;
        gw[b] = loss_scale * (-2.f * r / den - r * r / (den * den));
      }
    }
    // reverse recurrence E_k = A_k + F_k E_{k+1} (A = dL/dw * alpha, F = fac), S_k = E_{k+1}:
    // lane-local composition of its bins, then a reverse affine scan across lanes
    float a = 0.f, f = 1.f;
#pragma unroll
    for (int b = kMaxBinsPerLane - 1; b >= 0; --b)
      if (b < B) {
        a = gw[b] * st.alpha[b] + st.fac[b] * a;
        f = st.fac[b] * f;
      }
    float ea = a, ef = f;  // composition of lanes l..31
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const float a2 = __shfl_down_sync(0xffffffffu, ea, off);
      const float f2 = __shfl_down_sync(0xffffffffu, ef, off);
      if (lane + off < 32) {
        ea = ea + ef * a2;
        ef = ef * f2;
      }
    }
    float e_next = __shfl_down_sync(0xffffffffu, ea, 1);  // E at the start of lane l+1
    if (lane == 31) e_next = 0.f;
    const float delta = s.len * p.distance_scale;
#pragma unroll
    for (int b = kMaxBinsPerLane - 1; b >= 0; --b) {
      if (b < B) {
        const float g_alpha = st.T[b] * (gw[b] - e_next);
        const float g_sigma = g_alpha * expf(-st.sigma[b] * delta) * delta;
        const float x = st.o[b] + p.density_shift;
        const float g_o = (x > 20.f) ? g_sigma : g_sigma / (1.f + expf(-x));
        grad_o[ray * nb + lane * B + b] = g_o;
        e_next = gw[b] * st.alpha[b] + st.fac[b] * e_next;
      }
    }
    __syncwarp();
  }
  loss_acc = warp_sum_f(loss_acc);
  if (lane == 0 && loss_sum) atomicAdd(loss_sum, loss_acc * loss_scale);
}

int grid_blocks(int64_t total, int threads) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, threads), (int64_t)sm_count() * 16));
}

// ---- the proposal head on tensor cores: encode + 8 -> 64 (ReLU) -> 1 ---------------------
// Thread per coarse sample for the position and the 8-channel gather; 32 samples per warp for
// the MLP (mma.sync m16n8k16 BF16, FP32 accumulation). Layer 0 runs in split BF16 (features and
// W0 as hi + lo pairs, the lo * lo term dropped) so that the ReLU mask is the float32 one;
// dX = dH W0 takes dH as hi + lo and W0 as BF16.
// Backward: dH = g_o * w1 * [H > 0], dX = dH W0 (tensor cores), dW1 in registers, dW0 and the
// bias gradient (constant-1 feature column) by a block-wide MMA over the block's 128 samples,
// the grid gradient scattered with float4 atomics.
// MODE 0: the forward of training (the proposal loss and its backward read these outputs);
// MODE 1: the backward; MODE 2: the forward of rendering, one BF16 MMA pass per layer (features
// and hidden activations rounded to BF16, ReLU fused into the rounding) with the 64 -> 1 output
// layer on the tensor cores as well: a histogram to sample from needs no more precision.
// n_bins is a multiple of 32 and tiles are 32-aligned, so each warp's 32 samples lie on one ray.
constexpr int kHW = 4;            // warps per block
constexpr int kHT = kHW * 32;     // samples per block iteration
constexpr int HLD_X = 12;         // float32 feature tile [32][12]: 8 features, 1.0, 0, 0, 0
constexpr int HLD_H = 72;         // BF16 dH tile [32][72]
constexpr int HLD_W0 = 24;        // W0 [64][16 + pad] BF16 (inputs 8..15 zero)
constexpr int HLD_W0T = 72;       // W0^T [8][64 + pad]

struct HeadSmem {
  __nv_bfloat16 *w0, *w0l, *w0t;
  float *b0, *w1, *x;
  __nv_bfloat16* dh;
};

template <int MODE>
__host__ __device__ constexpr int64_t head_smem_bytes() {
  return 2 * 64 * HLD_W0 * 2 + 8 * HLD_W0T * 2 + 64 * 4 + 64 * 4 + (int64_t)kHW * 32 * HLD_X * 4 +
         (MODE == 1 ? (int64_t)kHW * 32 * HLD_H * 2 : 0);
}

// Two float32 values as a BF16 pair after a ReLU, in one conversion (the first value in the low
// half, as pack_bf16).
__device__ __forceinline__ uint32_t pack_bf16_relu(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

// A fragment (rows r, r + 8; columns c, c + 1 and c + 8, c + 9) of the float32 feature tile,
// rounded to BF16; columns at or past HLD_X read as zero.
__device__ __forceinline__ void head_frag_bf16(const float* xf, int r0, int c, uint32_t* a) {
  const float2 v00 = *reinterpret_cast<const float2*>(xf + r0 * HLD_X + c);
  const float2 v10 = *reinterpret_cast<const float2*>(xf + (r0 + 8) * HLD_X + c);
  a[0] = pack_bf16(v00.x, v00.y);
  a[1] = pack_bf16(v10.x, v10.y);
  if (c + 8 < HLD_X) {
    const float2 v01 = *reinterpret_cast<const float2*>(xf + r0 * HLD_X + c + 8);
    const float2 v11 = *reinterpret_cast<const float2*>(xf + (r0 + 8) * HLD_X + c + 8);
    a[2] = pack_bf16(v01.x, v01.y);
    a[3] = pack_bf16(v11.x, v11.y);
  } else {
    a[2] = a[3] = 0u;
  }
}

__device__ __forceinline__ void head_pair(const float* xf, int row, int col, uint32_t& hi, uint32_t& lo) {
  if (col < HLD_X) {
    const float2 v = *reinterpret_cast<const float2*>(xf + row * HLD_X + col);
    split_pair(v.x, v.y, hi, lo);
  } else {
    hi = lo = 0u;
  }
}

template <int MODE, typename T>
__global__ void __launch_bounds__(kHT) proposal_head_kernel(const FFProposal p, const T* __restrict__ grid,
                                                             const float* __restrict__ rays, int64_t n_rays,
                                                             const FFMlp m, float* __restrict__ o_out,
                                                             const float* __restrict__ g_o,
                                                             float* __restrict__ grad_grid, const FFMlpGrad gr) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  HeadSmem s;
  {
    unsigned char* q = smem_raw;
    s.w0 = (__nv_bfloat16*)q; q += 64 * HLD_W0 * 2;
    s.w0l = (__nv_bfloat16*)q; q += 64 * HLD_W0 * 2;
    s.w0t = (__nv_bfloat16*)q; q += 8 * HLD_W0T * 2;
    s.b0 = (float*)q; q += 64 * 4;
    s.w1 = (float*)q; q += 64 * 4;
    s.x = (float*)q; q += kHW * 32 * HLD_X * 4;
    s.dh = MODE == 1 ? (__nv_bfloat16*)q : nullptr;
  }
  for (int e = tid; e < 64 * 16; e += kHT) {
    const int j = e >> 4, k = e & 15;
    const float w = k < 8 ? m.weight[0][j * 8 + k] : 0.f;
    const __nv_bfloat16 v = __float2bfloat16_rn(w);
    s.w0[j * HLD_W0 + k] = v;
    s.w0l[j * HLD_W0 + k] = __float2bfloat16_rn(w - __bfloat162float(v));
    if (k < 8) s.w0t[k * HLD_W0T + j] = v;
  }
  for (int j = tid; j < 64; j += kHT) {
    s.b0[j] = m.bias[0] ? m.bias[0][j] : 0.f;
    s.w1[j] = m.weight[1][j];
  }
  __syncthreads();
  // MODE 2: W1 as the B fragments of the output layer (n-tile column 0 = the single output;
  // lanes of the other columns hold zeros), k-steps of 16 hidden units
  uint32_t w1b[MODE == 2 ? 4 : 1][2];
  if constexpr (MODE == 2) {
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int k0 = 16 * ks + 2 * t;
      w1b[ks][0] = g == 0 ? pack_bf16(s.w1[k0], s.w1[k0 + 1]) : 0u;
      w1b[ks][1] = g == 0 ? pack_bf16(s.w1[k0 + 8], s.w1[k0 + 9]) : 0u;
    }
  }
  float* xf = s.x + warp * 32 * HLD_X;
  const int64_t total = n_rays * p.n_bins;
  float acc_w0[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
  float acc_w1[8][2];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) acc_w1[nt][0] = acc_w1[nt][1] = 0.f;

  for (int64_t base = (int64_t)blockIdx.x * kHT; base < total; base += (int64_t)gridDim.x * kHT) {
    const int64_t e = base + warp * 32 + lane;
    // total is a multiple of 32, so a warp's samples are all valid or all past the end
    const bool valid = base + warp * 32 < total;
    float pos[3] = {0.f, 0.f, 0.f};
    float feat[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (valid) {
      int64_t ray;
      int k;
      Segment sg;
      if constexpr (MODE == 2) {  // the same values with fewer instructions (more registers)
        ray_bin(e, p.n_bins, ray, k);
        sg = segment_warp(p, rays, ray, lane);
      } else {
        ray = e / p.n_bins;
        k = (int)(e % p.n_bins);
        sg = segment(p, rays, ray);
      }
      const float tt = sg.t_in + ((float)k + 0.5f) * sg.len;
#pragma unroll
      for (int q = 0; q < 3; ++q) pos[q] = sg.o[q] + sg.d[q] * tt;
      Corners<3> c;
      grid_corners(p, pos, c);
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        if (c.idx[b] >= 0 && c.w[b] != 0.f) {
          float v[8];
          load8<T>(grid + (int64_t)c.idx[b] * 8, v);
#pragma unroll
          for (int q = 0; q < 8; ++q) feat[q] += v[q] * c.w[b];
        }
      }
    }
    {
      float4* xr = reinterpret_cast<float4*>(xf + lane * HLD_X);
      xr[0] = make_float4(feat[0], feat[1], feat[2], feat[3]);
      xr[1] = make_float4(feat[4], feat[5], feat[6], feat[7]);
      xr[2] = make_float4(valid ? 1.f : 0.f, 0.f, 0.f, 0.f);
    }
    __syncwarp();
    if constexpr (MODE == 2) {
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int r0 = 16 * mt + g;
        uint32_t a[4];
        head_frag_bf16(xf, r0, 2 * t, a);
        float oc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {  // hidden units [16 ks, 16 ks + 16): two n-tiles of layer 0
          float hc[2][4];
          uint32_t ha[4];
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            const int nt = 2 * ks + hh;
            const float bl = s.b0[nt * 8 + 2 * t], bh = s.b0[nt * 8 + 2 * t + 1];
            hc[hh][0] = bl; hc[hh][1] = bh; hc[hh][2] = bl; hc[hh][3] = bh;
            const __nv_bfloat16* wp = s.w0 + (nt * 8 + g) * HLD_W0 + 2 * t;
            mma_bf16(hc[hh], a, lds32(wp), lds32(wp + 8));
          }
          ha[0] = pack_bf16_relu(hc[0][0], hc[0][1]);
          ha[1] = pack_bf16_relu(hc[0][2], hc[0][3]);
          ha[2] = pack_bf16_relu(hc[1][0], hc[1][1]);
          ha[3] = pack_bf16_relu(hc[1][2], hc[1][3]);
          mma_bf16(oc, ha, w1b[ks][0], w1b[ks][1]);
        }
        // output column 0: rows r0 (oc[0]) and r0 + 8 (oc[2]) in the t == 0 lanes
        const int64_t row0 = base + warp * 32 + r0;
        if (t == 0 && valid) {
          o_out[row0] = oc[0];
          o_out[row0 + 8] = oc[2];
        }
      }
      __syncwarp();
      continue;
    }
    float dx[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int r0 = 16 * mt + g, r1 = r0 + 8;
      float hc[8][4];
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const float bl = s.b0[nt * 8 + 2 * t], bh = s.b0[nt * 8 + 2 * t + 1];
        hc[nt][0] = bl; hc[nt][1] = bh; hc[nt][2] = bl; hc[nt][3] = bh;
      }
      {
        uint32_t ah[4], al[4];
        head_pair(xf, r0, 2 * t, ah[0], al[0]);
        head_pair(xf, r1, 2 * t, ah[1], al[1]);
        head_pair(xf, r0, 2 * t + 8, ah[2], al[2]);
        head_pair(xf, r1, 2 * t + 8, ah[3], al[3]);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const __nv_bfloat16* wp = s.w0 + (nt * 8 + g) * HLD_W0 + 2 * t;
          const __nv_bfloat16* wl = s.w0l + (nt * 8 + g) * HLD_W0 + 2 * t;
          const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
          mma_bf16(hc[nt], ah, lds32(wl), lds32(wl + 8));
          mma_bf16(hc[nt], al, b0, b1);
          mma_bf16(hc[nt], ah, b0, b1);
        }
      }
      // o = relu(H) . w1 (rows r0 / r1): lane partial sums, then the quad
      float o0 = 0.f, o1 = 0.f;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
        for (int q = 0; q < 4; ++q) hc[nt][q] = fmaxf(hc[nt][q], 0.f);
        const float wa = s.w1[nt * 8 + 2 * t], wb = s.w1[nt * 8 + 2 * t + 1];
        o0 += hc[nt][0] * wa + hc[nt][1] * wb;
        o1 += hc[nt][2] * wa + hc[nt][3] * wb;
      }
      o0 += __shfl_xor_sync(0xffffffffu, o0, 1);
      o0 += __shfl_xor_sync(0xffffffffu, o0, 2);
      o1 += __shfl_xor_sync(0xffffffffu, o1, 1);
      o1 += __shfl_xor_sync(0xffffffffu, o1, 2);
      const int64_t row0 = base + warp * 32 + r0, row1 = row0 + 8;
      if constexpr (MODE == 0) {
        if (t == 0) {
          if (row0 < total) o_out[row0] = o0;
          if (row1 < total) o_out[row1] = o1;
        }
      } else {
        const float go0 = row0 < total ? g_o[row0] : 0.f;
        const float go1 = row1 < total ? g_o[row1] : 0.f;
        __nv_bfloat16* dhw = s.dh + warp * 32 * HLD_H;
#pragma unroll
        for (int q = 0; q < 4; ++q) dx[mt][q] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          float dh[2][4];
#pragma unroll
          for (int hh = 0; hh < 2; ++hh) {
            const int nt = 2 * ks + hh;
            const float wa = s.w1[nt * 8 + 2 * t], wb = s.w1[nt * 8 + 2 * t + 1];
            acc_w1[nt][0] += hc[nt][0] * go0 + hc[nt][2] * go1;
            acc_w1[nt][1] += hc[nt][1] * go0 + hc[nt][3] * go1;
            dh[hh][0] = hc[nt][0] > 0.f ? go0 * wa : 0.f;
            dh[hh][1] = hc[nt][1] > 0.f ? go0 * wb : 0.f;
            dh[hh][2] = hc[nt][2] > 0.f ? go1 * wa : 0.f;
            dh[hh][3] = hc[nt][3] > 0.f ? go1 * wb : 0.f;
          }
          uint32_t d[4], dl[4];
          split_pair(dh[0][0], dh[0][1], d[0], dl[0]);
          split_pair(dh[0][2], dh[0][3], d[1], dl[1]);
          split_pair(dh[1][0], dh[1][1], d[2], dl[2]);
          split_pair(dh[1][2], dh[1][3], d[3], dl[3]);
          __nv_bfloat16* p0 = dhw + r0 * HLD_H + 16 * ks + 2 * t;
          __nv_bfloat16* p1 = dhw + r1 * HLD_H + 16 * ks + 2 * t;
          sts32(p0, d[0]); sts32(p1, d[1]); sts32(p0 + 8, d[2]); sts32(p1 + 8, d[3]);
          const __nv_bfloat16* wp = s.w0t + g * HLD_W0T + 16 * ks + 2 * t;
          const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
          mma_bf16(dx[mt], dl, b0, b1);
          mma_bf16(dx[mt], d, b0, b1);
        }
      }
    }
    if constexpr (MODE == 0) {
      __syncwarp();
    } else {
      __syncthreads();  // all warps' X and dH tiles complete
      // dW0 (+ bias in column 8): this warp's hidden rows [16 warp, +16) over the block's samples
#pragma unroll 2
      for (int kk = 0; kk < 8; ++kk) {
        const int src = kk >> 1, h16 = (kk & 1) * 16;
        const __nv_bfloat16* dhs = s.dh + src * 32 * HLD_H;
        const float* xs = s.x + src * 32 * HLD_X;
        uint32_t af[4];
        ldsm_x4_t(af, dhs + (h16 + (lane & 7) + (lane >> 4) * 8) * HLD_H + 16 * warp + ((lane >> 3) & 1) * 8);
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          const int col = nt * 8 + g;
          uint32_t b0 = 0u, b1 = 0u;
          if (col < HLD_X) {
            b0 = pack_bf16(xs[(h16 + 2 * t) * HLD_X + col], xs[(h16 + 2 * t + 1) * HLD_X + col]);
            b1 = pack_bf16(xs[(h16 + 2 * t + 8) * HLD_X + col], xs[(h16 + 2 * t + 9) * HLD_X + col]);
          }
          mma_bf16(acc_w0[nt], af, b0, b1);
        }
      }
      __syncthreads();  // tiles consumed: X tile can hold dX
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        *reinterpret_cast<float2*>(xf + (16 * mt + g) * HLD_X + 2 * t) = make_float2(dx[mt][0], dx[mt][1]);
        *reinterpret_cast<float2*>(xf + (16 * mt + g + 8) * HLD_X + 2 * t) = make_float2(dx[mt][2], dx[mt][3]);
      }
      __syncwarp();
      if (valid) {
        const float4 g0 = reinterpret_cast<const float4*>(xf + lane * HLD_X)[0];
        const float4 g1 = reinterpret_cast<const float4*>(xf + lane * HLD_X)[1];
        Corners<3> c;
        grid_corners(p, pos, c);
#pragma unroll
        for (int b = 0; b < 8; ++b) {
          if (c.idx[b] >= 0 && c.w[b] != 0.f) {
            const float w = c.w[b];
            float4* dst = reinterpret_cast<float4*>(grad_grid + (int64_t)c.idx[b] * 8);
            atomicAdd(dst, make_float4(g0.x * w, g0.y * w, g0.z * w, g0.w * w));
            atomicAdd(dst + 1, make_float4(g1.x * w, g1.y * w, g1.z * w, g1.w * w));
          }
        }
      }
      __syncwarp();
    }
  }
  if constexpr (MODE == 1) {
#pragma unroll
    for (int nt = 0; nt < 2; ++nt) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = 16 * warp + g + (q >= 2 ? 8 : 0);
        const int col = nt * 8 + 2 * t + (q & 1);
        if (col < 8) {
          if (gr.weight[0]) atomicAdd(gr.weight[0] + row * 8 + col, acc_w0[nt][q]);
        } else if (col == 8) {
          if (gr.bias[0]) atomicAdd(gr.bias[0] + row, acc_w0[nt][q]);
        }
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        float v = acc_w1[nt][j];
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        v += __shfl_xor_sync(0xffffffffu, v, 8);
        v += __shfl_xor_sync(0xffffffffu, v, 16);
        if (g == 0 && gr.weight[1]) atomicAdd(gr.weight[1] + nt * 8 + 2 * t + j, v);
      }
    }
  }
}

// Blocks of `kern` resident per SM (at least 1): the persistent grid is sm_count() times this.
template <typename K>
int resident_blocks(K kern, int threads, int64_t smem) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, (size_t)smem) != cudaSuccess) {
    (void)cudaGetLastError();
    per_sm = 1;
  }
  return std::max(per_sm, 1);
}

template <int MODE>
cudaError_t launch_head(const FFProposal& p, const void* grid, const float* rays, int64_t n, const FFMlp& m,
                        float* o_out, const float* g_o, float* grad_grid, const FFMlpGrad& gr, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  constexpr int64_t smem = head_smem_bytes<MODE>();
  const int64_t tiles = ceil_div(n * p.n_bins, kHT);
  if (p.param_dtype == FF_BF16) {
    static const int per_sm = resident_blocks(proposal_head_kernel<MODE, __nv_bfloat16>, kHT, smem);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count() * per_sm));
    proposal_head_kernel<MODE, __nv_bfloat16><<<blocks, kHT, smem, st>>>(p, (const __nv_bfloat16*)grid, rays, n, m,
                                                                         o_out, g_o, grad_grid, gr);
  } else {
    static const int per_sm = resident_blocks(proposal_head_kernel<MODE, float>, kHT, smem);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count() * per_sm));
    proposal_head_kernel<MODE, float><<<blocks, kHT, smem, st>>>(p, (const float*)grid, rays, n, m, o_out, g_o,
                                                                 grad_grid, gr);
  }
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_proposal_head_forward(const FFProposal& p, const void* grid, const FFMlp& m, const float* rays,
                                         int64_t n, float* o_out, cudaStream_t s) {
  FFMlpGrad none = {};
  return launch_head<0>(p, grid, rays, n, m, o_out, nullptr, nullptr, none, s);
}

cudaError_t launch_proposal_head_infer(const FFProposal& p, const void* grid, const FFMlp& m, const float* rays,
                                       int64_t n, float* o_out, cudaStream_t s) {
  FFMlpGrad none = {};
  return launch_head<2>(p, grid, rays, n, m, o_out, nullptr, nullptr, none, s);
}

cudaError_t launch_proposal_head_backward(const FFProposal& p, const void* grid, const FFMlp& m, const float* rays,
                                          int64_t n, const float* g_o, float* grad_grid, const FFMlpGrad& gr,
                                          cudaStream_t s) {
  return launch_head<1>(p, grid, rays, n, m, nullptr, g_o, grad_grid, gr, s);
}

cudaError_t launch_proposal_encode(const FFProposal& p, const void* grid, const float* rays, int64_t n, float* feat,
                                   cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int blocks = grid_blocks(n * p.n_bins, 256);
  if (p.param_dtype == FF_BF16)
    proposal_encode_kernel<__nv_bfloat16><<<blocks, 256, 0, s>>>(p, (const __nv_bfloat16*)grid, rays, n, feat);
  else
    proposal_encode_kernel<float><<<blocks, 256, 0, s>>>(p, (const float*)grid, rays, n, feat);
  return cudaGetLastError();
}

cudaError_t launch_proposal_scatter(const FFProposal& p, const float* rays, int64_t n, const float* grad_feat,
                                    float* grad_grid, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  proposal_scatter_kernel<<<grid_blocks(n * p.n_bins, 256), 256, 0, s>>>(p, rays, n, grad_feat, grad_grid);
  return cudaGetLastError();
}

cudaError_t launch_proposal_resample(const FFProposal& p, const float* rays, int64_t n, const float* o_prop,
                                     const float* jitter, const float* u, float* w_prop, float* xyz, float* zd,
                                     int32_t* bin_of, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const FFRender none = {};
  proposal_resample_kernel<kResampleAll><<<grid_blocks(n * 32, 256), 256, 0, s>>>(
      p, none, rays, n, o_prop, jitter, u, w_prop, xyz, zd, bin_of, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_proposal_resample_occupied(const FFProposal& p, const FFRender& r, const float* rays, int64_t n,
                                              const float* o_prop, const float* jitter, int32_t* counts,
                                              int64_t* offsets, void* workspace, float* xyz, float* zd,
                                              cudaStream_t s) {
  if (n == 0) return cudaMemsetAsync(offsets, 0, sizeof(int64_t), s);
  const int blocks = grid_blocks(n * 32, 256);
  proposal_resample_kernel<kResampleCount><<<blocks, 256, 0, s>>>(p, r, rays, n, o_prop, jitter, nullptr, nullptr,
                                                                   nullptr, nullptr, nullptr, counts, nullptr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_scan(counts, n, offsets, workspace, s);
  if (e != cudaSuccess) return e;
  proposal_resample_kernel<kResampleEmit><<<blocks, 256, 0, s>>>(p, r, rays, n, o_prop, jitter, nullptr, nullptr,
                                                                  xyz, zd, nullptr, nullptr, offsets);
  return cudaGetLastError();
}

cudaError_t launch_proposal_loss(const FFProposal& p, const float* rays, int64_t n, const float* o_prop,
                                 const float* w_field, const int32_t* bin_of, float loss_scale, float* loss_sum,
                                 float* grad_o, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  proposal_loss_kernel<<<grid_blocks(n * 32, 256), 256, 0, s>>>(p, rays, n, o_prop, w_field, bin_of, loss_scale,
                                                                loss_sum, grad_o);
  return cudaGetLastError();
}

}  // namespace ffgb
