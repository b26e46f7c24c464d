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
      const float o = o_row[lane * B + b];
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

__global__ void __launch_bounds__(256) proposal_resample_kernel(
    const FFProposal p, const float* __restrict__ rays, int64_t n_rays, const float* __restrict__ o_prop,
    const float* __restrict__ jitter, const float* __restrict__ u_given, float* __restrict__ w_prop,
    float* __restrict__ xyz, float* __restrict__ zd, int32_t* __restrict__ bin_of) {
  __shared__ float cdf_s[8][kMaxBinsPerLane * 32 + 1];
  __shared__ float t_s[8][kMaxFine];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int nb = p.n_bins, nf = p.n_fine, B = nb / 32;
  float* cdf = cdf_s[wib];
  float* ts = t_s[wib];
  for (int64_t ray = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; ray < n_rays;
       ray += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const Segment s = segment(p, rays, ray);
    BinState st;
    bin_weights(p, o_prop + ray * nb, s.len, lane, B, st);
    // pdf = (w + 1e-5) / sum, cdf with a leading zero (sample_pdf, ray_utils.py:135-138)
    float lsum = 0.f;
#pragma unroll
    for (int b = 0; b < kMaxBinsPerLane; ++b)
      if (b < B) {
        w_prop[ray * nb + lane * B + b] = st.w[b];
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
    for (int i = lane; i < nf; i += 32) {
      float u;
      if (u_given)
        u = u_given[ray * nf + i];
      else
        u = ((float)i + (jitter ? jitter[ray] : 0.5f)) / (float)nf;
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
      const float t = eb + tt * (ea - eb);
      ts[i] = t;
      bin_of[ray * nf + i] = min(below, nb - 1);
#pragma unroll
      for (int q = 0; q < 3; ++q) xyz[(ray * nf + i) * 3 + q] = s.o[q] + s.d[q] * t;
    }
    __syncwarp();
    for (int i = lane; i < nf; i += 32) {
      const float t = ts[i];
      const float nxt = (i + 1 < nf) ? ts[i + 1] : s.t_out;
      zd[(ray * nf + i) * 2 + 0] = t;
      zd[(ray * nf + i) * 2 + 1] = fmaxf(nxt - t, 0.f);
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
    for (int i = lane; i < nf; i += 32) atomicAdd(&mass[bin_of[ray * nf + i]], w_field[ray * nf + i]);
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

}  // namespace

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
  proposal_resample_kernel<<<grid_blocks(n * 32, 256), 256, 0, s>>>(p, rays, n, o_prop, jitter, u, w_prop, xyz, zd,
                                                                    bin_of);
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
