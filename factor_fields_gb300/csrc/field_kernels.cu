// Drop-in field evaluation: get_coding forward and its backward scatter.
//
// Replaces, for basis_type = coeff_type = 'grid':
//   get_coeff   models/FactorFields.py:425-434  (F.grid_sample, align_corners=False, border)
//   get_basis   models/FactorFields.py:467-490  (grid_mapping + one F.grid_sample per level,
//                                                align_corners=True, zeros padding)
//   get_coding  models/FactorFields.py:523-527  (basis * coeff)
// and the ATen grid_sampler_{2d,3d}_backward scatter that autograd runs for them.
//
// One thread per point. The coefficient corners are computed once per point; each level's
// corners are computed once and its channels are walked in vectors of level_vec[l] channels
// (channels-last storage, so one corner's channels are one 8/16-byte load). All levels and the
// coefficient gather run in ONE launch (the reference issues one grid_sample per level).
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

template <int V, int BD, int CD, typename T>
__device__ __forceinline__ void level_forward(const FFField& f, int l, int foff, const T* __restrict__ basis,
                                              const T* __restrict__ coeff, const Corners<BD>& bc,
                                              const Corners<CD>& cc, int64_t i, float* feats, float* coeff_out,
                                              float* basis_out) {
  const T* bl = basis + f.level_offset[l];
  const int C = f.level_channels[l];
  const int64_t row = i * f.n_feat + foff;
  for (int c = 0; c < C; c += V) {
    float b[V], cv[V];
    gather<V, BD>(bl, f.level_stride[l], c, bc, b);
    gather<V, CD>(coeff, f.coeff_stride, foff + c, cc, cv);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      if (feats) feats[row + c + v] = b[v] * cv[v];
      if (coeff_out) coeff_out[row + c + v] = cv[v];
      if (basis_out) basis_out[row + c + v] = b[v];
    }
  }
}

template <int BD, int CD, typename T>
__global__ void __launch_bounds__(256) field_forward_kernel(const FFField f, const T* __restrict__ basis,
                                                            const T* __restrict__ coeff,
                                                            const float* __restrict__ x, int64_t n,
                                                            float* __restrict__ feats,
                                                            float* __restrict__ coeff_out,
                                                            float* __restrict__ basis_out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[CD];
#pragma unroll
    for (int k = 0; k < CD; ++k) p[k] = x[i * CD + k];
    Corners<CD> cc;
    coeff_corners<CD>(f, p, cc);
    int foff = 0;
    for (int l = 0; l < f.n_levels; ++l) {
      Corners<BD> bc;
      basis_corners<BD>(f, l, p, bc);
      switch (f.level_vec[l]) {
        case 4: level_forward<4, BD, CD, T>(f, l, foff, basis, coeff, bc, cc, i, feats, coeff_out, basis_out); break;
        case 2: level_forward<2, BD, CD, T>(f, l, foff, basis, coeff, bc, cc, i, feats, coeff_out, basis_out); break;
        default: level_forward<1, BD, CD, T>(f, l, foff, basis, coeff, bc, cc, i, feats, coeff_out, basis_out); break;
      }
      foff += f.level_channels[l];
    }
  }
}

template <int V, int BD, int CD, typename T>
__device__ __forceinline__ void level_backward(const FFField& f, int l, int foff, const T* __restrict__ basis,
                                               const T* __restrict__ coeff, const Corners<BD>& bc,
                                               const Corners<CD>& cc, int64_t i, const float* grad_feats,
                                               const float* grad_coeff_out, const float* grad_basis_out,
                                               float* grad_basis, float* grad_coeff) {
  const T* bl = basis + f.level_offset[l];
  float* gbl = grad_basis + f.level_offset[l];
  const int C = f.level_channels[l];
  const int64_t row = i * f.n_feat + foff;
  for (int c = 0; c < C; c += V) {
    float b[V], cv[V], gb[V], gc[V];
    gather<V, BD>(bl, f.level_stride[l], c, bc, b);
    gather<V, CD>(coeff, f.coeff_stride, foff + c, cc, cv);
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const float gf = grad_feats ? grad_feats[row + c + v] : 0.f;
      gb[v] = gf * cv[v] + (grad_basis_out ? grad_basis_out[row + c + v] : 0.f);
      gc[v] = gf * b[v] + (grad_coeff_out ? grad_coeff_out[row + c + v] : 0.f);
    }
    if (grad_basis) scatter<V, BD>(gbl, f.level_stride[l], c, bc, gb);
    if (grad_coeff) scatter<V, CD>(grad_coeff, f.coeff_stride, foff + c, cc, gc);
  }
}

template <int BD, int CD, typename T>
__global__ void __launch_bounds__(256) field_backward_kernel(const FFField f, const T* __restrict__ basis,
                                                             const T* __restrict__ coeff,
                                                             const float* __restrict__ x, int64_t n,
                                                             const float* __restrict__ grad_feats,
                                                             const float* __restrict__ grad_coeff_out,
                                                             const float* __restrict__ grad_basis_out,
                                                             float* __restrict__ grad_basis,
                                                             float* __restrict__ grad_coeff) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[CD];
#pragma unroll
    for (int k = 0; k < CD; ++k) p[k] = x[i * CD + k];
    Corners<CD> cc;
    coeff_corners<CD>(f, p, cc);
    int foff = 0;
    for (int l = 0; l < f.n_levels; ++l) {
      Corners<BD> bc;
      basis_corners<BD>(f, l, p, bc);
      switch (f.level_vec[l]) {
        case 4: level_backward<4, BD, CD, T>(f, l, foff, basis, coeff, bc, cc, i, grad_feats, grad_coeff_out, grad_basis_out, grad_basis, grad_coeff); break;
        case 2: level_backward<2, BD, CD, T>(f, l, foff, basis, coeff, bc, cc, i, grad_feats, grad_coeff_out, grad_basis_out, grad_basis, grad_coeff); break;
        default: level_backward<1, BD, CD, T>(f, l, foff, basis, coeff, bc, cc, i, grad_feats, grad_coeff_out, grad_basis_out, grad_basis, grad_coeff); break;
      }
      foff += f.level_channels[l];
    }
  }
}

int grid_for(int64_t n, int threads) {
  const int64_t want = ceil_div(n, threads);
  const int64_t cap = (int64_t)sm_count() * 16;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

template <typename T, typename Fn>
cudaError_t dispatch_dims(const FFField& f, Fn&& fn) {
  if (f.basis_dim == 2 && f.coord_dim == 2) return fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 2>{});
  if (f.basis_dim == 3 && f.coord_dim == 3) return fn(std::integral_constant<int, 3>{}, std::integral_constant<int, 3>{});
  if (f.basis_dim == 2 && f.coord_dim == 3) return fn(std::integral_constant<int, 2>{}, std::integral_constant<int, 3>{});
  return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_field_forward(const FFField& f, const void* basis, const void* coeff, const float* x, int64_t n,
                                 float* feats, float* coeff_out, float* basis_out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int threads = 256, blocks = grid_for(n, threads);
  auto run = [&](auto bd, auto cd) -> cudaError_t {
    constexpr int BD = decltype(bd)::value, CD = decltype(cd)::value;
    if (f.param_dtype == FF_BF16)
      field_forward_kernel<BD, CD, __nv_bfloat16><<<blocks, threads, 0, s>>>(
          f, (const __nv_bfloat16*)basis, (const __nv_bfloat16*)coeff, x, n, feats, coeff_out, basis_out);
    else
      field_forward_kernel<BD, CD, float><<<blocks, threads, 0, s>>>(f, (const float*)basis, (const float*)coeff, x,
                                                                       n, feats, coeff_out, basis_out);
    return cudaGetLastError();
  };
  return dispatch_dims<float>(f, run);
}

cudaError_t launch_field_backward(const FFField& f, const void* basis, const void* coeff, const float* x, int64_t n,
                                  const float* grad_feats, const float* grad_coeff_out, const float* grad_basis_out,
                                  float* grad_basis, float* grad_coeff_grid, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const int threads = 256, blocks = grid_for(n, threads);
  auto run = [&](auto bd, auto cd) -> cudaError_t {
    constexpr int BD = decltype(bd)::value, CD = decltype(cd)::value;
    if (f.param_dtype == FF_BF16)
      field_backward_kernel<BD, CD, __nv_bfloat16><<<blocks, threads, 0, s>>>(
          f, (const __nv_bfloat16*)basis, (const __nv_bfloat16*)coeff, x, n, grad_feats, grad_coeff_out, grad_basis_out,
          grad_basis, grad_coeff_grid);
    else
      field_backward_kernel<BD, CD, float><<<blocks, threads, 0, s>>>(f, (const float*)basis, (const float*)coeff,
                                                                        x, n, grad_feats, grad_coeff_out,
                                                                        grad_basis_out, grad_basis, grad_coeff_grid);
    return cudaGetLastError();
  };
  return dispatch_dims<float>(f, run);
}

}  // namespace ffgb
