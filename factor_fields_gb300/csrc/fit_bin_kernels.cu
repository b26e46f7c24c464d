// Binning of a fit batch by coefficient cell (a counting sort), so that the points a warp of the
// fused fit kernel handles share coefficient corners and their coefficient gradients can be
// summed on chip before the atomics (fused_kernels.cu, kFitBinned).
//
// The key of a point is the flat index of its coefficient cell, i.e. of its low trilinear corner
// (x0, y0[, z0]) under the get_coeff lookup (align_corners=False, border padding,
// models/FactorFields.py:425-434): every point of one cell has the same corner set. Order inside
// a cell is the order in which the atomics hand out ranks; results do not depend on it (the
// gradients are sums).
//
//   bin      key[i], rank[i] = atomicAdd(count[key], 1)        thread per point
//   scan     offsets = exclusive prefix sum of count           (render_kernels.cu)
//   permute  x_sorted[offsets[key] + rank] = x[i], same for the targets
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kBinThreads = 256;

template <int CD>
__global__ void __launch_bounds__(kBinThreads) fit_bin_kernel(const FFField f, const float* __restrict__ x,
                                                              int64_t n, int32_t n_keys, int32_t* __restrict__ count,
                                                              int32_t* __restrict__ key, int32_t* __restrict__ rank) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[CD];
#pragma unroll
    for (int k = 0; k < CD; ++k) p[k] = x[i * CD + k];
    Corners<CD> cc;
    coeff_corners<CD>(f, p, cc);
    int32_t k = cc.idx[0];
    if (k < 0 || k >= n_keys) k = 0;  // non-finite coordinates: any bin will do
    key[i] = k;
    rank[i] = atomicAdd(count + k, 1);
  }
}

template <int CD>
__global__ void __launch_bounds__(kBinThreads) fit_permute_kernel(const float* __restrict__ x,
                                                                  const float* __restrict__ target, int out_dim,
                                                                  int64_t n, const int32_t* __restrict__ key,
                                                                  const int32_t* __restrict__ rank,
                                                                  const int64_t* __restrict__ offsets,
                                                                  float* __restrict__ xs, float* __restrict__ ts) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = offsets[key[i]] + rank[i];
#pragma unroll
    for (int k = 0; k < CD; ++k) xs[pos * CD + k] = x[i * CD + k];
    for (int o = 0; o < out_dim; ++o) ts[pos * out_dim + o] = target[i * out_dim + o];
  }
}

int bin_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kBinThreads), (int64_t)sm_count() * 8));
}

int64_t align_up(int64_t b) { return (b + 255) & ~int64_t(255); }

}  // namespace

int64_t fit_bin_keys(const FFField& f) {
  int64_t k = 1;
  for (int d = 0; d < f.coord_dim; ++d) k *= f.coeff_reso[d];
  return k;
}

int64_t fit_bin_workspace_bytes(const FFField& f, int64_t n, int out_dim) {
  const int64_t keys = fit_bin_keys(f);
  return align_up(keys * 4) + 2 * align_up(n * 4) + align_up((keys + 1) * 8) + align_up(scan_workspace_bytes(keys)) +
         align_up(n * f.coord_dim * 4) + align_up(n * out_dim * 4);
}

cudaError_t launch_fit_bin(const FFField& f, const float* x, const float* target, int out_dim, int64_t n,
                           void* workspace, const float** xs_out, const float** ts_out, cudaStream_t st) {
  const int64_t keys = fit_bin_keys(f);
  unsigned char* w = static_cast<unsigned char*>(workspace);
  int32_t* count = reinterpret_cast<int32_t*>(w); w += align_up(keys * 4);
  int32_t* key = reinterpret_cast<int32_t*>(w); w += align_up(n * 4);
  int32_t* rank = reinterpret_cast<int32_t*>(w); w += align_up(n * 4);
  int64_t* offsets = reinterpret_cast<int64_t*>(w); w += align_up((keys + 1) * 8);
  void* scan_ws = w; w += align_up(scan_workspace_bytes(keys));
  float* xs = reinterpret_cast<float*>(w); w += align_up(n * f.coord_dim * 4);
  float* ts = reinterpret_cast<float*>(w);
  *xs_out = xs;
  *ts_out = ts;
  cudaError_t e = cudaMemsetAsync(count, 0, keys * 4, st);
  if (e != cudaSuccess) return e;
  const int blocks = bin_blocks(n);
  if (f.coord_dim == 3)
    fit_bin_kernel<3><<<blocks, kBinThreads, 0, st>>>(f, x, n, (int32_t)keys, count, key, rank);
  else
    fit_bin_kernel<2><<<blocks, kBinThreads, 0, st>>>(f, x, n, (int32_t)keys, count, key, rank);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = launch_scan(count, keys, offsets, scan_ws, st);
  if (e != cudaSuccess) return e;
  if (f.coord_dim == 3)
    fit_permute_kernel<3><<<blocks, kBinThreads, 0, st>>>(x, target, out_dim, n, key, rank, offsets, xs, ts);
  else
    fit_permute_kernel<2><<<blocks, kBinThreads, 0, st>>>(x, target, out_dim, n, key, rank, offsets, xs, ts);
  return cudaGetLastError();
}

}  // namespace ffgb
