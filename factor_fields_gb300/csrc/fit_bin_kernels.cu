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
//   bin      (key[i], rank[i] = atomicAdd(count[key], 1))        thread per point
//   scan     offsets = exclusive prefix sum of count             one block up to 2^15 keys, else
//                                                                the two-level scan (render_kernels.cu)
//   permute  row[offsets[key] + rank] = (x[i], target[i], 0 pad)  one 16-byte-multiple row per point
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kBinThreads = 256;
constexpr int kScanThreads1 = 1024;
constexpr int64_t kOneBlockKeys = kScanThreads1 * 32;  // scan in a single block up to this many keys

template <int CD>
__global__ void __launch_bounds__(kBinThreads) fit_bin_kernel(const FFField f, const float* __restrict__ x,
                                                              int64_t n, int32_t n_keys, int32_t* __restrict__ count,
                                                              int2* __restrict__ key_rank) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float p[CD];
#pragma unroll
    for (int k = 0; k < CD; ++k) p[k] = x[i * CD + k];
    Corners<CD> cc;
    coeff_corners<CD>(f, p, cc);
    int32_t k = cc.idx[0];
    if (k < 0 || k >= n_keys) k = 0;  // non-finite coordinates: any bin will do
    key_rank[i] = make_int2(k, atomicAdd(count + k, 1));
  }
}

// Exclusive prefix sum of n <= kOneBlockKeys counts in one block. Warp w owns the 32 x 32 counts
// [1024 w, 1024 (w + 1)); lane l holds counts 1024 w + 32 k + l (k < 32) in registers, loaded in
// one coalesced round. The warps' totals are scanned in shared memory; each warp then scans its
// counts 32 at a time (warp shuffle scan, carry from the previous 32).
__global__ void __launch_bounds__(kScanThreads1) fit_scan_one_block_kernel(const int32_t* __restrict__ count,
                                                                           int64_t n, int64_t* __restrict__ offsets) {
  constexpr int kWarps = kScanThreads1 / 32;
  __shared__ int64_t chunk_start[kWarps + 1];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int32_t v[32];
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const int64_t i = (int64_t)warp * 1024 + k * 32 + lane;
    v[k] = i < n ? count[i] : 0;
    s += v[k];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) chunk_start[warp + 1] = s;
  __syncthreads();
  if (tid == 0) {
    chunk_start[0] = 0;
    for (int w = 1; w <= kWarps; ++w) chunk_start[w] += chunk_start[w - 1];
  }
  __syncthreads();
  int64_t carry = chunk_start[warp];
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const int64_t i = (int64_t)warp * 1024 + k * 32 + lane;
    int32_t incl = v[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    if (i < n) offsets[i] = carry + incl - v[k];
    carry += __shfl_sync(0xffffffffu, incl, 31);
  }
  if (tid == 0) offsets[n] = chunk_start[kWarps];
}

// One row of `stride` floats per binned point: coordinates, targets, zero padding.
template <int CD>
__global__ void __launch_bounds__(kBinThreads) fit_permute_kernel(const float* __restrict__ x,
                                                                  const float* __restrict__ target, int out_dim,
                                                                  int64_t n, const int2* __restrict__ key_rank,
                                                                  const int64_t* __restrict__ offsets, int stride,
                                                                  float* __restrict__ rows) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int2 kr = key_rank[i];
    float4* dst = reinterpret_cast<float4*>(rows + (offsets[kr.x] + kr.y) * stride);
    if (CD == 3 && out_dim == 1) {
      dst[0] = make_float4(x[i * 3], x[i * 3 + 1], x[i * 3 + 2], target[i]);
    } else {
      for (int q = 0; q < stride; q += 4) {
        float v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = q + j;
          v[j] = c < CD ? x[i * CD + c] : (c < CD + out_dim ? target[i * out_dim + c - CD] : 0.f);
        }
        dst[q / 4] = make_float4(v[0], v[1], v[2], v[3]);
      }
    }
  }
}

int bin_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kBinThreads), (int64_t)sm_count() * 8));
}

int64_t align_up(int64_t b) { return (b + 255) & ~int64_t(255); }

int row_stride(const FFField& f, int out_dim) { return (int)(ceil_div(f.coord_dim + out_dim, 4) * 4); }

}  // namespace

int64_t fit_bin_keys(const FFField& f) {
  int64_t k = 1;
  for (int d = 0; d < f.coord_dim; ++d) k *= f.coeff_reso[d];
  return k;
}

int64_t fit_bin_workspace_bytes(const FFField& f, int64_t n, int out_dim) {
  const int64_t keys = fit_bin_keys(f);
  return align_up(keys * 4) + align_up(n * 8) + align_up((keys + 1) * 8) + align_up(scan_workspace_bytes(keys)) +
         align_up(n * row_stride(f, out_dim) * 4);
}

cudaError_t launch_fit_bin(const FFField& f, const float* x, const float* target, int out_dim, int64_t n,
                           void* workspace, const float** rows_out, int64_t* stride_out, cudaStream_t st) {
  const int64_t keys = fit_bin_keys(f);
  const int stride = row_stride(f, out_dim);
  unsigned char* w = static_cast<unsigned char*>(workspace);
  int32_t* count = reinterpret_cast<int32_t*>(w); w += align_up(keys * 4);
  int2* key_rank = reinterpret_cast<int2*>(w); w += align_up(n * 8);
  int64_t* offsets = reinterpret_cast<int64_t*>(w); w += align_up((keys + 1) * 8);
  void* scan_ws = w; w += align_up(scan_workspace_bytes(keys));
  float* rows = reinterpret_cast<float*>(w);
  *rows_out = rows;
  *stride_out = stride;
  cudaError_t e = cudaMemsetAsync(count, 0, keys * 4, st);
  if (e != cudaSuccess) return e;
  const int blocks = bin_blocks(n);
  if (f.coord_dim == 3)
    fit_bin_kernel<3><<<blocks, kBinThreads, 0, st>>>(f, x, n, (int32_t)keys, count, key_rank);
  else
    fit_bin_kernel<2><<<blocks, kBinThreads, 0, st>>>(f, x, n, (int32_t)keys, count, key_rank);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (keys <= kOneBlockKeys) {
    fit_scan_one_block_kernel<<<1, kScanThreads1, 0, st>>>(count, keys, offsets);
    e = cudaGetLastError();
  } else {
    e = launch_scan(count, keys, offsets, scan_ws, st);
  }
  if (e != cudaSuccess) return e;
  if (f.coord_dim == 3)
    fit_permute_kernel<3><<<blocks, kBinThreads, 0, st>>>(x, target, out_dim, n, key_rank, offsets, stride, rows);
  else
    fit_permute_kernel<2><<<blocks, kBinThreads, 0, st>>>(x, target, out_dim, n, key_rank, offsets, stride, rows);
  return cudaGetLastError();
}

int fit_bin_kernel_launches(const FFField& f) { return fit_bin_keys(f) <= kOneBlockKeys ? 3 : 5; }

}  // namespace ffgb
