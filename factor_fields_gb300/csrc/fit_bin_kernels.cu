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
//   bin      (key[i], rank[i] = atomicAdd(count[key], 1))          thread per point; optionally
//                                                                  also zeroes the step's gradients
//   alloc    start[key] = atomicAdd(cursor, count[key])           warp per 32 keys, one atomic per
//                                                                  warp: every key gets a contiguous
//                                                                  range; the order of the ranges is
//                                                                  whatever the atomics hand out
//   permute  row[start[key] + rank] = (x[i], target[i], 0 pad)    one 16-byte-multiple row per point
// Only contiguity matters (segments are found from the keys of adjacent lanes), so no scan.
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kBinThreads = 256;

// Buffers the bin kernel zeroes before the fit accumulates into them (FF_FIT_ZERO_GRADS).
struct ZeroSet {
  float* vec4[2];  // 16-byte aligned: grid gradients
  int64_t n4[2];   // float4 counts
  float* flt[6];   // MLP gradients, loss accumulator, the grid gradients' last (n % 4) elements
  int64_t n[6];
};

template <int CD>
__global__ void __launch_bounds__(kBinThreads) fit_bin_kernel(const FFField f, const float* __restrict__ x,
                                                              int64_t n, int32_t n_keys, int32_t* __restrict__ count,
                                                              int2* __restrict__ key_rank,
                                                              const __grid_constant__ ZeroSet zs) {
  pdl_launch_dependents();  // the alloc kernel may start; it waits for this one before reading counts
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = t0; i < n; i += stride) {
    float p[CD];
#pragma unroll
    for (int k = 0; k < CD; ++k) p[k] = x[i * CD + k];
    Corners<CD> cc;
    coeff_corners<CD, true>(f, p, cc);  // the low corner as the fit kernel computes it
    int32_t k = cc.idx[0];
    if (k < 0 || k >= n_keys) k = 0;  // non-finite coordinates: any bin will do
    key_rank[i] = make_int2(k, atomicAdd(count + k, 1));
  }
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    float4* q = reinterpret_cast<float4*>(zs.vec4[b]);
    for (int64_t i = t0; i < zs.n4[b]; i += stride) q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
#pragma unroll
  for (int b = 0; b < 6; ++b)
    for (int64_t i = t0; i < zs.n[b]; i += stride) zs.flt[b][i] = 0.f;
}

// Warp per 32 keys: a contiguous range of count[key] rows for every key, one atomic per warp.
__global__ void __launch_bounds__(kBinThreads) fit_alloc_kernel(const int32_t* __restrict__ count, int64_t n_keys,
                                                                int64_t* __restrict__ cursor,
                                                                int64_t* __restrict__ start) {
  pdl_launch_dependents();
  pdl_wait();  // the counts are complete
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w * 32 < n_keys; w += warps) {
    const int64_t k = w * 32 + lane;
    const int32_t c = k < n_keys ? count[k] : 0;
    int32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int32_t u = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += u;
    }
    int64_t base = 0;
    if (lane == 31 && incl > 0) base = atomicAdd(reinterpret_cast<unsigned long long*>(cursor),
                                                 (unsigned long long)incl);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (k < n_keys) start[k] = base + incl - c;
  }
}

// One row of `stride` floats per binned point: coordinates, targets, zero padding.
template <int CD>
__global__ void __launch_bounds__(kBinThreads) fit_permute_kernel(const float* __restrict__ x,
                                                                  const float* __restrict__ target, int out_dim,
                                                                  int64_t n, const int2* __restrict__ key_rank,
                                                                  const int64_t* __restrict__ start, int stride,
                                                                  float* __restrict__ rows) {
  pdl_wait();  // the ranges are complete
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int2 kr = key_rank[i];
    float4* dst = reinterpret_cast<float4*>(rows + (start[kr.x] + kr.y) * stride);
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
  // the fit kernel (3 blocks per SM fill the register file) launches once every block is past here
  pdl_launch_dependents();
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

int64_t field_basis_elems(const FFField& f) {
  int64_t most = 0;
  for (int l = 0; l < f.n_levels; ++l) {
    int64_t cells = 1;
    for (int d = 0; d < f.basis_dim; ++d) cells *= f.level_reso[l];
    most = std::max(most, f.level_offset[l] + cells * f.level_stride[l]);
  }
  return most;
}

int64_t fit_bin_workspace_bytes(const FFField& f, int64_t n, int out_dim) {
  const int64_t keys = fit_bin_keys(f);
  return align_up(keys * 4 + 16) + align_up(n * 8) + align_up(keys * 8) + align_up(n * row_stride(f, out_dim) * 4) +
         align_up(n * f.coord_dim * 4) + align_up(n * out_dim * 4);
}

// Workspace layout: count[keys] + cursor | key_rank[n] | start[keys] | rows[n][stride] |
// x[n][coord_dim] | target[n][out_dim] (the last two: a host batch's device copy).
cudaError_t fit_bin_stage_host(const FFField& f, const float** x, const float** target, int out_dim, int64_t n,
                               void* workspace, cudaStream_t st) {
  const int64_t keys = fit_bin_keys(f);
  unsigned char* w = static_cast<unsigned char*>(workspace) + align_up(keys * 4 + 16) + align_up(n * 8) +
                     align_up(keys * 8) + align_up(n * row_stride(f, out_dim) * 4);
  float* xs = reinterpret_cast<float*>(w);
  float* ts = reinterpret_cast<float*>(w + align_up(n * f.coord_dim * 4));
  if (n > 0) {
    // cudaMemcpyDefault: the direction comes from the pointers (unified addressing)
    cudaError_t e = cudaMemcpyAsync(xs, *x, n * f.coord_dim * 4, cudaMemcpyDefault, st);
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(ts, *target, n * out_dim * 4, cudaMemcpyDefault, st);
    if (e != cudaSuccess) return e;
  }
  *x = xs;
  *target = ts;
  return cudaSuccess;
}
const float* fit_bin_rows(const FFField& f, int64_t n, int out_dim, const void* workspace, int64_t* stride_out) {
  const int64_t keys = fit_bin_keys(f);
  *stride_out = row_stride(f, out_dim);
  return reinterpret_cast<const float*>(static_cast<const unsigned char*>(workspace) + align_up(keys * 4 + 16) +
                                        align_up(n * 8) + align_up(keys * 8));
}

cudaError_t launch_fit_bin(const FFField& f, const float* x, const float* target, int out_dim, int64_t n,
                           void* workspace, const FitZero* zero, cudaStream_t st) {
  const int64_t keys = fit_bin_keys(f);
  const int stride = row_stride(f, out_dim);
  unsigned char* w = static_cast<unsigned char*>(workspace);
  int32_t* count = reinterpret_cast<int32_t*>(w);
  int64_t* cursor = reinterpret_cast<int64_t*>(w + ((keys * 4 + 7) & ~int64_t(7)));
  w += align_up(keys * 4 + 16);
  int2* key_rank = reinterpret_cast<int2*>(w); w += align_up(n * 8);
  int64_t* start = reinterpret_cast<int64_t*>(w); w += align_up(keys * 8);
  float* rows = reinterpret_cast<float*>(w);
  cudaError_t e = cudaMemsetAsync(count, 0, ((keys * 4 + 7) & ~int64_t(7)) + 8, st);
  if (e != cudaSuccess) return e;
  ZeroSet zs = {};
  if (zero) {
    float* grids[2] = {zero->grad_basis, zero->grad_coeff};
    const int64_t elems[2] = {field_basis_elems(f), keys * f.coeff_stride};
    for (int b = 0; b < 2; ++b) {
      if (!grids[b]) continue;
      zs.vec4[b] = grids[b];
      zs.n4[b] = elems[b] / 4;
      zs.flt[4 + b] = grids[b] + zs.n4[b] * 4;
      zs.n[4 + b] = elems[b] % 4;
    }
    for (int b = 0; b < 4; ++b) {
      zs.flt[b] = zero->other[b];
      zs.n[b] = zero->other[b] ? zero->other_n[b] : 0;
    }
  }
  const int blocks = bin_blocks(std::max<int64_t>(n, zs.n4[0]));
  if (f.coord_dim == 3)
    fit_bin_kernel<3><<<blocks, kBinThreads, 0, st>>>(f, x, n, (int32_t)keys, count, key_rank, zs);
  else
    fit_bin_kernel<2><<<blocks, kBinThreads, 0, st>>>(f, x, n, (int32_t)keys, count, key_rank, zs);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const int ablocks = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(keys, kBinThreads), (int64_t)sm_count() * 8));
  e = launch_pdl(fit_alloc_kernel, dim3(ablocks), dim3(kBinThreads), 0, st, (const int32_t*)count, keys, cursor, start);
  if (e != cudaSuccess) return e;
  const int pblocks = bin_blocks(n);
  if (f.coord_dim == 3)
    e = launch_pdl(fit_permute_kernel<3>, dim3(pblocks), dim3(kBinThreads), 0, st, x, target, out_dim, n,
                   (const int2*)key_rank, (const int64_t*)start, stride, rows);
  else
    e = launch_pdl(fit_permute_kernel<2>, dim3(pblocks), dim3(kBinThreads), 0, st, x, target, out_dim, n,
                   (const int2*)key_rank, (const int64_t*)start, stride, rows);
  return e;
}

}  // namespace ffgb
