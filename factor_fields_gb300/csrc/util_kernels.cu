// Zeroing of several float32 buffers in one launch (a fit step's gradient buffers and loss
// accumulator: one kernel instead of one fill per tensor). float4 stores where a buffer is
// 16-byte aligned, scalar stores for the rest; blockIdx.y selects the buffer.
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kZeroThreads = 256;

struct ZeroJob {
  float* p[kMaxZeroBuffers];
  int64_t n[kMaxZeroBuffers];
};

// __grid_constant__: blockIdx.y indexes the parameter in place (a plain by-value struct indexed
// at run time is first copied to every thread's local memory)
__global__ void __launch_bounds__(kZeroThreads) zero_buffers_kernel(const __grid_constant__ ZeroJob job) {
  float* p = job.p[blockIdx.y];
  const int64_t n = job.n[blockIdx.y];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t head = 0;  // scalar elements before the first 16-byte boundary
  if (reinterpret_cast<uintptr_t>(p) & 15) head = min(n, (int64_t)((16 - (reinterpret_cast<uintptr_t>(p) & 15)) / 4));
  const int64_t n4 = (n - head) / 4;
  float4* q = reinterpret_cast<float4*>(p + head);
  for (int64_t i = t0; i < n4; i += stride) q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  const int64_t tail = head + n4 * 4;
  for (int64_t i = t0; i < head; i += stride) p[i] = 0.f;
  for (int64_t i = tail + t0; i < n; i += stride) p[i] = 0.f;
}

}  // namespace

cudaError_t launch_zero_buffers(float* const* ptrs, const int64_t* counts, int n_buffers, cudaStream_t st) {
  for (int b0 = 0; b0 < n_buffers; b0 += kMaxZeroBuffers) {
    ZeroJob job = {};
    int nb = 0;
    int64_t most = 0;
    for (int b = b0; b < n_buffers && nb < kMaxZeroBuffers; ++b) {
      if (counts[b] <= 0) continue;
      job.p[nb] = ptrs[b];
      job.n[nb] = counts[b];
      most = std::max(most, counts[b]);
      ++nb;
    }
    if (nb == 0) continue;
    const int64_t want = ceil_div(ceil_div(most, 4), kZeroThreads);
    const int bx = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 8));
    zero_buffers_kernel<<<dim3(bx, nb), kZeroThreads, 0, st>>>(job);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace ffgb
