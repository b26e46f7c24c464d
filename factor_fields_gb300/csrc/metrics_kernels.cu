// Image metrics of the evaluation renderer (renderer.py:30-98): mean squared error (PSNR) and
// SSIM as utils.py:110-156 computes it (rgb_ssim, from mip-NeRF): per channel, an 11-tap
// Gaussian (sigma 1.5) separable 'valid' blur of x, y, x^2, y^2, x*y (the products rounded to
// float32 like the reference's tensor ops, the blurs in float64 like scipy), variances clipped at
// 0, covariance clipped to +-sqrt(var0 var1), then the SSIM map averaged over the valid window.
//
//   vertical   thread per (channel, valid row, column): 5 float64 sums over 11 rows
//   horizontal thread per (channel, valid row, valid column): 5 sums over 11 columns, the SSIM
//              term, and the block's partial sums of SSIM and squared error (float64 atomics)
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kTaps = 11;
constexpr int kMetThreads = 256;

struct Taps {
  double w[kTaps];
};

__global__ void __launch_bounds__(kMetThreads) ssim_vertical_kernel(const float* __restrict__ a,
                                                                    const float* __restrict__ b, int h, int w, int c,
                                                                    const Taps taps, double* __restrict__ tmp) {
  const int hv = h - (kTaps - 1);
  const int64_t total = (int64_t)c * hv * w;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % w), y = (int)((t / w) % hv), ch = (int)(t / ((int64_t)w * hv));
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int k = 0; k < kTaps; ++k) {
      const int64_t i = ((int64_t)(y + k) * w + x) * c + ch;  // images are [h][w][c]
      const float u = a[i], v = b[i];
      const double wk = taps.w[k];
      s[0] += wk * (double)u;
      s[1] += wk * (double)v;
      s[2] += wk * (double)__fmul_rn(u, u);
      s[3] += wk * (double)__fmul_rn(v, v);
      s[4] += wk * (double)__fmul_rn(u, v);
    }
#pragma unroll
    for (int q = 0; q < 5; ++q) tmp[q * total + t] = s[q];
  }
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) r += sh[i];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kMetThreads) ssim_horizontal_kernel(const double* __restrict__ tmp, int h, int w,
                                                                      int c, const Taps taps, double c1, double c2,
                                                                      const float* __restrict__ a,
                                                                      const float* __restrict__ b,
                                                                      double* __restrict__ sums) {
  __shared__ double sh[kMetThreads / 32];
  const int hv = h - (kTaps - 1), wv = w - (kTaps - 1);
  const int64_t plane = (int64_t)c * hv * w, total = (int64_t)c * hv * wv;
  const int64_t n_px = (int64_t)h * w * c;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double ssim = 0.0, sq = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += stride) {
    const int x = (int)(t % wv), y = (int)((t / wv) % hv), ch = (int)(t / ((int64_t)wv * hv));
    double s[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    const int64_t row = ((int64_t)ch * hv + y) * w;
#pragma unroll
    for (int k = 0; k < kTaps; ++k) {
#pragma unroll
      for (int q = 0; q < 5; ++q) s[q] += taps.w[k] * tmp[q * plane + row + x + k];
    }
    const double mu00 = s[0] * s[0], mu11 = s[1] * s[1], mu01 = s[0] * s[1];
    const double s00 = fmax(0.0, s[2] - mu00), s11 = fmax(0.0, s[3] - mu11);
    double s01 = s[4] - mu01;
    s01 = (s01 > 0.0 ? 1.0 : (s01 < 0.0 ? -1.0 : 0.0)) * fmin(sqrt(s00 * s11), fabs(s01));
    ssim += ((2.0 * mu01 + c1) * (2.0 * s01 + c2)) / ((mu00 + mu11 + c1) * (s00 + s11 + c2));
  }
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_px; i += stride) {
    const double d = (double)a[i] - (double)b[i];
    sq += d * d;
  }
  const double s_ssim = block_sum(ssim, sh);
  const double s_sq = block_sum(sq, sh);
  if (threadIdx.x == 0) {
    atomicAdd(sums, s_ssim);
    atomicAdd(sums + 1, s_sq);
  }
}

}  // namespace

int64_t image_metrics_workspace_bytes(int h, int w, int c) {
  return 5 * (int64_t)c * (h - (kTaps - 1)) * w * 8 + 2 * 8;
}

cudaError_t launch_image_metrics(const float* a, const float* b, int h, int w, int c, float max_val,
                                 void* workspace, double* out_host, cudaStream_t st) {
  Taps taps;
  double tot = 0.0;
  const int hw = kTaps / 2;
  const double shift = (2.0 * hw - kTaps + 1) / 2.0;
  for (int i = 0; i < kTaps; ++i) {
    const double f = (i - hw + shift) / 1.5;
    taps.w[i] = std::exp(-0.5 * f * f);
    tot += taps.w[i];
  }
  for (int i = 0; i < kTaps; ++i) taps.w[i] /= tot;
  const double c1 = (0.01 * max_val) * (0.01 * max_val), c2 = (0.03 * max_val) * (0.03 * max_val);
  double* tmp = static_cast<double*>(workspace);
  double* sums = tmp + 5 * (int64_t)c * (h - (kTaps - 1)) * w;
  cudaError_t e = cudaMemsetAsync(sums, 0, 2 * sizeof(double), st);
  if (e != cudaSuccess) return e;
  const int64_t vtot = (int64_t)c * (h - (kTaps - 1)) * w;
  const int vb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(vtot, kMetThreads), (int64_t)sm_count() * 8));
  ssim_vertical_kernel<<<vb, kMetThreads, 0, st>>>(a, b, h, w, c, taps, tmp);
  const int64_t htot = (int64_t)c * (h - (kTaps - 1)) * (w - (kTaps - 1));
  const int hb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(htot, kMetThreads), (int64_t)sm_count() * 8));
  ssim_horizontal_kernel<<<hb, kMetThreads, 0, st>>>(tmp, h, w, c, taps, c1, c2, a, b, sums);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  double host[2] = {0.0, 0.0};
  e = cudaMemcpyAsync(host, sums, sizeof(host), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return e;
  out_host[0] = host[1] / (double)((int64_t)h * w * c);  // mse
  out_host[1] = host[0] / (double)htot;                  // ssim
  return cudaSuccess;
}

}  // namespace ffgb
