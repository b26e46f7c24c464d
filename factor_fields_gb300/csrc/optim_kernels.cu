// Adam (torch.optim.Adam, amsgrad=False, no weight decay; the reference's optimizer,
// train_per_scene.py:132, betas (0.9, 0.99)) fused with what a training step does around it:
// the update of every parameter, its BF16 copy for the field kernels, and the gradient zeroing
// of the next step, in one pass over the parameter (read p, g, m, v; write p, m, v, the BF16
// copy, g = 0).
//
// Per element, in torch's order (_single_tensor_adam):
//   m = lerp(m, g, 1 - beta1)              (m + w (g - m) for w < 0.5, else g - (g - m)(1 - w))
//   v = v * beta2 + (1 - beta2) * g * g    (mul_, addcmul_)
//   p = p - step_size * m / (sqrt(v) / sqrt(bc2) + eps),  step_size = lr / bc1
// with bc1 = 1 - beta1^t, bc2 = 1 - beta2^t. The host schedule computes them in double precision
// from each parameter's step and lr, as torch does in Python floats. The scheduled form reads the
// learning rate and the step counter from device memory, so that a captured CUDA graph replays
// the update with the current values; every thread forms the scales in float32 there, beta^t as
// exp2(t log2 beta) with log2 beta from the host in double (within a few ulp of the host
// schedule's; this GPU's FP64 rate is too low for a double pow per block: that measured 70 us
// for a 2.1 M-element update against ~12 us).
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kAdamThreads = 256;
constexpr int kMaxAdamParams = 8;  // parameters per launch

struct AdamParamDev {
  float* p;
  float* g;
  float* m;
  float* v;
  __nv_bfloat16* shadow;
  int64_t n;
  float neg_step_size;  // -lr / bc1 (host schedule)
  float bc2_sqrt;
  const double* lr;     // scheduled form: this parameter's learning rate in device memory
};

struct AdamJob {
  AdamParamDev prm[kMaxAdamParams];
  float w1;  // 1 - beta1 (lerp weight)
  float beta2, one_minus_beta2, eps;
  int zero_grad;
  float log2_beta1, log2_beta2;  // the scheduled form's bias corrections
  const int64_t* step;           // scheduled form: t after this update, shared by all parameters
};

struct AdamScale {
  float neg_step_size, bc2_sqrt;
};

__device__ __forceinline__ float adam_elem(float& p, float g, float& m, float& v, const AdamJob& j,
                                           const AdamScale& a) {
  const float w = j.w1;
  m = w < 0.5f ? __fadd_rn(m, __fmul_rn(w, __fsub_rn(g, m)))
               : __fsub_rn(g, __fmul_rn(__fsub_rn(g, m), __fsub_rn(1.f, w)));
  v = __fadd_rn(__fmul_rn(v, j.beta2), __fmul_rn(__fmul_rn(j.one_minus_beta2, g), g));
  const float denom = __fadd_rn(__fdiv_rn(__fsqrt_rn(v), a.bc2_sqrt), j.eps);
  p = __fadd_rn(p, __fmul_rn(a.neg_step_size, __fdiv_rn(m, denom)));
  return p;
}

// blockIdx.y: the parameter. float4 path when all four arrays are 16-byte aligned.
__global__ void __launch_bounds__(kAdamThreads) adam_kernel(const __grid_constant__ AdamJob job) {
  const AdamParamDev& a = job.prm[blockIdx.y];
  AdamScale sc = {a.neg_step_size, a.bc2_sqrt};
  if (job.step) {  // scheduled: the scales from lr and t in device memory
    const float t = (float)*job.step;
    const float bc1 = 1.f - exp2f(t * job.log2_beta1), bc2 = 1.f - exp2f(t * job.log2_beta2);
    sc.neg_step_size = -(float)*a.lr / bc1;
    sc.bc2_sqrt = sqrtf(bc2);
  }
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x, stride = (int64_t)gridDim.x * blockDim.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(a.p) | reinterpret_cast<uintptr_t>(a.g) |
                     reinterpret_cast<uintptr_t>(a.m) | reinterpret_cast<uintptr_t>(a.v)) & 15) == 0 &&
                   (!a.shadow || (reinterpret_cast<uintptr_t>(a.shadow) & 7) == 0);
  int64_t done = 0;
  if (vec) {
    const int64_t n4 = a.n / 4;
    float4* p4 = reinterpret_cast<float4*>(a.p);
    float4* g4 = reinterpret_cast<float4*>(a.g);
    float4* m4 = reinterpret_cast<float4*>(a.m);
    float4* v4 = reinterpret_cast<float4*>(a.v);
    for (int64_t i = t0; i < n4; i += stride) {
      float4 p = p4[i], g = g4[i], m = m4[i], v = v4[i];
      adam_elem(p.x, g.x, m.x, v.x, job, sc);
      adam_elem(p.y, g.y, m.y, v.y, job, sc);
      adam_elem(p.z, g.z, m.z, v.z, job, sc);
      adam_elem(p.w, g.w, m.w, v.w, job, sc);
      p4[i] = p;
      m4[i] = m;
      v4[i] = v;
      if (job.zero_grad) g4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
      if (a.shadow) {
        __nv_bfloat162 lo = __floats2bfloat162_rn(p.x, p.y), hi = __floats2bfloat162_rn(p.z, p.w);
        uint2 pk;
        pk.x = *reinterpret_cast<uint32_t*>(&lo);
        pk.y = *reinterpret_cast<uint32_t*>(&hi);
        reinterpret_cast<uint2*>(a.shadow)[i] = pk;
      }
    }
    done = n4 * 4;
  }
  for (int64_t i = done + t0; i < a.n; i += stride) {
    float p = a.p[i], m = a.m[i], v = a.v[i];
    const float g = a.g[i];
    adam_elem(p, g, m, v, job, sc);
    a.p[i] = p;
    a.m[i] = m;
    a.v[i] = v;
    if (job.zero_grad) a.g[i] = 0.f;
    if (a.shadow) a.shadow[i] = __float2bfloat16_rn(p);
  }
}

}  // namespace

cudaError_t launch_adam(const FFAdamParam* prm, int n, float beta1, float beta2, float eps, bool zero_grad,
                        cudaStream_t st, const double* lr_dev, const int64_t* step_dev) {
  for (int b0 = 0; b0 < n; b0 += kMaxAdamParams) {
    AdamJob job = {};
    job.w1 = (float)(1.0 - (double)beta1);
    job.beta2 = beta2;
    job.one_minus_beta2 = (float)(1.0 - (double)beta2);
    job.eps = eps;
    job.zero_grad = zero_grad ? 1 : 0;
    job.log2_beta1 = (float)std::log2((double)beta1);
    job.log2_beta2 = (float)std::log2((double)beta2);
    job.step = step_dev;
    int cnt = 0;
    int64_t most = 0;
    for (int b = b0; b < n && cnt < kMaxAdamParams; ++b) {
      const FFAdamParam& q = prm[b];
      if (q.n <= 0) continue;
      AdamParamDev& a = job.prm[cnt++];
      a.p = q.param;
      a.g = q.grad;
      a.m = q.exp_avg;
      a.v = q.exp_avg_sq;
      a.shadow = static_cast<__nv_bfloat16*>(q.param_bf16);
      a.n = q.n;
      if (step_dev) {
        a.lr = lr_dev + b;
      } else {
        const double bc1 = 1.0 - std::pow((double)beta1, (double)q.step);
        const double bc2 = 1.0 - std::pow((double)beta2, (double)q.step);
        a.neg_step_size = (float)(-(double)q.lr / bc1);
        a.bc2_sqrt = (float)std::sqrt(bc2);
      }
      most = std::max(most, q.n);
    }
    if (cnt == 0) continue;
    const int bx = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(ceil_div(most, 4), kAdamThreads),
                                                               (int64_t)sm_count() * 8));
    adam_kernel<<<dim3(bx, cnt), kAdamThreads, 0, st>>>(job);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}


}  // namespace ffgb
