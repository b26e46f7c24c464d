// Fused field + MLP head: the "faster form" beside the drop-in kernels.
//
// One persistent launch per batch does, for every point, what the reference spreads over
// 6+1 grid_sample launches, a product, two nn.Linear layers, the loss and their backward
// (models/FactorFields.py:11-33, 425-527, 113-159 and autograd):
//
//   gather   per-level mapping + bi/trilinear basis gathers and the coefficient gather
//            (thread per point, channels-last vector loads), basis * coeff in registers
//   forward  H = relu(X W0^T + b0), O = H W1^T on tensor cores: mma.sync m16n8k16 BF16 with
//            FP32 accumulation, 32 points per warp (two 16-row m-tiles)
//   loss     FIT: dO = d(mean L1 or MSE)/dO against the targets; BWD: dO given
//   backward dH = (dO W1) * [H > 0], dX = dH W0 (tensor cores); weight gradients
//            dW0 = dH^T X, dW1^T = H^T dO as MMAs over the warp's 32 points (operands read
//            transposed from shared memory with ldmatrix.trans), reduced into block-private
//            shared-memory accumulators and flushed once per block
//   scatter dL/dbasis = dX * coeff, dL/dcoeff = dX * basis, scattered with float4 / float2
//            atomics into the float32 gradient grids (interpolation weights recomputed)
//
// Level structure is compile-time: basis_dims = [4, 4, 4, 2, 2, 2] (sum 18), which keeps each
// point's 18 basis and 18 coefficient values in registers between the gather and the scatter.
// MLP: in 18 -> 64 (bias, ReLU) -> out <= 32 (no bias), MLPMixer with num_layers = 2.
#include <utility>

#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kHid = 64;
constexpr int kF = 18;  // sum(basis_dims)
constexpr int kNtIn = 3;  // n-tiles of 8 covering the 18 input features
constexpr int kLevelC[6] = {4, 4, 4, 2, 2, 2};
constexpr int kLevelOff[6] = {0, 4, 8, 12, 14, 16};

// Shared-memory row strides (elements), chosen so ldmatrix / 32-bit fragment loads of 8 rows
// fall in 8 distinct 16-byte bank groups.
constexpr int LD_X = 40;    // X tile [32 pts][32 features] bf16
constexpr int LD_H = 72;    // H, dH tiles [32 pts][64] bf16
constexpr int LD_W0 = 40;   // W0 [64 hidden][32 in] bf16
constexpr int LD_W0T = 72;  // W0^T [32 in][64 hidden] bf16
constexpr int LD_W1 = 72;   // W1 [32 out][64 hidden] bf16
constexpr int LD_W1T = 40;  // W1^T [64 hidden][32 out] bf16
constexpr int LD_ACC = 40;  // fp32 accumulators dW0 [64][40], dW1^T [64][40]
constexpr int LD_DX = 33;   // fp32 dX staging [32 pts][33]

template <int OUTT>
constexpr int ld_do() { return OUTT == 1 ? 8 : OUTT * 8 + 8; }

enum { kFwd = 0, kBwd = 1, kFit = 2 };

struct FusedArgs {
  FFField f;
  const void* basis;
  const void* coeff;
  const float* w0;  // [64, 18]
  const float* b0;  // [64]
  const float* w1;  // [out, 64]
  int out_dim;
  const float* x;
  int64_t n;
  float* out;             // kFwd: [n, out]
  const float* grad_out;  // kBwd: [n, out]
  const float* target;    // kFit: [n, out]
  int loss_kind;
  float loss_scale;
  float* loss_sum;
  float* grad_basis;
  float* grad_coeff;
  float* grad_w0;
  float* grad_b0;
  float* grad_w1;
};

// ---- PTX wrappers ------------------------------------------------------------------------

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ void ldsm_x4(uint32_t* r, const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t* r, const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(a));
}

__device__ __forceinline__ void ldsm_x2_t(uint32_t* r, const void* p) {
  const uint32_t a = (uint32_t)__cvta_generic_to_shared(p);
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(a));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ uint32_t lds32(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void sts32(__nv_bfloat16* p, uint32_t v) { *reinterpret_cast<uint32_t*>(p) = v; }

__device__ __forceinline__ bool bf16_lo_pos(uint32_t v) { return __uint_as_float(v << 16) > 0.f; }
__device__ __forceinline__ bool bf16_hi_pos(uint32_t v) { return __uint_as_float(v & 0xffff0000u) > 0.f; }

template <typename Fn, int... Ls>
__device__ __forceinline__ void for_levels(std::integer_sequence<int, Ls...>, Fn&& fn) {
  (fn(std::integral_constant<int, Ls>{}), ...);
}

// ---- shared memory layout -----------------------------------------------------------------

struct Smem {
  __nv_bfloat16 *w0, *w0t, *w1, *w1t;
  float *b0, *acc_w0, *acc_w1t, *acc_b0;
  __nv_bfloat16 *x, *xl, *h, *dh, *dout;  // per warp; xl = low BF16 part of the features
};

template <int MODE, int OUTT>
__host__ __device__ constexpr int64_t smem_bytes() {
  int64_t b = 0;
  b += 64 * LD_W0 * 2 + 32 * LD_W0T * 2 + 32 * LD_W1 * 2 + 64 * LD_W1T * 2 + 64 * 4;
  if (MODE != kFwd) b += 2 * 64 * LD_ACC * 4 + 64 * 4;
  b += (int64_t)kWarps * 2 * 32 * LD_X * 2;
  if (MODE != kFwd) b += (int64_t)kWarps * (2 * 32 * LD_H * 2 + 32 * ld_do<OUTT>() * 2);
  return b;
}

template <int MODE, int OUTT>
__device__ __forceinline__ Smem carve(unsigned char* base, int warp) {
  Smem s;
  unsigned char* p = base;
  auto take = [&](int64_t bytes) { unsigned char* r = p; p += (bytes + 15) & ~int64_t(15); return r; };
  s.w0 = (__nv_bfloat16*)take(64 * LD_W0 * 2);
  s.w0t = (__nv_bfloat16*)take(32 * LD_W0T * 2);
  s.w1 = (__nv_bfloat16*)take(32 * LD_W1 * 2);
  s.w1t = (__nv_bfloat16*)take(64 * LD_W1T * 2);
  s.b0 = (float*)take(64 * 4);
  s.acc_w0 = s.acc_w1t = s.acc_b0 = nullptr;
  if (MODE != kFwd) {
    s.acc_w0 = (float*)take(64 * LD_ACC * 4);
    s.acc_w1t = (float*)take(64 * LD_ACC * 4);
    s.acc_b0 = (float*)take(64 * 4);
  }
  unsigned char* xs = take((int64_t)kWarps * 32 * LD_X * 2);
  unsigned char* xls = take((int64_t)kWarps * 32 * LD_X * 2);
  s.x = (__nv_bfloat16*)xs + warp * 32 * LD_X;
  s.xl = (__nv_bfloat16*)xls + warp * 32 * LD_X;
  s.h = s.dh = s.dout = nullptr;
  if (MODE != kFwd) {
    unsigned char* hs = take((int64_t)kWarps * 32 * LD_H * 2);
    unsigned char* dhs = take((int64_t)kWarps * 32 * LD_H * 2);
    unsigned char* ds = take((int64_t)kWarps * 32 * ld_do<OUTT>() * 2);
    s.h = (__nv_bfloat16*)hs + warp * 32 * LD_H;
    s.dh = (__nv_bfloat16*)dhs + warp * 32 * LD_H;
    s.dout = (__nv_bfloat16*)ds + warp * 32 * ld_do<OUTT>();
  }
  return s;
}

// ---- the kernel -------------------------------------------------------------------------

template <int MODE, int BD, int CD, int OUTT, typename T>
__global__ void __launch_bounds__(kThreads) fused_field_mlp_kernel(const FusedArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const Smem s = carve<MODE, OUTT>(smem_raw, warp);
  const FFField& f = a.f;
  const int out = a.out_dim;
  const T* basis = static_cast<const T*>(a.basis);
  const T* coeff = static_cast<const T*>(a.coeff);

  // stage the MLP weights as BF16 in both orientations; zero the accumulators
  for (int e = tid; e < 64 * 32; e += kThreads) {
    const int j = e >> 5, k = e & 31;
    const __nv_bfloat16 v = __float2bfloat16_rn(k < kF ? a.w0[j * kF + k] : 0.f);
    s.w0[j * LD_W0 + k] = v;
    s.w0t[k * LD_W0T + j] = v;
  }
  for (int e = tid; e < 32 * 64; e += kThreads) {
    const int o = e >> 6, h = e & 63;
    const __nv_bfloat16 v = __float2bfloat16_rn(o < out ? a.w1[o * kHid + h] : 0.f);
    s.w1[o * LD_W1 + h] = v;
    s.w1t[h * LD_W1T + o] = v;
  }
  for (int j = tid; j < 64; j += kThreads) s.b0[j] = a.b0[j];
  if (MODE != kFwd) {
    for (int e = tid; e < 64 * LD_ACC; e += kThreads) {
      s.acc_w0[e] = 0.f;
      s.acc_w1t[e] = 0.f;
    }
    for (int j = tid; j < 64; j += kThreads) s.acc_b0[j] = 0.f;
  }
  __syncthreads();

  float loss_acc = 0.f;
  float db0[8][2];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) db0[nt][0] = db0[nt][1] = 0.f;

  const int64_t stride_pts = (int64_t)gridDim.x * kWarps * 32;
  for (int64_t base = ((int64_t)blockIdx.x * kWarps + warp) * 32; base < a.n; base += stride_pts) {
    const int64_t i = base + lane;
    const bool valid = i < a.n;
    float bv[kF], cv[kF];
    float p[CD];
    // ---------------- gather ----------------
    if (valid) {
#pragma unroll
      for (int k = 0; k < CD; ++k) p[k] = a.x[i * CD + k];
      Corners<CD> cc;
      coeff_corners<CD>(f, p, cc);
      for_levels(std::make_integer_sequence<int, 6>{}, [&](auto lc) {
        constexpr int l = decltype(lc)::value;
        constexpr int C = kLevelC[l], OFF = kLevelOff[l];
        Corners<BD> bc;
        basis_corners<BD>(f, l, p, bc);
        const T* bl = basis + f.level_offset[l];
        gather<C, BD>(bl, f.level_stride[l], 0, bc, bv + OFF);
        gather<C, CD>(coeff, f.coeff_stride, OFF, cc, cv + OFF);
      });
    } else {
#pragma unroll
      for (int k = 0; k < kF; ++k) bv[k] = cv[k] = 0.f;
    }
    // features into this warp's X tiles, row = lane, as a BF16 pair hi + lo (hi = bf16(f),
    // lo = bf16(f - hi)): layer 0 runs on both, so H (and the ReLU mask the backward uses) keeps
    // ~16 mantissa bits of the float32 features instead of BF16's 8.
    {
      __nv_bfloat16* xr = s.x + lane * LD_X;
      __nv_bfloat16* xlr = s.xl + lane * LD_X;
#pragma unroll
      for (int k = 0; k < 32; k += 2) {
        uint32_t hi = 0u, lo = 0u;
        if (k < kF) {
          const float f0 = bv[k] * cv[k], f1 = bv[k + 1] * cv[k + 1];
          hi = pack_bf16(f0, f1);
          lo = pack_bf16(f0 - __uint_as_float(hi << 16), f1 - __uint_as_float(hi & 0xffff0000u));
        }
        sts32(xr + k, hi);
        sts32(xlr + k, lo);
      }
    }
    __syncwarp();

    float dx[2][kNtIn][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      // ---------------- layer 0: H = relu(X W0^T + b0) ----------------
      float hc[8][4];
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const float bl = s.b0[nt * 8 + 2 * t], bh = s.b0[nt * 8 + 2 * t + 1];
        hc[nt][0] = bl; hc[nt][1] = bh; hc[nt][2] = bl; hc[nt][3] = bh;
      }
#pragma unroll
      for (int ks = 0; ks < 2; ++ks) {
        uint32_t af[4], afl[4];
        const int xo = (16 * mt + (lane & 7) + ((lane >> 3) & 1) * 8) * LD_X + 16 * ks + (lane >> 4) * 8;
        ldsm_x4(af, s.x + xo);
        ldsm_x4(afl, s.xl + xo);
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const __nv_bfloat16* wp = s.w0 + (nt * 8 + g) * LD_W0 + 16 * ks + 2 * t;
          const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
          mma_bf16(hc[nt], afl, b0, b1);
          mma_bf16(hc[nt], af, b0, b1);
        }
      }
      uint32_t ha[4][4];  // relu(H) as BF16 A fragments over the 64 hidden units (4 k-steps)
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const float* c0 = hc[2 * ks];
        const float* c1 = hc[2 * ks + 1];
        ha[ks][0] = pack_bf16(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f));
        ha[ks][1] = pack_bf16(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f));
        ha[ks][2] = pack_bf16(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f));
        ha[ks][3] = pack_bf16(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f));
      }
      if (MODE != kFwd) {
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          __nv_bfloat16* r0 = s.h + (16 * mt + g) * LD_H + 16 * ks + 2 * t;
          __nv_bfloat16* r1 = r0 + 8 * LD_H;
          sts32(r0, ha[ks][0]); sts32(r1, ha[ks][1]); sts32(r0 + 8, ha[ks][2]); sts32(r1 + 8, ha[ks][3]);
        }
      }
      // ---------------- layer 1: O = H W1^T ----------------
      float oc[OUTT][4];
#pragma unroll
      for (int nt = 0; nt < OUTT; ++nt) oc[nt][0] = oc[nt][1] = oc[nt][2] = oc[nt][3] = 0.f;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
        for (int nt = 0; nt < OUTT; ++nt) {
          const __nv_bfloat16* wp = s.w1 + (nt * 8 + g) * LD_W1 + 16 * ks + 2 * t;
          mma_bf16(oc[nt], ha[ks], lds32(wp), lds32(wp + 8));
        }
      }
      const int64_t row0 = base + 16 * mt + g, row1 = row0 + 8;
      if (MODE == kFwd) {
#pragma unroll
        for (int nt = 0; nt < OUTT; ++nt) {
          const int c0 = nt * 8 + 2 * t;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            if (c0 + j < out) {
              if (row0 < a.n) a.out[row0 * out + c0 + j] = oc[nt][j];
              if (row1 < a.n) a.out[row1 * out + c0 + j] = oc[nt][2 + j];
            }
          }
        }
        continue;
      }
      // ---------------- dO ----------------
      float dc[OUTT][4];
#pragma unroll
      for (int nt = 0; nt < OUTT; ++nt) {
        const int c0 = nt * 8 + 2 * t;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int64_t row = (q < 2) ? row0 : row1;
          const int col = c0 + (q & 1);
          float d = 0.f;
          if (row < a.n && col < out) {
            if (MODE == kFit) {
              const float err = oc[nt][q] - a.target[row * out + col];
              if (a.loss_kind == FF_LOSS_L1) {
                loss_acc += fabsf(err);
                d = (err > 0.f ? 1.f : (err < 0.f ? -1.f : 0.f)) * a.loss_scale;
              } else {
                loss_acc += err * err;
                d = 2.f * err * a.loss_scale;
              }
            } else {
              d = a.grad_out[row * out + col];
            }
          }
          dc[nt][q] = d;
        }
        __nv_bfloat16* d0 = s.dout + (16 * mt + g) * ld_do<OUTT>() + c0;
        sts32(d0, pack_bf16(dc[nt][0], dc[nt][1]));
        sts32(d0 + 8 * ld_do<OUTT>(), pack_bf16(dc[nt][2], dc[nt][3]));
      }
      // ---------------- dH = (dO W1) * [H > 0] ----------------
      float dh[8][4];
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) dh[nt][0] = dh[nt][1] = dh[nt][2] = dh[nt][3] = 0.f;
#pragma unroll
      for (int ks = 0; ks < (OUTT + 1) / 2; ++ks) {
        uint32_t af[4];
        af[0] = pack_bf16(dc[2 * ks][0], dc[2 * ks][1]);
        af[1] = pack_bf16(dc[2 * ks][2], dc[2 * ks][3]);
        if (2 * ks + 1 < OUTT) {
          af[2] = pack_bf16(dc[2 * ks + 1][0], dc[2 * ks + 1][1]);
          af[3] = pack_bf16(dc[2 * ks + 1][2], dc[2 * ks + 1][3]);
        } else {
          af[2] = af[3] = 0u;
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
          const __nv_bfloat16* wp = s.w1t + (nt * 8 + g) * LD_W1T + 16 * ks + 2 * t;
          mma_bf16(dh[nt], af, lds32(wp), lds32(wp + 8));
        }
      }
      uint32_t dha[4][4];
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const uint32_t hr0 = ha[nt >> 1][(nt & 1) * 2], hr1 = ha[nt >> 1][(nt & 1) * 2 + 1];
        if (!bf16_lo_pos(hr0)) dh[nt][0] = 0.f;
        if (!bf16_hi_pos(hr0)) dh[nt][1] = 0.f;
        if (!bf16_lo_pos(hr1)) dh[nt][2] = 0.f;
        if (!bf16_hi_pos(hr1)) dh[nt][3] = 0.f;
        db0[nt][0] += dh[nt][0] + dh[nt][2];
        db0[nt][1] += dh[nt][1] + dh[nt][3];
      }
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        dha[ks][0] = pack_bf16(dh[2 * ks][0], dh[2 * ks][1]);
        dha[ks][1] = pack_bf16(dh[2 * ks][2], dh[2 * ks][3]);
        dha[ks][2] = pack_bf16(dh[2 * ks + 1][0], dh[2 * ks + 1][1]);
        dha[ks][3] = pack_bf16(dh[2 * ks + 1][2], dh[2 * ks + 1][3]);
        __nv_bfloat16* r0 = s.dh + (16 * mt + g) * LD_H + 16 * ks + 2 * t;
        __nv_bfloat16* r1 = r0 + 8 * LD_H;
        sts32(r0, dha[ks][0]); sts32(r1, dha[ks][1]); sts32(r0 + 8, dha[ks][2]); sts32(r1 + 8, dha[ks][3]);
      }
      // ---------------- dX = dH W0 ----------------
#pragma unroll
      for (int nt = 0; nt < kNtIn; ++nt) dx[mt][nt][0] = dx[mt][nt][1] = dx[mt][nt][2] = dx[mt][nt][3] = 0.f;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
#pragma unroll
        for (int nt = 0; nt < kNtIn; ++nt) {
          const __nv_bfloat16* wp = s.w0t + (nt * 8 + g) * LD_W0T + 16 * ks + 2 * t;
          mma_bf16(dx[mt][nt], dha[ks], lds32(wp), lds32(wp + 8));
        }
      }
    }
    if (MODE == kFwd) {
      __syncwarp();
      continue;
    }
    __syncwarp();
    // ---------------- weight gradients over the warp's 32 points ----------------
    // dW0[64 x 24] += dH^T X     (A = dH^T via ldmatrix.trans, B = X via ldmatrix.trans)
#pragma unroll
    for (int mh = 0; mh < 4; ++mh) {
      float acc[kNtIn][4];
#pragma unroll
      for (int nt = 0; nt < kNtIn; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
      for (int kp = 0; kp < 2; ++kp) {
        uint32_t af[4], bf[4], bf2[2];
        ldsm_x4_t(af, s.dh + (16 * kp + (lane & 7) + (lane >> 4) * 8) * LD_H + 16 * mh + ((lane >> 3) & 1) * 8);
        ldsm_x4_t(bf, s.x + (16 * kp + (lane & 7) + ((lane >> 3) & 1) * 8) * LD_X + (lane >> 4) * 8);
        ldsm_x2_t(bf2, s.x + (16 * kp + (lane & 7) + ((lane >> 3) & 1) * 8) * LD_X + 16);
        mma_bf16(acc[0], af, bf[0], bf[1]);
        mma_bf16(acc[1], af, bf[2], bf[3]);
        mma_bf16(acc[2], af, bf2[0], bf2[1]);
      }
#pragma unroll
      for (int nt = 0; nt < kNtIn; ++nt) {
        float* r0 = s.acc_w0 + (16 * mh + g) * LD_ACC + nt * 8 + 2 * t;
        atomicAdd(r0, acc[nt][0]);
        atomicAdd(r0 + 1, acc[nt][1]);
        atomicAdd(r0 + 8 * LD_ACC, acc[nt][2]);
        atomicAdd(r0 + 8 * LD_ACC + 1, acc[nt][3]);
      }
    }
    // dW1^T[64 x 8*OUTT] += H^T dO
#pragma unroll
    for (int mh = 0; mh < 4; ++mh) {
      float acc[OUTT][4];
#pragma unroll
      for (int nt = 0; nt < OUTT; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
      for (int kp = 0; kp < 2; ++kp) {
        uint32_t af[4];
        ldsm_x4_t(af, s.h + (16 * kp + (lane & 7) + (lane >> 4) * 8) * LD_H + 16 * mh + ((lane >> 3) & 1) * 8);
#pragma unroll
        for (int nt = 0; nt < OUTT; ++nt) {
          uint32_t bf[2];
          ldsm_x2_t(bf, s.dout + (16 * kp + (lane & 7) + ((lane >> 3) & 1) * 8) * ld_do<OUTT>() + nt * 8);
          mma_bf16(acc[nt], af, bf[0], bf[1]);
        }
      }
#pragma unroll
      for (int nt = 0; nt < OUTT; ++nt) {
        float* r0 = s.acc_w1t + (16 * mh + g) * LD_ACC + nt * 8 + 2 * t;
        atomicAdd(r0, acc[nt][0]);
        atomicAdd(r0 + 1, acc[nt][1]);
        atomicAdd(r0 + 8 * LD_ACC, acc[nt][2]);
        atomicAdd(r0 + 8 * LD_ACC + 1, acc[nt][3]);
      }
    }
    __syncwarp();
    // ---------------- scatter dL/dbasis, dL/dcoeff ----------------
    float* dxs = reinterpret_cast<float*>(s.h);  // H tile is free now: stage dX [32][LD_DX] fp32
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
      for (int nt = 0; nt < kNtIn; ++nt) {
        float* r0 = dxs + (16 * mt + g) * LD_DX + nt * 8 + 2 * t;
        r0[0] = dx[mt][nt][0];
        r0[1] = dx[mt][nt][1];
        r0[8 * LD_DX] = dx[mt][nt][2];
        r0[8 * LD_DX + 1] = dx[mt][nt][3];
      }
    }
    __syncwarp();
    if (valid) {
      float gf[kF];
#pragma unroll
      for (int k = 0; k < kF; ++k) gf[k] = dxs[lane * LD_DX + k];
      Corners<CD> cc;
      coeff_corners<CD>(f, p, cc);
      for_levels(std::make_integer_sequence<int, 6>{}, [&](auto lc) {
        constexpr int l = decltype(lc)::value;
        constexpr int C = kLevelC[l], OFF = kLevelOff[l];
        float gb[C], gc[C];
#pragma unroll
        for (int v = 0; v < C; ++v) {
          gb[v] = gf[OFF + v] * cv[OFF + v];
          gc[v] = gf[OFF + v] * bv[OFF + v];
        }
        Corners<BD> bc;
        basis_corners<BD>(f, l, p, bc);
        scatter<C, BD>(a.grad_basis + f.level_offset[l], f.level_stride[l], 0, bc, gb);
        scatter<C, CD>(a.grad_coeff, f.coeff_stride, OFF, cc, gc);
      });
    }
    __syncwarp();
  }

  if (MODE == kFwd) return;
  // loss partial sums
  if (MODE == kFit) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
    if (lane == 0 && a.loss_sum) atomicAdd(a.loss_sum, loss_acc);
  }
  // bias gradient: reduce the per-lane column sums over g (lanes sharing t)
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      float v = db0[nt][j];
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 8);
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      if (g == 0) atomicAdd(s.acc_b0 + nt * 8 + 2 * t + j, v);
    }
  }
  __syncthreads();
  for (int e = tid; e < 64 * kF; e += kThreads) {
    const int j = e / kF, k = e % kF;
    if (a.grad_w0) atomicAdd(a.grad_w0 + e, s.acc_w0[j * LD_ACC + k]);
  }
  for (int e = tid; e < out * 64; e += kThreads) {
    const int o = e >> 6, h = e & 63;
    if (a.grad_w1) atomicAdd(a.grad_w1 + e, s.acc_w1t[h * LD_ACC + o]);
  }
  for (int j = tid; j < 64; j += kThreads)
    if (a.grad_b0) atomicAdd(a.grad_b0 + j, s.acc_b0[j]);
}

template <int MODE, int BD, int CD, int OUTT, typename T>
cudaError_t launch_one(const FusedArgs& a, cudaStream_t st) {
  constexpr int64_t smem = smem_bytes<MODE, OUTT>();
  auto kern = fused_field_mlp_kernel<MODE, BD, CD, OUTT, T>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 1;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
  if (e != cudaSuccess || per_sm < 1) per_sm = 1;
  const int64_t tiles = ceil_div(a.n, kThreads);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count() * per_sm));
  kern<<<blocks, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

template <int MODE, int OUTT, typename T>
cudaError_t dispatch_dims(const FusedArgs& a, cudaStream_t st) {
  const FFField& f = a.f;
  if (f.basis_dim == 2 && f.coord_dim == 2) return launch_one<MODE, 2, 2, OUTT, T>(a, st);
  if (f.basis_dim == 3 && f.coord_dim == 3) return launch_one<MODE, 3, 3, OUTT, T>(a, st);
  if (f.basis_dim == 2 && f.coord_dim == 3) return launch_one<MODE, 2, 3, OUTT, T>(a, st);
  return cudaErrorInvalidValue;
}

template <int MODE>
cudaError_t dispatch(const FusedArgs& a, cudaStream_t st) {
  const bool bf = a.f.param_dtype == FF_BF16;
  const int o = a.out_dim;
  if (o <= 8) return bf ? dispatch_dims<MODE, 1, __nv_bfloat16>(a, st) : dispatch_dims<MODE, 1, float>(a, st);
  if (o <= 16) return bf ? dispatch_dims<MODE, 2, __nv_bfloat16>(a, st) : dispatch_dims<MODE, 2, float>(a, st);
  return bf ? dispatch_dims<MODE, 4, __nv_bfloat16>(a, st) : dispatch_dims<MODE, 4, float>(a, st);
}

FusedArgs make_args(const FFField& f, const void* basis, const void* coeff, const FFMlp& m, const float* x,
                    int64_t n) {
  FusedArgs a = {};
  a.f = f;
  a.basis = basis;
  a.coeff = coeff;
  a.w0 = m.weight[0];
  a.b0 = m.bias[0];
  a.w1 = m.weight[1];
  a.out_dim = m.out_dim;
  a.x = x;
  a.n = n;
  return a;
}

}  // namespace

const char* fused_unsupported(const FFField& f, const FFMlp& m) {
  if (f.n_levels != 6) return "the fused path needs 6 basis levels with basis_dims [4,4,4,2,2,2]";
  for (int l = 0; l < 6; ++l)
    if (f.level_channels[l] != kLevelC[l] || f.level_vec[l] != kLevelC[l] || f.level_stride[l] != kLevelC[l])
      return "the fused path needs basis_dims [4,4,4,2,2,2] stored unpadded";
  if (f.n_feat != kF) return "the fused path needs 18 features";
  if (m.n_layers != 2 || m.hidden_dim != kHid || m.in_dim != kF)
    return "the fused path needs an MLPMixer with num_layers=2, hidden_dim=64, in_dim=18";
  if (m.out_dim < 1 || m.out_dim > 32) return "the fused path needs 1 <= out_dim <= 32";
  if (!m.bias[0] || m.bias[1]) return "the fused path needs a bias on layer 0 and none on layer 1 (MLPMixer)";
  return nullptr;
}

cudaError_t launch_fused_forward(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                 const float* x, int64_t n, float* out, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, x, n);
  a.out = out;
  return dispatch<kFwd>(a, st);
}

cudaError_t launch_fused_backward(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                  const float* x, int64_t n, const float* grad_out, float* grad_basis,
                                  float* grad_coeff, const FFMlpGrad& g, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, x, n);
  a.grad_out = grad_out;
  a.grad_basis = grad_basis;
  a.grad_coeff = grad_coeff;
  a.grad_w0 = g.weight[0];
  a.grad_b0 = g.bias[0];
  a.grad_w1 = g.weight[1];
  return dispatch<kBwd>(a, st);
}

cudaError_t launch_fused_fit(const FFField& f, const void* basis, const void* coeff, const FFMlp& m, const float* x,
                             const float* target, int64_t n, int loss_kind, float loss_scale, float* loss_sum,
                             float* grad_basis, float* grad_coeff, const FFMlpGrad& g, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, x, n);
  a.target = target;
  a.loss_kind = loss_kind;
  a.loss_scale = loss_scale;
  a.loss_sum = loss_sum;
  a.grad_basis = grad_basis;
  a.grad_coeff = grad_coeff;
  a.grad_w0 = g.weight[0];
  a.grad_b0 = g.bias[0];
  a.grad_w1 = g.weight[1];
  return dispatch<kFit>(a, st);
}

}  // namespace ffgb
