// Fused field + MLP head: the "faster form" beside the drop-in kernels. This header holds the
// kernel template; fused_kernels.cu (forward), fused_bwd_kernels.cu, fused_fit_kernels.cu and
// fused_fit_binned_kernels.cu instantiate one mode each, so that they compile in parallel.
//
// One persistent launch per batch does, for every point, what the reference spreads over
// 6+1 grid_sample launches, a product, two nn.Linear layers, the loss and their backward
// (models/FactorFields.py:11-33, 425-527, 113-159 and autograd):
//
//   gather   division-free per-level mapping, bi/trilinear basis gathers (one vector load per
//            corner and level) and the 18-channel coefficient gather (16-byte loads), in a
//            thread-per-point layout; basis * coeff -> a float32 feature tile in shared memory
//   forward  H = relu(X W0^T + b0), O = H W1^T on tensor cores: mma.sync m16n8k16 BF16 with
//            FP32 accumulation, 32 points per warp. X enters layer 0 as a BF16 pair hi + lo
//            (two MMAs) so H and the ReLU mask keep ~16 mantissa bits of the float32 features.
//   loss     FIT: dO = d(mean L1 or MSE)/dO against the targets; BWD: dO given
//   backward dH = (dO W1) * [H > 0], dX = dH W0 on tensor cores. Weight gradients are reduced
//            block-wide: after a barrier each warp computes its 16-row slice of
//            dW0 = dH^T [X | 1] over the block's 128 points (ldmatrix.trans operands), keeping
//            the slice in registers for the whole launch; the constant-1 column yields the
//            bias gradient. dW1 comes from registers when out_dim == 1, else from a second
//            block-wide MMA over H^T dO; then dH^T is not stored but recomputed in the
//            block-wide phase as (W1^T dO^T) [H^T > 0] from the dO and H tiles (one tile less of
//            shared memory: 3 blocks per SM with the 28-wide head). One global atomic per weight
//            entry per block at exit.
//   scatter dL/dbasis = dX * coeff, dL/dcoeff = dX * basis with float4 / float2 atomics into
//            the float32 gradient grids (interpolation weights recomputed, never stored).
//            Binned 2-D fits can keep the level-0 basis gradients (<= 32^2 cells x 4 channels)
//            block-private in shared memory instead: shared-memory atomics per point and one
//            float4 atomic per touched cell when the block ends (FF_FIT_LEVEL0_SHARED).
//
// Level structure is compile-time: basis_dims = [4, 4, 4, 2, 2, 2] (sum 18), which keeps each
// point's 18 basis and 18 coefficient values in registers between the gather and the scatter.
// MLP: in 18 -> 64 (bias, ReLU) -> out <= 32 (no bias): MLPMixer with num_layers = 2.
#pragma once

#include <atomic>
#include <type_traits>
#include <utility>

#include "composite_common.cuh"
#include "ff_common.cuh"
#include "ff_internal.h"
#include "mma_util.cuh"

namespace ffgb {

namespace {

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * 32;
constexpr int kTile = kThreads;  // points per block iteration
constexpr int kHid = 64;
constexpr int kF = 18;    // sum(basis_dims)
constexpr int kNtIn = 3;  // n-tiles of 8 covering the 18 input features (+ the constant-1 column)
constexpr int kLevelC[6] = {4, 4, 4, 2, 2, 2};
constexpr int kLevelOff[6] = {0, 4, 8, 12, 14, 16};

// Shared-memory row strides (elements).
constexpr int LD_XF = 20;   // float32 feature tile [32 pts][20]: 18 features, 1.0, 0
constexpr int LD_H = 72;    // BF16 H / dH tiles [32 pts][64]
// Row strides of 40 keep the 32-bit fragment loads bank-conflict free. (With the 28-wide head
// the backward fits 2 blocks per SM; a stride of 36 would fit 3, but measured slower: the
// third block's shared memory is taken from the L1 that the grid gathers hit.)
constexpr int LD_W0 = 40;   // W0 [64 hidden][32 in] BF16
constexpr int LD_W0T = 72;  // W0^T [32 in][64 hidden]
constexpr int LD_W1 = 72;   // W1 [32 out][64 hidden]
constexpr int LD_W1T = 40;  // W1^T [64 hidden][32 out]

template <int OUTT>
constexpr int ld_do() { return OUTT == 2 ? 24 : 40; }

// kFitBinned: kFit on a batch binned by coefficient cell (fit_bin_kernels.cu); only the
// coefficient scatter differs (segment-cooperative, see coop_coeff_scatter).
// kRender: kFwd on rays of exactly nf samples each (ray-major points), the outputs composited in
// the epilogue instead of written out (see the render epilogue below).
enum { kFwd = 0, kBwd = 1, kFit = 2, kFitBinned = 3, kRender = 4 };

template <int MODE>
constexpr bool is_fit() { return MODE == kFit || MODE == kFitBinned; }

template <int MODE>
constexpr bool is_fwd() { return MODE == kFwd || MODE == kRender; }

constexpr int LD_OUT = 29;  // kRender: float32 output tile [32 samples][29] per warp (odd: conflict-free rows)
constexpr int kPartStride = 8;  // kRender: per-warp chunk partials (product, acc, depth, rgb) in shared memory

struct FusedArgs {
  FFField f;
  const void* basis;
  const void* coeff;
  const float* w0;  // [64, 18]
  const float* b0;  // [64]
  const float* w1;  // [out, 64]
  int out_dim;
  const float* x;
  int64_t x_stride;  // floats between consecutive points' coordinates (coord_dim, or the packed row)
  int64_t n;
  const int64_t* n_dev;  // optional device count: the points processed are min(n, *n_dev)
  float* out;             // kFwd: [n, out]
  const float* grad_out;  // kBwd: [n, out]
  const float* target;    // kFit: [n, out] rows t_stride floats apart
  int64_t t_stride;
  int packed_rows;  // fits, coord_dim 3, out_dim 1: x holds 16-byte-aligned rows (x, y, z, target)
  int loss_kind;
  float loss_scale;
  float* loss_sum;
  float loss_mul;  // the loss accumulates loss_mul * sum (1, or loss_scale for the mean)
  float* grad_basis;
  float* grad_coeff;
  float* grad_w0;
  float* grad_b0;
  float* grad_w1;
  int level0_shared;  // binned 2-D fits: level-0 basis gradients accumulated in shared memory
  int programmatic;   // binned fits launched right after their row permutation: start during it
  // kRender: the points are the samples of rays of exactly nf samples (32, 64 or 128), ray r at
  // rows [r nf, (r + 1) nf); rd's density and colour rules, each sample's (z, dist) in zd
  FFRender rd;
  const float* rays;  // [n / nf, 6]
  const float* zd;    // [n, 2]
  int nf;
  float* rgb;    // [n / nf, 3]
  float* depth;  // [n / nf] or NULL
};

// Level-0 gradients in shared memory: at most this many float32 values (32^2 cells x 4 channels).
constexpr int kL0Floats = 4096;

// A-fragment register pair (hi, lo) for two consecutive float32 features of the X tile;
// columns at or past LD_XF read as zero.
__device__ __forceinline__ void x_pair(const float* xf, int row, int col, uint32_t& hi, uint32_t& lo) {
  if (col < LD_XF) {
    const float2 v = *reinterpret_cast<const float2*>(xf + row * LD_XF + col);
    hi = pack_bf16(v.x, v.y);
    lo = pack_bf16(v.x - bf_lo(hi), v.y - bf_hi(hi));
  } else {
    hi = lo = 0u;
  }
}

template <typename Fn, int... Ls>
__device__ __forceinline__ void for_levels(std::integer_sequence<int, Ls...>, Fn&& fn) {
  (fn(std::integral_constant<int, Ls>{}), ...);
}

// ---- shared memory layout -----------------------------------------------------------------

struct Smem {
  __nv_bfloat16 *w0, *w0t, *w1, *w1t;
  float* b0;
  float* xf;            // [kWarps][32][LD_XF]
  __nv_bfloat16* dh;    // [kWarps][32][LD_H]        (out_dim == 1)
  __nv_bfloat16* h;     // [kWarps][32][LD_H]        (out_dim > 1)
  __nv_bfloat16* dout;  // [kWarps][32][ld_do]       (out_dim > 1)
  float* g0;            // [kL0Floats] level-0 basis gradients (level0-shared variant)
  float* ob;            // kRender: [kWarps][32][LD_OUT] MLP outputs
  float* part;          // kRender: [kWarps][kPartStride] chunk partials
};

template <int MODE, int OUTT, bool L0S = false>
__host__ __device__ constexpr int64_t smem_bytes() {
  int64_t b = 64 * LD_W0 * 2 + 32 * LD_W0T * 2 + 32 * LD_W1 * 2 + 64 * LD_W1T * 2 + 64 * 4;
  b += (int64_t)kWarps * 32 * LD_XF * 4;
  if (!is_fwd<MODE>() && OUTT == 1) b += (int64_t)kWarps * 32 * LD_H * 2;                  // dH
  if (!is_fwd<MODE>() && OUTT > 1) b += (int64_t)kWarps * 32 * (LD_H + ld_do<OUTT>()) * 2;  // H, dO
  if (L0S) b += (int64_t)kL0Floats * 4;
  if (MODE == kRender) b += (int64_t)kWarps * 32 * LD_OUT * 4 + (int64_t)kWarps * kPartStride * 4;
  return b;
}

template <int MODE, int OUTT, bool L0S = false>
__device__ __forceinline__ Smem carve(unsigned char* base) {
  Smem s;
  unsigned char* p = base;
  auto take = [&](int64_t bytes) { unsigned char* r = p; p += (bytes + 15) & ~int64_t(15); return r; };
  s.w0 = (__nv_bfloat16*)take(64 * LD_W0 * 2);
  s.w0t = (__nv_bfloat16*)take(32 * LD_W0T * 2);
  s.w1 = (__nv_bfloat16*)take(32 * LD_W1 * 2);
  s.w1t = (__nv_bfloat16*)take(64 * LD_W1T * 2);
  s.b0 = (float*)take(64 * 4);
  s.xf = (float*)take((int64_t)kWarps * 32 * LD_XF * 4);
  s.dh = s.h = s.dout = nullptr;
  if (!is_fwd<MODE>() && OUTT == 1) s.dh = (__nv_bfloat16*)take((int64_t)kWarps * 32 * LD_H * 2);
  if (!is_fwd<MODE>() && OUTT > 1) {
    s.h = (__nv_bfloat16*)take((int64_t)kWarps * 32 * LD_H * 2);
    s.dout = (__nv_bfloat16*)take((int64_t)kWarps * 32 * ld_do<OUTT>() * 2);
  }
  s.g0 = L0S ? (float*)take((int64_t)kL0Floats * 4) : nullptr;
  s.ob = s.part = nullptr;
  if (MODE == kRender) {
    s.ob = (float*)take((int64_t)kWarps * 32 * LD_OUT * 4);
    s.part = (float*)take((int64_t)kWarps * kPartStride * 4);
  }
  return s;
}

// Level-0 basis gradients (4 channels) of one point into the block's shared-memory copy; the
// corner set lies inside the level (basis_corners_fast), so every index is below the level's
// cell count.
template <int D>
__device__ __forceinline__ void scatter_shared4(float* g0, const Corners<D>& cn, const float* g) {
#pragma unroll
  for (int k = 0; k < Corners<D>::K; ++k) {
    if (cn.w[k] != 0.f) {
      float* p = g0 + cn.idx[k] * 4;
#pragma unroll
      for (int v = 0; v < 4; ++v) atomicAdd(p + v, g[v] * cn.w[k]);
    }
  }
}

// ---- segment-cooperative coefficient scatter (binned batches) ----------------------------
// Lanes holding points of the same coefficient cell (equal key = low-corner index, adjacent
// after binning) form a segment; all of them scatter to the same corners. Lane r of a segment
// of length L sums corners r, r + L, ... over the segment's members (their 18 coefficient
// gradients and corner weights staged in shared memory) and issues one set of float4/float2
// atomics per corner, so a cell's corners take one atomic per segment instead of one per point.
// On an unbinned batch every segment has length 1 and this is the plain per-point scatter.
// gs: this warp's [32][LD_XF] float tile (free: dX has been read), ws: [32][8] floats.
template <int CD, bool kSkipZero = false>
__device__ __forceinline__ void coop_coeff_scatter(float* __restrict__ grad, int stride, const Corners<CD>& cc,
                                                   const float* gc, bool valid, float* gs, float* ws, int lane) {
  constexpr int K = Corners<CD>::K;
  const int key = valid ? cc.idx[0] : (int)(0x80000000u | (unsigned)lane);  // invalid lanes: own segments
  __syncwarp();  // every lane has read its dX row
  {
    float* row = gs + lane * LD_XF;
#pragma unroll
    for (int k = 0; k < 16; k += 4) *reinterpret_cast<float4*>(row + k) = make_float4(gc[k], gc[k + 1], gc[k + 2], gc[k + 3]);
    *reinterpret_cast<float2*>(row + 16) = make_float2(gc[16], gc[17]);
#pragma unroll
    for (int b = 0; b < K; ++b) ws[lane * 8 + b] = cc.w[b];
  }
  const int kprev = __shfl_up_sync(0xffffffffu, key, 1);
  const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || kprev != key);
  const int s0 = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
  const unsigned later = lane == 31 ? 0u : (heads & (0xffffffffu << (lane + 1)));
  const int s1 = later ? __ffs(later) - 1 : 32;
  const int L = s1 - s0;
  __syncwarp();
  float acc[18];
#pragma unroll
  for (int k = 0; k < 18; ++k) acc[k] = 0.f;
  int c = lane - s0, j = 0;
  bool any = !kSkipZero;  // kSkipZero: a corner of zero weight over the whole segment gets no atomics
  while (c < K) {
    const float w = ws[(s0 + j) * 8 + c];
    if (kSkipZero) any |= w != 0.f;
    const float* g = gs + (s0 + j) * LD_XF;
#pragma unroll
    for (int k = 0; k < 16; k += 4) {
      const float4 v = *reinterpret_cast<const float4*>(g + k);
      acc[k] += w * v.x; acc[k + 1] += w * v.y; acc[k + 2] += w * v.z; acc[k + 3] += w * v.w;
    }
    const float2 v2 = *reinterpret_cast<const float2*>(g + 16);
    acc[16] += w * v2.x;
    acc[17] += w * v2.y;
    if (++j == L) {
      int idx = -1;
#pragma unroll
      for (int q = 0; q < K; ++q)
        if (q == c) idx = cc.idx[q];
      if (idx >= 0 && any) {
        float* p = grad + (int64_t)idx * stride;
#pragma unroll
        for (int k = 0; k < 4; ++k)
          atomicAdd(reinterpret_cast<float4*>(p) + k, make_float4(acc[4 * k], acc[4 * k + 1], acc[4 * k + 2], acc[4 * k + 3]));
        atomicAdd(reinterpret_cast<float2*>(p + 16), make_float2(acc[16], acc[17]));
      }
#pragma unroll
      for (int k = 0; k < 18; ++k) acc[k] = 0.f;
      j = 0;
      any = !kSkipZero;
      c += L;
    }
  }
}

// ---- the kernel -------------------------------------------------------------------------

template <int MODE, int BD, int CD, int OUTT, typename T, bool L0S = false>
__global__ void __launch_bounds__(kThreads, is_fwd<MODE>() ? 4 : 3) fused_field_mlp_kernel(const FusedArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
  const Smem s = carve<MODE, OUTT, L0S>(smem_raw);
  const FFField& f = a.f;
  const int out = a.out_dim;
  // fits of one output on packed 16-byte rows (x, y, z, target): one load per point
  constexpr bool kPackedRow = is_fit<MODE>() && OUTT == 1 && CD == 3;
  const T* basis = static_cast<const T*>(a.basis);
  const T* coeff = static_cast<const T*>(a.coeff);
  float* xf = s.xf + warp * 32 * LD_XF;  // this warp's feature tile

  // stage the MLP weights as BF16 in both orientations
  for (int e = tid; e < 64 * 32; e += kThreads) {
    const int j = e >> 5, k = e & 31;
    const __nv_bfloat16 v = __float2bfloat16_rn(k < kF ? a.w0[j * kF + k] : 0.f);
    s.w0[j * LD_W0 + k] = v;
    s.w0t[k * LD_W0T + j] = v;
  }
  for (int e = tid; e < 32 * 64; e += kThreads) {
    const int o = e >> 6, hh = e & 63;
    const __nv_bfloat16 v = __float2bfloat16_rn(o < out ? a.w1[o * kHid + hh] : 0.f);
    s.w1[o * LD_W1 + hh] = v;
    s.w1t[hh * LD_W1T + o] = v;
  }
  for (int j = tid; j < 64; j += kThreads) s.b0[j] = a.b0[j];
  if constexpr (L0S) {
    for (int e = tid; e < kL0Floats / 4; e += kThreads) reinterpret_cast<float4*>(s.g0)[e] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
  // a binned fit launched programmatically starts during the permutation of its rows: the weights
  // and shared memory above do not depend on it (the weights were final before the binning
  // started); the rows and the gradient buffers below do
  if constexpr (MODE == kFitBinned) pdl_wait();
  __syncthreads();

  float loss_acc = 0.f;
  float acc_w0[kNtIn][4];                        // dW0 slice: hidden rows [16*warp, +16), cols 0..23
  float acc_w1[OUTT == 1 ? 8 : 1][2];            // out_dim <= 8: per-lane H * dO partial sums
  float acc_w1t[OUTT > 1 ? OUTT : 1][4];         // out_dim > 8: dW1^T slice
#pragma unroll
  for (int nt = 0; nt < kNtIn; ++nt) acc_w0[nt][0] = acc_w0[nt][1] = acc_w0[nt][2] = acc_w0[nt][3] = 0.f;
#pragma unroll
  for (int nt = 0; nt < (OUTT == 1 ? 8 : 1); ++nt) acc_w1[nt][0] = acc_w1[nt][1] = 0.f;
#pragma unroll
  for (int nt = 0; nt < (OUTT > 1 ? OUTT : 1); ++nt) acc_w1t[nt][0] = acc_w1t[nt][1] = acc_w1t[nt][2] = acc_w1t[nt][3] = 0.f;

  const int64_t n_pts = a.n_dev ? min(a.n, *a.n_dev) : a.n;
  for (int64_t base = (int64_t)blockIdx.x * kTile; base < n_pts; base += (int64_t)gridDim.x * kTile) {
    const int64_t i = base + warp * 32 + lane;
    const bool valid = i < n_pts;
    float bv[kF], cv[kF];
    float p[CD];
    // ---------------- gather ----------------
    float tgt = 0.f;  // packed rows: the point's target, read with its coordinates
    if (valid) {
      if (kPackedRow && a.packed_rows) {
        const float4 r = *reinterpret_cast<const float4*>(a.x + i * 4);
        p[0] = r.x; p[1] = r.y; p[2] = r.z;
        tgt = r.w;
      } else {
#pragma unroll
        for (int k = 0; k < CD; ++k) p[k] = a.x[i * a.x_stride + k];
      }
      Corners<CD> cc;
      coeff_corners<CD, true>(f, p, cc);
      // image sets (2-D basis, coefficient volume over (x, y, image)): half the corners weigh 0
      gather_coeff18<CD, BD == 2 && CD == 3>(coeff, f.coeff_stride, cc, f.coeff_interp != FF_INTERP_NEAREST, cv);
      const bool all_b = f.basis_interp != FF_INTERP_NEAREST;
      for_levels(std::make_integer_sequence<int, 6>{}, [&](auto lc) {
        constexpr int l = decltype(lc)::value;
        Corners<BD> bc;
        basis_corners_fast<BD>(f, l, p, bc);
        constexpr int C = kLevelC[l], OFF = kLevelOff[l];
        gather_inside<C, BD>(basis + f.level_offset[l], f.level_stride[l], bc, all_b, bv + OFF);
      });
    } else {
#pragma unroll
      for (int k = 0; k < kF; ++k) bv[k] = cv[k] = 0.f;
    }
    {
      float* xr = xf + lane * LD_XF;
#pragma unroll
      for (int k = 0; k < kF; k += 2)
        *reinterpret_cast<float2*>(xr + k) = make_float2(bv[k] * cv[k], bv[k + 1] * cv[k + 1]);
      *reinterpret_cast<float2*>(xr + kF) = make_float2(valid ? 1.f : 0.f, 0.f);
    }
    __syncwarp();

    float dx[2][kNtIn][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const int r0 = 16 * mt + g, r1 = r0 + 8;
      // ---------------- layer 0: H = relu(X W0^T + b0), X = hi + lo ----------------
      uint32_t ha[4][4];  // relu(H) as BF16 A fragments over the 64 hidden units (hi part)
      // layer 1 (O = H W1^T) accumulates per half of the hidden units, H as hi + lo
      float oc[OUTT][4];
#pragma unroll
      for (int nt = 0; nt < OUTT; ++nt) oc[nt][0] = oc[nt][1] = oc[nt][2] = oc[nt][3] = 0.f;
#pragma unroll
      for (int half = 0; half < 2; ++half) {  // hidden units [32*half, 32*half + 32)
        float hc[4][4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int nt = 4 * half + q;
          const float bl = s.b0[nt * 8 + 2 * t], bh = s.b0[nt * 8 + 2 * t + 1];
          hc[q][0] = bl; hc[q][1] = bh; hc[q][2] = bl; hc[q][3] = bh;
        }
#pragma unroll
        for (int ks = 0; ks < 2; ++ks) {
          uint32_t ah[4], al[4];
          x_pair(xf, r0, 16 * ks + 2 * t, ah[0], al[0]);
          x_pair(xf, r1, 16 * ks + 2 * t, ah[1], al[1]);
          x_pair(xf, r0, 16 * ks + 2 * t + 8, ah[2], al[2]);
          x_pair(xf, r1, 16 * ks + 2 * t + 8, ah[3], al[3]);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const __nv_bfloat16* wp = s.w0 + ((4 * half + q) * 8 + g) * LD_W0 + 16 * ks + 2 * t;
            const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
            mma_bf16(hc[q], al, b0, b1);
            mma_bf16(hc[q], ah, b0, b1);
          }
        }
#pragma unroll
        for (int kk = 0; kk < 2; ++kk) {
          const float* c0 = hc[2 * kk];
          const float* c1 = hc[2 * kk + 1];
          const int ks = 2 * half + kk;
          uint32_t* hk = ha[ks];
          uint32_t hl[4];
          split_pair(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f), hk[0], hl[0]);
          split_pair(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f), hk[1], hl[1]);
          split_pair(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f), hk[2], hl[2]);
          split_pair(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f), hk[3], hl[3]);
#pragma unroll
          for (int nt = 0; nt < OUTT; ++nt) {
            const __nv_bfloat16* wp = s.w1 + (nt * 8 + g) * LD_W1 + 16 * ks + 2 * t;
            const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
            mma_bf16(oc[nt], hl, b0, b1);
            mma_bf16(oc[nt], hk, b0, b1);
          }
        }
      }
      if constexpr (!is_fwd<MODE>() && OUTT > 1) {
        __nv_bfloat16* hw = s.h + warp * 32 * LD_H;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          __nv_bfloat16* p0 = hw + r0 * LD_H + 16 * ks + 2 * t;
          __nv_bfloat16* p1 = hw + r1 * LD_H + 16 * ks + 2 * t;
          sts32(p0, ha[ks][0]); sts32(p1, ha[ks][1]); sts32(p0 + 8, ha[ks][2]); sts32(p1 + 8, ha[ks][3]);
        }
      }
      const int64_t row0 = base + warp * 32 + r0, row1 = row0 + 8;
      if constexpr (MODE == kFwd) {
#pragma unroll
        for (int nt = 0; nt < OUTT; ++nt) {
          const int c0 = nt * 8 + 2 * t;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            if (c0 + j < out) {
              if (row0 < n_pts) a.out[row0 * out + c0 + j] = oc[nt][j];
              if (row1 < n_pts) a.out[row1 * out + c0 + j] = oc[nt][2 + j];
            }
          }
        }
      } else if constexpr (MODE == kRender) {
        float* ob = s.ob + warp * 32 * LD_OUT;
#pragma unroll
        for (int nt = 0; nt < OUTT; ++nt) {
          const int c0 = nt * 8 + 2 * t;
#pragma unroll
          for (int j = 0; j < 2; ++j) {
            if (c0 + j < out) {
              ob[r0 * LD_OUT + c0 + j] = oc[nt][j];
              ob[r1 * LD_OUT + c0 + j] = oc[nt][2 + j];
            }
          }
        }
      } else {
        // ---------------- dO ----------------
        float tr0 = 0.f, tr1 = 0.f;  // packed rows: targets of rows r0 / r1 from their point lanes
        if constexpr (kPackedRow) {
          tr0 = __shfl_sync(0xffffffffu, tgt, r0);
          tr1 = __shfl_sync(0xffffffffu, tgt, r1);
        }
        float dc[OUTT][4];
#pragma unroll
        for (int nt = 0; nt < OUTT; ++nt) {
          const int c0 = nt * 8 + 2 * t;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int64_t row = (q < 2) ? row0 : row1;
            const int col = c0 + (q & 1);
            float d = 0.f;
            if (row < n_pts && col < out) {
              if constexpr (is_fit<MODE>()) {
                const float tv = (kPackedRow && a.packed_rows) ? ((q < 2) ? tr0 : tr1)
                                                               : a.target[row * a.t_stride + col];
                const float err = oc[nt][q] - tv;
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
        }
        if constexpr (OUTT == 1) {
          // out_dim == 1: dW1[0][j] = sum over points of H[pt][j] * dO[pt]. dO of rows r0 / r1
          // sits in the quad's t == 0 lane; each lane accumulates its 16 hidden columns.
          const float d0 = __shfl_sync(0xffffffffu, dc[0][0], lane & ~3);
          const float d1 = __shfl_sync(0xffffffffu, dc[0][2], lane & ~3);
#pragma unroll
          for (int nt = 0; nt < 8; ++nt) {
            const uint32_t h0 = ha[nt >> 1][(nt & 1) * 2], h1 = ha[nt >> 1][(nt & 1) * 2 + 1];
            acc_w1[nt][0] += bf_lo(h0) * d0 + bf_lo(h1) * d1;
            acc_w1[nt][1] += bf_hi(h0) * d0 + bf_hi(h1) * d1;
          }
        } else {
          __nv_bfloat16* dw = s.dout + warp * 32 * ld_do<OUTT>();
#pragma unroll
          for (int nt = 0; nt < OUTT; ++nt) {
            const int c0 = nt * 8 + 2 * t;
            sts32(dw + r0 * ld_do<OUTT>() + c0, pack_bf16(dc[nt][0], dc[nt][1]));
            sts32(dw + r1 * ld_do<OUTT>() + c0, pack_bf16(dc[nt][2], dc[nt][3]));
          }
        }
        // ---------------- dH = (dO W1) * [H > 0], dX = dH W0 ----------------
        // dO and dH enter their GEMMs as BF16 pairs hi + lo (two MMAs each), so the gradients
        // keep ~16 mantissa bits through the sums over outputs and hidden units.
        __nv_bfloat16* dhw = s.dh + warp * 32 * LD_H;  // out_dim == 1 only (else unused)
#pragma unroll
        for (int nt = 0; nt < kNtIn; ++nt) dx[mt][nt][0] = dx[mt][nt][1] = dx[mt][nt][2] = dx[mt][nt][3] = 0.f;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          float dh[4][4];
#pragma unroll
          for (int q = 0; q < 4; ++q) dh[q][0] = dh[q][1] = dh[q][2] = dh[q][3] = 0.f;
#pragma unroll
          for (int ks = 0; ks < (OUTT + 1) / 2; ++ks) {
            uint32_t af[4], al[4];
            split_pair(dc[2 * ks][0], dc[2 * ks][1], af[0], al[0]);
            split_pair(dc[2 * ks][2], dc[2 * ks][3], af[1], al[1]);
            if (2 * ks + 1 < OUTT) {
              split_pair(dc[2 * ks + 1][0], dc[2 * ks + 1][1], af[2], al[2]);
              split_pair(dc[2 * ks + 1][2], dc[2 * ks + 1][3], af[3], al[3]);
            } else {
              af[2] = af[3] = al[2] = al[3] = 0u;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
              const __nv_bfloat16* wp = s.w1t + ((4 * half + q) * 8 + g) * LD_W1T + 16 * ks + 2 * t;
              const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
              mma_bf16(dh[q], al, b0, b1);
              mma_bf16(dh[q], af, b0, b1);
            }
          }
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int nt = 4 * half + q;
            const uint32_t h0 = ha[nt >> 1][(nt & 1) * 2], h1 = ha[nt >> 1][(nt & 1) * 2 + 1];
            if (!(bf_lo(h0) > 0.f)) dh[q][0] = 0.f;
            if (!(bf_hi(h0) > 0.f)) dh[q][1] = 0.f;
            if (!(bf_lo(h1) > 0.f)) dh[q][2] = 0.f;
            if (!(bf_hi(h1) > 0.f)) dh[q][3] = 0.f;
          }
#pragma unroll
          for (int kk = 0; kk < 2; ++kk) {
            uint32_t d[4], dl[4];
            split_pair(dh[2 * kk][0], dh[2 * kk][1], d[0], dl[0]);
            split_pair(dh[2 * kk][2], dh[2 * kk][3], d[1], dl[1]);
            split_pair(dh[2 * kk + 1][0], dh[2 * kk + 1][1], d[2], dl[2]);
            split_pair(dh[2 * kk + 1][2], dh[2 * kk + 1][3], d[3], dl[3]);
            const int ks = 2 * half + kk;
            if constexpr (OUTT == 1) {
              __nv_bfloat16* p0 = dhw + r0 * LD_H + 16 * ks + 2 * t;
              __nv_bfloat16* p1 = dhw + r1 * LD_H + 16 * ks + 2 * t;
              sts32(p0, d[0]); sts32(p1, d[1]); sts32(p0 + 8, d[2]); sts32(p1 + 8, d[3]);
            }
            // dX += dH[:, 16 ks .. 16 ks + 15] W0[16 ks .. 16 ks + 15, :]
#pragma unroll
            for (int nt = 0; nt < kNtIn; ++nt) {
              const __nv_bfloat16* wp = s.w0t + (nt * 8 + g) * LD_W0T + 16 * ks + 2 * t;
              const uint32_t b0 = lds32(wp), b1 = lds32(wp + 8);
              mma_bf16(dx[mt][nt], dl, b0, b1);
              mma_bf16(dx[mt][nt], d, b0, b1);
            }
          }
        }
      }
    }
    if constexpr (MODE == kFwd) {
      __syncwarp();
      continue;
    } else if constexpr (MODE == kRender) {
      // ---------------- compositing (ff_composite_forward_zd's rules) ----------------
      // Lane j takes sample j of the warp's tile. A ray's nf samples fill nf / 32 consecutive
      // warps of the block (tiles are 128-aligned and nf divides 128); its chunks chain their
      // transmittance through shared memory in chunk order, as the compositing kernel does.
      __syncwarp();
      const int64_t i = base + warp * 32 + lane;
      const bool live = base + warp * 32 < n_pts;  // n_pts is a multiple of nf, hence of 32
      const int wpr = a.nf >> 5;                   // warps per ray
      const int chunk = warp & (wpr - 1);
      const int64_t ray = (base + warp * 32) / a.nf;
      const float* row = s.ob + (warp * 32 + lane) * LD_OUT;
      SampleVals sv = {0.f, 0.f, 0.f, 0.f, 0.f, 1.f};
      float yb[9];
      if (live) {
        const float2 zd = *reinterpret_cast<const float2*>(a.zd + 2 * i);
        sv = sample_vals_at(a.rd, zd.x, zd.y, row[0]);
        const float dir[3] = {a.rays[ray * 6 + 3], a.rays[ray * 6 + 4], a.rays[ray * 6 + 5]};
        sh2_basis(dir, yb);
      }
      float excl;
      const float prod = excl_trans(sv.fac, lane, excl);
      float t_in = 1.f;  // transmittance entering this chunk
      if (wpr > 1) {
        if (lane == 0) s.part[warp * kPartStride] = prod;
        __syncthreads();
        for (int q = warp - chunk; q < warp; ++q) t_in *= s.part[q * kPartStride];
      }
      const float w = live ? sv.alpha * (t_in * excl) : 0.f;
      float acc = w, dep = w * sv.z, col[3] = {0.f, 0.f, 0.f};
      if (live && w > a.rd.weight_thres) {
        float c[3], lin[3];
        sample_rgb(row, yb, c, lin);
        col[0] = w * c[0]; col[1] = w * c[1]; col[2] = w * c[2];
      }
      acc = warp_sum(acc);
      dep = warp_sum(dep);
      col[0] = warp_sum(col[0]); col[1] = warp_sum(col[1]); col[2] = warp_sum(col[2]);
      if (wpr > 1) {
        if (lane == 0) {
          float* pp = s.part + warp * kPartStride;
          pp[1] = acc; pp[2] = dep; pp[3] = col[0]; pp[4] = col[1]; pp[5] = col[2];
        }
        __syncthreads();
        if (chunk == 0) {
          acc = dep = col[0] = col[1] = col[2] = 0.f;
          for (int q = warp; q < warp + wpr; ++q) {
            const float* pp = s.part + q * kPartStride;
            acc += pp[1]; dep += pp[2]; col[0] += pp[3]; col[1] += pp[4]; col[2] += pp[5];
          }
        }
      }
      if (live && chunk == 0 && lane == 0) {
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          float v = col[c];
          if (a.rd.white_bg) v = v + (1.f - acc);
          a.rgb[ray * 3 + c] = fminf(fmaxf(v, 0.f), 1.f);
        }
        if (a.depth) a.depth[ray] = dep;
      }
      if (wpr > 1) __syncthreads();  // the partials are read before the next tile writes them
      continue;
    } else {
      __syncthreads();  // every warp's X and dH (and H, dO) tiles are complete
      // ---------------- block-wide weight gradients ----------------
      // dW0[16*warp + .., 0..23] += dH^T [X | 1] over the block's 128 points: 8 k-steps of 16.
#pragma unroll 2
      for (int kk = 0; kk < 8; ++kk) {
        const int src = kk >> 1, h16 = (kk & 1) * 16;
        const float* xs = s.xf + src * 32 * LD_XF;
        uint32_t af[4];  // dH^T of hidden units 16 warp .. + 15 over the 16 points: an A fragment
        uint32_t ah[4];  // H^T of the same (out_dim > 1)
        if constexpr (OUTT == 1) {
          const __nv_bfloat16* dhs = s.dh + src * 32 * LD_H;
          ldsm_x4_t(af, dhs + (h16 + (lane & 7) + (lane >> 4) * 8) * LD_H + 16 * warp + ((lane >> 3) & 1) * 8);
        } else {
          // no dH tile: dH^T = (W1^T dO^T) [H^T > 0], recomputed here from the dO tile (BF16) and
          // the H tile's mask, so that 3 blocks fit per SM with the 28-wide head
          const __nv_bfloat16* hs = s.h + src * 32 * LD_H;
          ldsm_x4_t(ah, hs + (h16 + (lane & 7) + (lane >> 4) * 8) * LD_H + 16 * warp + ((lane >> 3) & 1) * 8);
          const __nv_bfloat16* ds = s.dout + src * 32 * ld_do<OUTT>();
          float c[2][4];
#pragma unroll
          for (int n2 = 0; n2 < 2; ++n2) c[n2][0] = c[n2][1] = c[n2][2] = c[n2][3] = 0.f;
#pragma unroll
          for (int ks = 0; ks < (OUTT + 1) / 2; ++ks) {  // K = the outputs, 16 per step
            uint32_t a4[4];
            const __nv_bfloat16* wp = s.w1t + (16 * warp + g) * LD_W1T + 16 * ks + 2 * t;
            a4[0] = lds32(wp);
            a4[1] = lds32(wp + 8 * LD_W1T);
            a4[2] = lds32(wp + 8);
            a4[3] = lds32(wp + 8 * LD_W1T + 8);
#pragma unroll
            for (int n2 = 0; n2 < 2; ++n2) {  // points h16 + 8 n2 .. + 7 (B = dO^T, rows of the dO tile)
              const __nv_bfloat16* bp = ds + (h16 + 8 * n2 + g) * ld_do<OUTT>() + 16 * ks + 2 * t;
              mma_bf16(c[n2], a4, lds32(bp), lds32(bp + 8));
            }
          }
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float* cc = c[i >> 1] + 2 * (i & 1);
            af[i] = pack_bf16(bf_lo(ah[i]) > 0.f ? cc[0] : 0.f, bf_hi(ah[i]) > 0.f ? cc[1] : 0.f);
          }
        }
#pragma unroll
        for (int nt = 0; nt < kNtIn; ++nt) {
          const int col = nt * 8 + g;
          uint32_t b0 = 0u, b1 = 0u;
          if (col < LD_XF) {
            b0 = pack_bf16(xs[(h16 + 2 * t) * LD_XF + col], xs[(h16 + 2 * t + 1) * LD_XF + col]);
            b1 = pack_bf16(xs[(h16 + 2 * t + 8) * LD_XF + col], xs[(h16 + 2 * t + 9) * LD_XF + col]);
          }
          mma_bf16(acc_w0[nt], af, b0, b1);
        }
        if constexpr (OUTT > 1) {
          const __nv_bfloat16* ds = s.dout + src * 32 * ld_do<OUTT>();
#pragma unroll
          for (int nt = 0; nt < OUTT; ++nt) {
            uint32_t bf[2];
            ldsm_x2_t(bf, ds + (h16 + (lane & 7) + ((lane >> 3) & 1) * 8) * ld_do<OUTT>() + nt * 8);
            mma_bf16(acc_w1t[nt], ah, bf[0], bf[1]);
          }
        }
      }
      __syncthreads();  // tiles consumed: the feature tile can now hold dX
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
#pragma unroll
        for (int nt = 0; nt < kNtIn; ++nt) {
          const int c0 = nt * 8 + 2 * t;
          if (c0 < kF) {
            *reinterpret_cast<float2*>(xf + (16 * mt + g) * LD_XF + c0) = make_float2(dx[mt][nt][0], dx[mt][nt][1]);
            *reinterpret_cast<float2*>(xf + (16 * mt + g + 8) * LD_XF + c0) = make_float2(dx[mt][nt][2], dx[mt][nt][3]);
          }
        }
      }
      __syncwarp();
      // ---------------- scatter dL/dbasis = dX * coeff, dL/dcoeff = dX * basis ----------------
      // segment-cooperative coefficient scatter: binned fit batches, and the BF16 backward, whose
      // points are ray samples in ray order (consecutive samples share coefficient cells)
      if constexpr (MODE == kFitBinned || (MODE == kBwd && std::is_same<T, __nv_bfloat16>::value)) {
        float gc[kF];
        Corners<CD> cc;
        if (valid) {
          const float* xr = xf + lane * LD_XF;
#pragma unroll
          for (int k = 0; k < kF; ++k) {
            const float gx = xr[k];
            gc[k] = gx * bv[k];
            bv[k] = gx * cv[k];  // bv now holds dL/dbasis
          }
          coeff_corners<CD, true>(f, p, cc);
          for_levels(std::make_integer_sequence<int, 6>{}, [&](auto lc) {
            constexpr int l = decltype(lc)::value;
            Corners<BD> bc;
            basis_corners_fast<BD>(f, l, p, bc);
            constexpr int C = kLevelC[l], OFF = kLevelOff[l];
            if constexpr (L0S && l == 0)
              scatter_shared4<BD>(s.g0, bc, bv + OFF);
            else
              scatter_inside<C, BD>(a.grad_basis + f.level_offset[l], f.level_stride[l], bc, bv + OFF);
          });
        } else {
#pragma unroll
          for (int k = 0; k < kF; ++k) gc[k] = 0.f;
#pragma unroll
          for (int b = 0; b < Corners<CD>::K; ++b) {
            cc.idx[b] = -1;
            cc.w[b] = 0.f;
          }
        }
        // scratch for the segment weights: this warp's dH (out_dim 1) or H tile, both consumed
        coop_coeff_scatter<CD, BD == 2 && CD == 3>(a.grad_coeff, f.coeff_stride, cc, gc, valid, xf,
                               reinterpret_cast<float*>((OUTT == 1 ? s.dh : s.h) + warp * 32 * LD_H), lane);
      } else if (valid) {
        float gc[kF];
        const float* xr = xf + lane * LD_XF;
#pragma unroll
        for (int k = 0; k < kF; ++k) {
          const float gx = xr[k];
          gc[k] = gx * bv[k];
          bv[k] = gx * cv[k];  // bv now holds dL/dbasis
        }
        Corners<CD> cc;
        coeff_corners<CD, true>(f, p, cc);
        scatter_coeff18<CD>(a.grad_coeff, f.coeff_stride, cc, gc);
        for_levels(std::make_integer_sequence<int, 6>{}, [&](auto lc) {
          constexpr int l = decltype(lc)::value;
          Corners<BD> bc;
          basis_corners_fast<BD>(f, l, p, bc);
          constexpr int C = kLevelC[l], OFF = kLevelOff[l];
          if constexpr (L0S && l == 0)
            scatter_shared4<BD>(s.g0, bc, bv + OFF);
          else
            scatter_inside<C, BD>(a.grad_basis + f.level_offset[l], f.level_stride[l], bc, bv + OFF);
        });
      }
      __syncwarp();
    }
  }

  if constexpr (L0S) {
    // the block's level-0 gradients: one float4 atomic per touched cell (every block runs the
    // same number of tile iterations, so all threads reach this barrier)
    __syncthreads();
    const int cells = f.level_reso[0] * f.level_reso[0];
    float4* dst = reinterpret_cast<float4*>(a.grad_basis + f.level_offset[0]);
    for (int e = tid; e < cells; e += kThreads) {
      const float4 v = reinterpret_cast<const float4*>(s.g0)[e];
      if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) atomicAdd(dst + e, v);
    }
  }
  if constexpr (!is_fwd<MODE>()) {
    if constexpr (is_fit<MODE>()) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) loss_acc += __shfl_xor_sync(0xffffffffu, loss_acc, o);
      if (lane == 0 && a.loss_sum) atomicAdd(a.loss_sum, loss_acc * a.loss_mul);
    }
    // dW0 slice (rows 16*warp + g, + 8; cols 8*nt + 2t, + 1): features -> grad_w0, column 18 -> grad_b0
#pragma unroll
    for (int nt = 0; nt < kNtIn; ++nt) {
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int row = 16 * warp + g + (q >= 2 ? 8 : 0);
        const int col = nt * 8 + 2 * t + (q & 1);
        if (col < kF) {
          if (a.grad_w0) atomicAdd(a.grad_w0 + row * kF + col, acc_w0[nt][q]);
        } else if (col == kF) {
          if (a.grad_b0) atomicAdd(a.grad_b0 + row, acc_w0[nt][q]);
        }
      }
    }
    if constexpr (OUTT == 1) {
      // out_dim <= 8 with one n-tile: column 0 accumulated in registers (out_dim == 1)
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          float v = acc_w1[nt][j];
          v += __shfl_xor_sync(0xffffffffu, v, 4);
          v += __shfl_xor_sync(0xffffffffu, v, 8);
          v += __shfl_xor_sync(0xffffffffu, v, 16);
          if (g == 0 && a.grad_w1) atomicAdd(a.grad_w1 + nt * 8 + 2 * t + j, v);
        }
      }
    } else {
#pragma unroll
      for (int nt = 0; nt < OUTT; ++nt) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int hid = 16 * warp + g + (q >= 2 ? 8 : 0);
          const int o = nt * 8 + 2 * t + (q & 1);
          if (o < out && a.grad_w1) atomicAdd(a.grad_w1 + o * kHid + hid, acc_w1t[nt][q]);
        }
      }
    }
  }
}

template <int MODE, int BD, int CD, int OUTT, typename T, bool L0S>
cudaError_t launch_kernel(const FusedArgs& a, cudaStream_t st) {
  constexpr int64_t smem = smem_bytes<MODE, OUTT, L0S>();
  auto kern = fused_field_mlp_kernel<MODE, BD, CD, OUTT, T, L0S>;
  // the shared-memory opt-in and the occupancy query, once per process and device (atomic cache
  // entries: threads racing on the first launch repeat the same idempotent set-up)
  static std::atomic<int> per_sm_cache[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  int per_sm = (dev >= 0 && dev < 64) ? per_sm_cache[dev].load(std::memory_order_relaxed) : 0;
  if (per_sm == 0) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess || per_sm < 1) {
      (void)cudaGetLastError();
      per_sm = 1;
    }
    if (dev >= 0 && dev < 64) per_sm_cache[dev].store(per_sm, std::memory_order_relaxed);
  }
  const int64_t tiles = ceil_div(a.n, kTile);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count() * per_sm));
  if (MODE == kFitBinned && a.programmatic) return launch_pdl(kern, dim3(blocks), dim3(kThreads), (size_t)smem, st, a);
  kern<<<blocks, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

// Level-0 gradients in shared memory: binned BF16 fits of a 2-D basis whose level 0 (4 channels,
// stride 4) has at most kL0Floats / 4 cells.
inline bool level0_fits_shared(const FFField& f) {
  return f.basis_dim == 2 && f.level_stride[0] == 4 && (int64_t)f.level_reso[0] * f.level_reso[0] * 4 <= kL0Floats;
}

template <int MODE, int BD, int CD, int OUTT, typename T>
cudaError_t launch_one(const FusedArgs& a, cudaStream_t st) {
  if constexpr (MODE == kFitBinned && BD == 2 && std::is_same<T, __nv_bfloat16>::value) {
    if (a.level0_shared && level0_fits_shared(a.f)) return launch_kernel<MODE, BD, CD, OUTT, T, true>(a, st);
  }
  return launch_kernel<MODE, BD, CD, OUTT, T, false>(a, st);
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
  if (o == 1) return bf ? dispatch_dims<MODE, 1, __nv_bfloat16>(a, st) : dispatch_dims<MODE, 1, float>(a, st);
  if (o <= 16) return bf ? dispatch_dims<MODE, 2, __nv_bfloat16>(a, st) : dispatch_dims<MODE, 2, float>(a, st);
  return bf ? dispatch_dims<MODE, 4, __nv_bfloat16>(a, st) : dispatch_dims<MODE, 4, float>(a, st);
}

// BF16 grids only (the binned fit; float32 grids take the per-point fit on the binned batch)
template <int MODE>
cudaError_t dispatch_bf16(const FusedArgs& a, cudaStream_t st) {
  const int o = a.out_dim;
  if (o == 1) return dispatch_dims<MODE, 1, __nv_bfloat16>(a, st);
  if (o <= 16) return dispatch_dims<MODE, 2, __nv_bfloat16>(a, st);
  return dispatch_dims<MODE, 4, __nv_bfloat16>(a, st);
}

inline FusedArgs make_args(const FFField& f, const void* basis, const void* coeff, const FFMlp& m, const float* x,
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
  a.x_stride = f.coord_dim;
  a.t_stride = m.out_dim;
  a.loss_mul = 1.f;
  a.n = n;
  return a;
}

}  // namespace

}  // namespace ffgb
