// MLPRender_Fea colour head (models/FactorFields.py:162-203) on the fifth-generation tensor
// cores: tcgen05.mma with 16-bit operands in shared memory and FP32 accumulators in tensor memory.
// Two kernels, each one persistent CTA per SM walking tiles of 128 listed head samples (sample r
// of a tile = TMEM lane r):
//
// head_fwd16_kernel (the forward): FP16 operands, one MMA pass per layer, two tiles in flight
// (512 threads software-pipelined over two tile buffers and their TMEM accumulators: the MMAs of
// one tile run while the CUDA cores work on the other); described above it.
//
// head_tc_kernel (the backward, with the forward recomputed): 512 threads, warp w serves TMEM
// lane quadrant w % 4 (rows 32 (w % 4) .. + 31) and the 32-column slice w / 4 of every 128-wide
// accumulator, so each epilogue is one tcgen05.ld x32 per thread. Per tile, for 3 layers 128
// hidden units wide:
//
//   stage  the tile's feature rows (channels 0..C) and ray directions into shared memory,
//          warp per row (coalesced), through app_idx / app_ray; the loads of the next tile are
//          issued into registers right after, so their latency overlaps this tile's work
//   X   = [feat, dir, PE(feat, 2), PE(dir, 6)]  in shared memory as a BF16 pair X_hi + X_lo
//          (~16 significant bits); a thread builds one row's 8-column chunk (columns decoded at
//          compile time) with one 16-byte store into each of X_hi and X_lo
//   F1  S = X_hi W0^T + X_lo W0^T   (tcgen05, M 128, N 128, K = in_dim padded to 16)
//       H0 = relu(S + b0)           -> shared memory as H0_hi + H0_lo, ReLU mask in registers
//   F2  S = H0_hi W1^T + H0_lo W1^T (N 128, K 128)
//       H1 = relu(S + b1), y = H1 W2^T (row partials of the 4 column slices summed through
//       shared memory), rgb = sigmoid(y)
// and then the backward (nothing is stored between the launches):
//       dy = dL/drgb rgb (1 - rgb), dH1 = (dy W2) [H1 > 0] -> shared memory (BF16)
//   B1  S  = dH1 W1                 (B = W1 read MN-major)
//   B2  dW1 += dH1^T H0_hi          (A = dH1, B = H0, both read MN-major; TMEM-resident over tiles)
//       dH0 = S [H0 > 0]            -> shared memory, over H0_hi (consumed by B2)
//   B3  dW0 += dH0^T X_hi           (TMEM-resident over tiles)
//   B4  S  = dH0 W0                 (the feature-related input columns only)
//       dL/dfeat = the chain rule through the positional encoding: each thread adds its columns'
//       terms to a per-row shared-memory sum, and a warp per row writes the rows out
// dW2 and db1 are warp reduce-scatters into per-lane registers; db0 accumulates in dW0's column
// in_dim, where X holds a constant 1 (W0's column there is zero). At the end each CTA adds its
// dW0 / dW1 (read from TMEM, one row per quadrant thread) and the register sums to the float32
// gradients with one atomic per entry.
//
// The forward operands X and H0 carry ~16 significant bits (two BF16 MMAs each): with one BF16
// rounding, inputs near a ReLU kink land on the other side of it in a fraction of the 128 x 128
// units per tile, and each flip moves that sample's input gradient by a whole term (up to ~20% of
// max |dL/dfeat| on random heads). The backward operands (dH1, dH0) and the weight-gradient
// operands are single BF16 values (~0.2% effect). The positional encoding uses the hardware
// sin/cos (__sincosf; absolute error ~1e-5 at the largest arguments, |x| <= 32 |d|), below the
// resolution of the BF16 pair.
//
// Operands are stored once, in the core-matrix-row layout of tc_util.cuh, and read as K-major or
// MN-major operands as each product needs (transposes cost nothing). Shared memory: W0, W1, X_hi,
// a 64 KB region R that holds X_lo during F1, then H0_hi and H0_lo for F2, then H0_hi and dH1 (the
// row partials of y pass through the second half first), then dH0 and dH1, then the dL/dfeat row
// sums; the staged feature rows, directions and row indices. TMEM columns (backward): [0, S) the
// per-tile accumulator S, then dW1 (128), then dW0 (in_dim padded): at most 512.
// Every wait on an mbarrier has an iteration limit: when it runs out the kernel reports
// FF_ERR_LIMIT through `status`, stops, waits (again with a limit) for its MMAs and frees TMEM.
#include <utility>

#include "ff_common.cuh"
#include "ff_internal.h"
#include "tc_util.cuh"

namespace ffgb {

namespace {

constexpr int kH = 128;          // hidden units of both hidden layers
constexpr int kTile = 128;       // samples per tile = TMEM lanes
constexpr int kThreads = 512;    // 16 warps: lane quadrant w % 4, column slice w / 4
constexpr uint32_t kPolls = 1u << 22;  // mbarrier polls before a wait gives up (MMAs finish in microseconds)

template <int C, int F, int V>
struct Shape {
  static constexpr int IN = 3 + C + 6 * V + 2 * F * C;
  static constexpr int IN_PAD = (IN + 15) / 16 * 16;
  static constexpr int NX = (C + 3 + 2 * F * C + 15) / 16 * 16;  // input columns whose gradient is needed
  static constexpr int S_COLS = NX > 128 ? (NX + 31) / 32 * 32 : 128;
  static constexpr int COL_DW1 = S_COLS;
  static constexpr int COL_DW0 = S_COLS + 128;
  static_assert(COL_DW0 + (IN_PAD + 31) / 32 * 32 <= 512, "tensor-memory budget");
  static_assert(NX <= 256 && IN_PAD <= 256, "MMA N limit");
  static_assert(C + 1 <= 32, "a feature row is staged by one warp");
  static constexpr int FS = (C + 1) | 1;  // staged row stride in floats (odd: rows on distinct banks)
  static constexpr int W0_B = kH * IN_PAD * 2;
  static constexpr int W1_B = kH * kH * 2;
  static constexpr int X_B = kTile * IN_PAD * 2;
  static constexpr int H_B = kTile * kH * 2;
  static constexpr int R_B = X_B > 2 * H_B ? X_B : 2 * H_B;  // X_lo, or H0_hi + H0_lo / dH1
  static constexpr int FEAT_B = kTile * FS * 4;
  static constexpr int DIR_B = kTile * 4 * 4;
  static constexpr int IDX_B = kTile * 4;
  static constexpr int F32_B = 5 * kH * 4;  // W2 [3][128], b0, b1
  static_assert(kTile * 4 * 4 * 4 <= H_B && FEAT_B <= R_B, "aliased buffers fit");
  static_assert((W0_B + W1_B + X_B + R_B + FEAT_B + DIR_B + IDX_B) % 16 == 0, "float4 reads of W2 / b0 / b1");
  static constexpr int smem() { return W0_B + W1_B + X_B + R_B + FEAT_B + DIR_B + IDX_B + F32_B + 64; }
};

struct HeadArgs {
  const float* w[3];
  const float* b[2];
  const float* feat;
  int feat_stride;
  const float* rays;
  const int32_t* app_idx;
  const int32_t* app_ray;
  int64_t n;
  float* rgb_out;          // forward: rows app_idx of [M, 3]
  const float* grad_rgb;   // backward: rows app_idx of [M, 3]
  float* grad_feat;        // backward: channels 1..C of rows app_idx
  float* gw[3];
  float* gb[2];
  int32_t* status;
};

// K-major / MN-major descriptors of a core-matrix-row buffer with `cols` columns: the 16-wide
// K step s of a K-major operand (rows = M or N) starts at column 16 s; of an MN-major operand
// (rows = K) at row 16 s. LBO = the core stride along K, SBO = along M / N.
__device__ __forceinline__ uint64_t desc_k(uint32_t base, int cols, int s) {
  return tc::smem_desc(base + (uint32_t)(s * 2 * 128), 128u, (uint32_t)(cols / 8 * 128));
}
__device__ __forceinline__ uint64_t desc_mn(uint32_t base, int cols, int s) {
  return tc::smem_desc(base + (uint32_t)(s * 2 * (cols / 8) * 128), (uint32_t)(cols / 8 * 128), 128u);
}

__device__ __forceinline__ void st_shared_v4(uint32_t saddr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(saddr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

// Eight consecutive values of row t (columns k0 .. k0 + 7, k0 % 8 == 0) as one 16-byte store.
__device__ __forceinline__ void store8(uint32_t buf, int cols, int t, int k0, const float* v) {
  st_shared_v4(buf + tc::core_off(t, k0, cols), tc::pack2_bf16(v[0], v[1]), tc::pack2_bf16(v[2], v[3]),
               tc::pack2_bf16(v[4], v[5]), tc::pack2_bf16(v[6], v[7]));
}

// The same as a BF16 pair: hi = bf16(v) into hi_buf, lo = bf16(v - hi) into lo_buf.
__device__ __forceinline__ void store8_split(uint32_t hi_buf, uint32_t lo_buf, int cols, int t, int k0,
                                             const float* v) {
  uint32_t h[4], l[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    h[q] = tc::pack2_bf16(v[2 * q], v[2 * q + 1]);
    l[q] = tc::pack2_bf16(v[2 * q] - __uint_as_float(h[q] << 16), v[2 * q + 1] - __uint_as_float(h[q] & 0xffff0000u));
  }
  const uint32_t off = tc::core_off(t, k0, cols);
  st_shared_v4(hi_buf + off, h[0], h[1], h[2], h[3]);
  st_shared_v4(lo_buf + off, l[0], l[1], l[2], l[3]);
}

// Column K of the head's input row (the reference's order, models/FactorFields.py:188-195),
// decoded at compile time: fr = the staged feature row (fr[kOff + c] = feature c), dr = the ray
// direction; past in_dim a constant 1 (column in_dim, which in_pad always has), then 0. Positional-encoding columns use the hardware sin / cos.
template <int C, int F, int V, int K, int kOff>
__device__ __forceinline__ float x_col(const float* fr, const float* dr) {
  if constexpr (K < C) {
    return fr[kOff + K];
  } else if constexpr (K < C + 3) {
    return dr[K - C];
  } else if constexpr (K < C + 3 + 2 * C * F) {
    constexpr int k = K - C - 3;
    constexpr bool kCos = k >= C * F;
    constexpr int j = kCos ? k - C * F : k;
    const float x = fr[kOff + j / F] * (float)(1 << (j % F));
    return kCos ? __cosf(x) : __sinf(x);
  } else if constexpr (K < C + 3 + 2 * C * F + 6 * V) {
    constexpr int k = K - C - 3 - 2 * C * F;
    constexpr bool kCos = k >= 3 * V;
    constexpr int j = kCos ? k - 3 * V : k;
    const float x = dr[j / V] * (float)(1 << (j % V));
    return kCos ? __cosf(x) : __sinf(x);
  } else if constexpr (K == C + 3 + 2 * C * F + 6 * V) {
    return 1.f;  // the first pad column: W0's is zero; dW0's is the bias gradient sum_s dH0
  } else {
    return 0.f;
  }
}

// Columns 8 CH .. 8 CH + 7 of row rr: as a BF16 pair (one 16-byte store into each of X_hi and
// X_lo), or with kF16 as FP16 values (one 16-byte store into X; Xlo unused).
template <int C, int F, int V, bool kF16, int kOff, int CH, int... J>
__device__ __forceinline__ void build_chunk(uint32_t X, uint32_t Xlo, int rr, const float* fr, const float* dr,
                                            std::integer_sequence<int, J...>, float* raw_max = nullptr) {
  const float v[8] = {x_col<C, F, V, CH * 8 + J, kOff>(fr, dr)...};
  if constexpr (kF16) {
    st_shared_v4(X + tc::core_off(rr, CH * 8, Shape<C, F, V>::IN_PAD), tc::pack2_f16(v[0], v[1]),
                 tc::pack2_f16(v[2], v[3]), tc::pack2_f16(v[4], v[5]), tc::pack2_f16(v[6], v[7]));
    if constexpr (CH * 8 < C + 3) {  // features and direction: the unbounded inputs
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (CH * 8 + j < C + 3) *raw_max = fmaxf(*raw_max, fabsf(v[j]));
    }
  } else {
    store8_split(X, Xlo, Shape<C, F, V>::IN_PAD, rr, CH * 8, v);
  }
}

// Chunks O, O + 4, O + 8, ... of row rr (all compile-time: one dispatch per tile, not per chunk).
template <int C, int F, int V, bool kF16, int kOff, int O, int J = 0>
__device__ __forceinline__ void build_seq(uint32_t X, uint32_t Xlo, int rr, const float* fr, const float* dr,
                                          float* raw_max) {
  constexpr int CH = 4 * J + O;
  if constexpr (CH < Shape<C, F, V>::IN_PAD / 8) {
    build_chunk<C, F, V, kF16, kOff, CH>(X, Xlo, rr, fr, dr, std::make_integer_sequence<int, 8>{}, raw_max);
    build_seq<C, F, V, kF16, kOff, O, J + 1>(X, Xlo, rr, fr, dr, raw_max);
  }
}

// X of row rr: the thread's chunk sequence `part` (0..3) dispatched once.
template <int C, int F, int V, bool kF16, int kOff>
__device__ __forceinline__ void build_row(int part, uint32_t X, uint32_t Xlo, int rr, const float* fr, const float* dr,
                                          float* raw_max) {
  switch (part) {
    case 0: build_seq<C, F, V, kF16, kOff, 0>(X, Xlo, rr, fr, dr, raw_max); break;
    case 1: build_seq<C, F, V, kF16, kOff, 1>(X, Xlo, rr, fr, dr, raw_max); break;
    case 2: build_seq<C, F, V, kF16, kOff, 2>(X, Xlo, rr, fr, dr, raw_max); break;
    default: build_seq<C, F, V, kF16, kOff, 3>(X, Xlo, rr, fr, dr, raw_max); break;
  }
}

// dL/dfeat terms of the 32 dX columns 32 CI .. 32 CI + 31 (inside [0, NX)) of row r, added to the
// row sums gr: raw feature columns directly, PE columns through d/dx sin(x 2^f) = 2^f cos(x 2^f),
// d/dx cos(x 2^f) = -2^f sin(x 2^f).
template <int C, int F, int V, int CI, int... J>
__device__ __forceinline__ void pe_back_chunk(const float* v, const float* fr, float* gr,
                                              std::integer_sequence<int, J...>) {
  auto one = [&](auto jc) {
    constexpr int k = CI * 32 + decltype(jc)::value;
    if constexpr (k < C) {
      atomicAdd(gr + k, v[decltype(jc)::value]);
    } else if constexpr (k >= C + 3 && k < C + 3 + 2 * F * C) {
      constexpr bool kCos = k >= C + 3 + F * C;
      constexpr int jj = k - C - 3 - (kCos ? F * C : 0);
      constexpr int c = jj / F, f = jj % F;
      const float x = fr[1 + c] * (float)(1 << f);
      atomicAdd(gr + c, (float)(1 << f) * (kCos ? -__sinf(x) : __cosf(x)) * v[decltype(jc)::value]);
    }
  };
  (one(std::integral_constant<int, J>{}), ...);
}

template <int C, int F, int V, int CI = 0>
__device__ __forceinline__ void pe_back_at(int ci, const float* v, const float* fr, float* gr) {
  if constexpr (CI < (Shape<C, F, V>::NX + 31) / 32) {
    if (ci == CI) {
      pe_back_chunk<C, F, V, CI>(v, fr, gr, std::make_integer_sequence<int, 32>{});
      return;
    }
    pe_back_at<C, F, V, CI + 1>(ci, v, fr, gr);
  }
}

// Warp reduce-scatter: lane l returns the sum over the warp's lanes of v[l].
__device__ __forceinline__ float warp_reduce_scatter32(float* v, int lane) {
#pragma unroll
  for (int o = 16, n = 16; o >= 1; o >>= 1, n >>= 1) {
    const bool upper = (lane & o) != 0;
#pragma unroll
    for (int i = 0; i < n; ++i) {
      const float send = upper ? v[i] : v[i + n];
      const float keep = upper ? v[i + n] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, o);
    }
  }
  return v[0];
}

template <int C, int F, int V>
__global__ void __launch_bounds__(kThreads, 1) head_tc_kernel(const HeadArgs a) {
  using S = Shape<C, F, V>;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int quad = warp & 3, part = warp >> 2;  // TMEM lane quadrant and 32-column slice
  const int r = quad * 32 + lane;               // this thread's row (sample) in the epilogues
  unsigned char* p = smem;
  const uint32_t sW0 = tc::smem_u32(p); p += S::W0_B;
  const uint32_t sW1 = tc::smem_u32(p); p += S::W1_B;
  const uint32_t sX = tc::smem_u32(p); p += S::X_B;
  unsigned char* pR = p;
  const uint32_t sR = tc::smem_u32(p); p += S::R_B;
  const uint32_t sXlo = sR;               // F1
  const uint32_t sH0 = sR;                // H0_hi (F2, B2), then dH0 (B3, B4)
  const uint32_t sH0lo = sR + S::H_B;     // H0_lo (F2)
  const uint32_t sDH1 = sR + S::H_B;      // dH1 (B1, B2), after F2
  float4* yp = reinterpret_cast<float4*>(pR + S::H_B);  // [4 slices][128 rows] partial y, before dH1
  float* gfs = reinterpret_cast<float*>(pR);            // [128][FS] dL/dfeat row sums, after B3 / B4
  float* fs = reinterpret_cast<float*>(p); p += S::FEAT_B;
  float* ds = reinterpret_cast<float*>(p); p += S::DIR_B;
  int32_t* idx_s = reinterpret_cast<int32_t*>(p); p += S::IDX_B;
  float* w2s = reinterpret_cast<float*>(p); p += 3 * kH * 4;
  float* b0s = reinterpret_cast<float*>(p); p += kH * 4;
  float* b1s = reinterpret_cast<float*>(p); p += kH * 4;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);
  uint32_t* taddr_s = reinterpret_cast<uint32_t*>(p + 8);
  const uint32_t mb = tc::smem_u32(mbar);
  constexpr uint32_t kTmemCols = 512u;

  // ---- weights -> shared memory (BF16 core layout; W2 rounded to BF16 like W0, W1; biases float32) ----
  for (int e = t; e < kH * S::IN_PAD; e += kThreads) {
    const int rr = e / S::IN_PAD, c = e % S::IN_PAD;
    const float v = c < S::IN ? a.w[0][rr * S::IN + c] : 0.f;
    *reinterpret_cast<__nv_bfloat16*>(smem + tc::core_off(rr, c, S::IN_PAD)) = __float2bfloat16_rn(v);
  }
  for (int e = t; e < kH * kH; e += kThreads) {
    const int rr = e / kH, c = e % kH;
    *reinterpret_cast<__nv_bfloat16*>(smem + S::W0_B + tc::core_off(rr, c, kH)) = __float2bfloat16_rn(a.w[1][e]);
  }
  for (int e = t; e < 3 * kH; e += kThreads) w2s[e] = __bfloat162float(__float2bfloat16_rn(a.w[2][e]));
  if (t < kH) {
    b0s[t] = a.b[0] ? a.b[0][t] : 0.f;
    b1s[t] = a.b[1] ? a.b[1][t] : 0.f;
  }
  tc::fence_smem_to_async();
  if (t == 0) {
    tc::mbar_init(mb, 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(taddr_s), kTmemCols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *taddr_s;
  const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
  const uint32_t tS = tmem;
  const uint32_t tDW1 = tmem + S::COL_DW1, tDW0 = tmem + S::COL_DW0;

  uint32_t phase = 0;
  bool ok = true, any_tile = false;
  float acc_db1 = 0.f, acc_dw2[3] = {0.f, 0.f, 0.f};  // column 32 part + lane

  // waits for the MMAs committed last; all threads agree on the outcome
  auto wait_mma = [&]() {
    const bool done = tc::mbar_wait(mb, phase & 1u, kPolls);
    ++phase;
    ok = __syncthreads_and(done) != 0;
    tc::fence_after_sync();
    return ok;
  };

  const int64_t n_tiles = ceil_div(a.n, kTile);
  // rows staged by this warp: its feature channel (lane <= C), direction component (lane < 3) and
  // row index, held in registers from the previous tile's prefetch
  constexpr int kRowsPerWarp = kTile / (kThreads / 32);
  float pf[kRowsPerWarp], pd[kRowsPerWarp];
  int32_t pix[kRowsPerWarp];
  auto load_rows = [&](int64_t tl) {
    int64_t ray[kRowsPerWarp];
#pragma unroll
    for (int i = 0; i < kRowsPerWarp; ++i) {
      const int64_t row = tl * kTile + warp * kRowsPerWarp + i;
      const bool valid = row < a.n;
      pix[i] = valid ? a.app_idx[row] : -1;
      ray[i] = valid ? (int64_t)a.app_ray[row] : -1;
    }
#pragma unroll
    for (int i = 0; i < kRowsPerWarp; ++i) {
      pf[i] = (pix[i] >= 0 && lane <= C) ? a.feat[(int64_t)pix[i] * a.feat_stride + lane] : 0.f;
      pd[i] = (ray[i] >= 0 && lane < 3) ? a.rays[ray[i] * 6 + 3 + lane] : 0.f;
    }
  };
  if ((int64_t)blockIdx.x < n_tiles) load_rows(blockIdx.x);
  for (int64_t tile = blockIdx.x; tile < n_tiles && ok; tile += gridDim.x) {
    // ---- the tile's feature rows (channels 0..C), directions and row indices -> shared memory
    // (loaded into registers one tile ahead), then the next tile's loads are issued ----
#pragma unroll
    for (int i = 0; i < kRowsPerWarp; ++i) {
      const int rr = warp * kRowsPerWarp + i;
      if (lane <= C) fs[rr * S::FS + lane] = pf[i];
      if (lane < 3) ds[rr * 4 + lane] = pd[i];
      if (lane == 0) idx_s[rr] = pix[i];
    }
    __syncthreads();
    if (tile + gridDim.x < n_tiles) load_rows(tile + gridDim.x);
    // ---- X: thread = row r, its 8-column chunks part, + 4, + 8, ... (one 16-byte store each
    // into X_hi and X_lo) ----
    build_row<C, F, V, false, 1>(part, sX, sXlo, r, fs + r * S::FS, ds + r * 4, nullptr);
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    // ---- F1: S = X_hi W0^T + X_lo W0^T ----
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t id = tc::idesc_bf16(128, kH, false, false);
#pragma unroll 1
      for (int s = 0; s < S::IN_PAD / 16; ++s)
        tc::mma_f16kind(tS, desc_k(sX, S::IN_PAD, s), desc_k(sW0, S::IN_PAD, s), id, s > 0);
#pragma unroll 1
      for (int s = 0; s < S::IN_PAD / 16; ++s)
        tc::mma_f16kind(tS, desc_k(sXlo, S::IN_PAD, s), desc_k(sW0, S::IN_PAD, s), id, 1u);
      tc::mma_commit(mb);
    }
    if (!wait_mma()) break;
    // ---- H0 = relu(S + b0) (this thread's 32 columns) ----
    uint32_t mask0 = 0;
    {
      float v[32];
      tc::tmem_ld32(tS + lane_off + part * 32, v);
      const float4* b0v = reinterpret_cast<const float4*>(b0s + part * 32);  // warp-uniform: broadcasts
#pragma unroll
      for (int j4 = 0; j4 < 8; ++j4) {
        const float4 b = b0v[j4];
        const float bb[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int j = 4 * j4 + q;
          const float h = v[j] + bb[q];
          mask0 |= (h > 0.f ? 1u : 0u) << j;
          v[j] = fmaxf(h, 0.f);
        }
      }
#pragma unroll
      for (int g = 0; g < 4; ++g) store8_split(sH0, sH0lo, kH, r, part * 32 + g * 8, v + g * 8);
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    // ---- F2: S = H0_hi W1^T + H0_lo W1^T ----
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t id = tc::idesc_bf16(128, kH, false, false);
#pragma unroll 1
      for (int s = 0; s < kH / 16; ++s) tc::mma_f16kind(tS, desc_k(sH0, kH, s), desc_k(sW1, kH, s), id, s > 0);
#pragma unroll 1
      for (int s = 0; s < kH / 16; ++s) tc::mma_f16kind(tS, desc_k(sH0lo, kH, s), desc_k(sW1, kH, s), id, 1u);
      tc::mma_commit(mb);
    }
    if (!wait_mma()) break;
    // ---- y = relu(S + b1) W2^T: the slice's partial sums, summed over the 4 slices ----
    float h1[32];
    {
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
      tc::tmem_ld32(tS + lane_off + part * 32, h1);
      const float4* b1v = reinterpret_cast<const float4*>(b1s + part * 32);
      const float4* w2v = reinterpret_cast<const float4*>(w2s + part * 32);  // rows kH / 4 float4 apart
#pragma unroll
      for (int j4 = 0; j4 < 8; ++j4) {
        const float4 b = b1v[j4], wa = w2v[j4], wb = w2v[kH / 4 + j4], wc = w2v[kH / 2 + j4];
        const float bb[4] = {b.x, b.y, b.z, b.w}, w0[4] = {wa.x, wa.y, wa.z, wa.w};
        const float w1[4] = {wb.x, wb.y, wb.z, wb.w}, w2[4] = {wc.x, wc.y, wc.z, wc.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int j = 4 * j4 + q;
          const float h = fmaxf(h1[j] + bb[q], 0.f);
          h1[j] = h;
          y0 += h * w0[q];
          y1 += h * w1[q];
          y2 += h * w2[q];
        }
      }
      yp[part * kTile + r] = make_float4(y0, y1, y2, 0.f);
    }
    __syncthreads();
    float rgb[3];
    {
      float4 ys = yp[r];
#pragma unroll
      for (int q = 1; q < 4; ++q) {
        const float4 o = yp[q * kTile + r];
        ys.x += o.x; ys.y += o.y; ys.z += o.z;
      }
      rgb[0] = 1.f / (1.f + expf(-ys.x));
      rgb[1] = 1.f / (1.f + expf(-ys.y));
      rgb[2] = 1.f / (1.f + expf(-ys.z));
    }
    const int32_t sidx = idx_s[r];
    {
      float dy[3];
#pragma unroll
      for (int o = 0; o < 3; ++o) dy[o] = sidx >= 0 ? a.grad_rgb[(int64_t)sidx * 3 + o] * rgb[o] * (1.f - rgb[o]) : 0.f;
      __syncthreads();  // every slice has read yp before dH1 overwrites it
      // dH1 = (dy W2) [H1 > 0]; dW2 += dy^T H1, db1 += sum dH1 (warp reduce-scatters)
      {
        float dh[32];
        const float4* w2v = reinterpret_cast<const float4*>(w2s + part * 32);
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          const float4 wa = w2v[j4], wb = w2v[kH / 4 + j4], wc = w2v[kH / 2 + j4];
          const float w0[4] = {wa.x, wa.y, wa.z, wa.w}, w1[4] = {wb.x, wb.y, wb.z, wb.w};
          const float w2[4] = {wc.x, wc.y, wc.z, wc.w};
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int j = 4 * j4 + q;
            dh[j] = h1[j] > 0.f ? dy[0] * w0[q] + dy[1] * w1[q] + dy[2] * w2[q] : 0.f;
          }
        }
#pragma unroll
        for (int g = 0; g < 4; ++g) store8(sDH1, kH, r, part * 32 + g * 8, dh + g * 8);
        acc_db1 += warp_reduce_scatter32(dh, lane);
#pragma unroll
        for (int o = 0; o < 3; ++o) {
          float pr[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) pr[j] = dy[o] * h1[j];
          acc_dw2[o] += warp_reduce_scatter32(pr, lane);
        }
      }
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      // ---- B1: S = dH1 W1;  B2: dW1 += dH1^T H0_hi ----
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t id1 = tc::idesc_bf16(128, kH, false, true);
#pragma unroll 1
        for (int s = 0; s < kH / 16; ++s) tc::mma_f16kind(tS, desc_k(sDH1, kH, s), desc_mn(sW1, kH, s), id1, s > 0);
        const uint32_t id2 = tc::idesc_bf16(128, kH, true, true);
#pragma unroll 1
        for (int s = 0; s < kTile / 16; ++s)
          tc::mma_f16kind(tDW1, desc_mn(sDH1, kH, s), desc_mn(sH0, kH, s), id2, (any_tile || s > 0) ? 1u : 0u);
        tc::mma_commit(mb);
      }
      if (!wait_mma()) break;
      // ---- dH0 = S [H0 > 0] (over H0_hi); db0 accumulates in dW0's column in_dim (X = 1 there) ----
      {
        float v[32];
        tc::tmem_ld32(tS + lane_off + part * 32, v);
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = ((mask0 >> j) & 1u) ? v[j] : 0.f;
#pragma unroll
        for (int g = 0; g < 4; ++g) store8(sH0, kH, r, part * 32 + g * 8, v + g * 8);
      }
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      // ---- B3: dW0 += dH0^T X_hi;  B4: S = dH0 W0 (columns [0, NX)) ----
      if (t == 0) {
        tc::fence_after_sync();
        const uint32_t id3 = tc::idesc_bf16(128, S::IN_PAD, true, true);
#pragma unroll 1
        for (int s = 0; s < kTile / 16; ++s)
          tc::mma_f16kind(tDW0, desc_mn(sH0, kH, s), desc_mn(sX, S::IN_PAD, s), id3, (any_tile || s > 0) ? 1u : 0u);
        const uint32_t id4 = tc::idesc_bf16(128, S::NX, false, true);
#pragma unroll 1
        for (int s = 0; s < kH / 16; ++s) tc::mma_f16kind(tS, desc_k(sH0, kH, s), desc_mn(sW0, S::IN_PAD, s), id4, s > 0);
        tc::mma_commit(mb);
      }
      if (!wait_mma()) break;
      any_tile = true;
      // ---- dL/dfeat through the positional encoding: per-row sums in shared memory ----
      for (int e = t; e < kTile * S::FS; e += kThreads) gfs[e] = 0.f;
      __syncthreads();
      {
        const float* fr = fs + r * S::FS;
        float* gr = gfs + r * S::FS;
#pragma unroll 1
        for (int ci = part; ci < (S::NX + 31) / 32; ci += 4) {  // 32-column loads inside S
          float v[32];
          tc::tmem_ld32(tS + lane_off + ci * 32, v);
          pe_back_at<C, F, V>(ci, v, fr, gr);
        }
      }
      __syncthreads();
#pragma unroll 1
      for (int i = 0; i < kTile / 16; ++i) {  // a warp per row: coalesced writes of channels 1..C
        const int rr = warp * (kTile / 16) + i;
        const int32_t si = idx_s[rr];
        if (si >= 0 && lane < C) a.grad_feat[(int64_t)si * a.feat_stride + 1 + lane] = gfs[rr * S::FS + lane];
      }
      tc::fence_before_sync();
      __syncthreads();
    }
  }

  if (!ok) {
    if (t == 0 && a.status) atomicExch(a.status, FF_ERR_LIMIT);
    (void)tc::mbar_wait(mb, phase & 1u, kPolls);  // the MMAs in flight, if they ever finish
  } else if (any_tile) {
    // ---- flush: dW1 / dW0 rows from TMEM (row = this thread's lane), the register sums ----
    {
      float v[32];
      tc::tmem_ld32(tDW1 + lane_off + part * 32, v);
      if (a.gw[1])
#pragma unroll
        for (int j = 0; j < 32; ++j) atomicAdd(a.gw[1] + r * kH + part * 32 + j, v[j]);
    }
#pragma unroll 1
    for (int ci = part; ci < (S::IN_PAD + 31) / 32; ci += 4) {
      float v[32];
      tc::tmem_ld32(tDW0 + lane_off + ci * 32, v);  // columns past IN_PAD (inside the allocation) unused
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        if (ci * 32 + j < S::IN) {
          if (a.gw[0]) atomicAdd(a.gw[0] + r * S::IN + ci * 32 + j, v[j]);
        } else if (ci * 32 + j == S::IN) {
          if (a.gb[0]) atomicAdd(a.gb[0] + r, v[j]);  // db0[r] = sum over samples of dH0[., r]
        }
      }
    }
    const int col = part * 32 + lane;
    if (a.gb[1]) atomicAdd(a.gb[1] + col, acc_db1);
    if (a.gw[2])
#pragma unroll
      for (int o = 0; o < 3; ++o) atomicAdd(a.gw[2] + o * kH + col, acc_dw2[o]);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// ---- forward: FP16 operands, software-pipelined over tiles ----
//
// The forward alone has no gradient operands, so X and H0 are single FP16 values (11
// significant bits; W0 and W1 hold BF16 values, which FP16 represents exactly in its normal
// range): one MMA pass per layer and half the operand bytes. The freed shared memory holds two
// tiles' operand buffers, staged rows and TMEM accumulators, and the tiles are pipelined so that
// the tensor core works while the CUDA cores do:
//
//   iteration i (buffer b = i & 1; F1 of tile i was issued at the end of iteration i - 2):
//     load the row indices of tile i + 2;  wait F1(i); H0(i) = relu(S_b + b0) -> X_b (FP16)
//     issue F2(i) -> S_b;  copy the rows of tile i + 2 -> R_b (cp.async)   (overlaps F2(i))
//     wait F2(i); y partials -> X_b; rgb = sigmoid(y) out
//     build X(i + 2) from R_b -> X_b;  issue F1(i + 2) -> S_b      (runs during iteration i + 1)
//
// 512 threads; warp w serves TMEM lane quadrant w % 4 and the 32-column slice w / 4, as in the
// backward kernel. A staged row holds features 1..C, the direction and the row index.
template <int C, int F, int V>
struct Fwd16 {
  using S = Shape<C, F, V>;
  static constexpr int RS = (C + 4) | 1;  // features at [0, C), direction at [C, C + 3), index at C + 3
  static constexpr int W0_B = S::W0_B, W1_B = S::W1_B;
  static constexpr int X_B = kTile * S::IN_PAD * 2;  // X, then H0 [128 x 128], then the y partials
  static constexpr int ROW_B = kTile * RS * 4;
  static constexpr int F32_B = 5 * kH * 4;
  static_assert(kH * kH * 2 <= X_B && 4 * kTile * 16 <= X_B, "H0 and the y partials fit in X's buffer");
  static_assert(X_B % 16 == 0 && ROW_B % 16 == 0 && W0_B % 16 == 0, "16-byte alignment");
  static constexpr int smem() { return W0_B + W1_B + 2 * X_B + 2 * ROW_B + F32_B + 64; }
};

constexpr float kF16Max = 65504.f;

// 4-byte asynchronous global -> shared copy; with v false the destination is zero-filled and
// nothing is read (src is any valid address).
__device__ __forceinline__ void cp_async4(float* dst, const float* src, bool v) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(v ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int C, int F, int V>
__global__ void __launch_bounds__(kThreads, 1) head_fwd16_kernel(const HeadArgs a) {
  using S = Shape<C, F, V>;
  using L = Fwd16<C, F, V>;
  extern __shared__ __align__(1024) unsigned char smem[];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int quad = warp & 3, part = warp >> 2;  // TMEM lane quadrant and 32-column slice
  const int r = quad * 32 + lane;               // this thread's row in the epilogues
  unsigned char* p = smem;
  const uint32_t sW0 = tc::smem_u32(p); p += L::W0_B;
  const uint32_t sW1 = tc::smem_u32(p); p += L::W1_B;
  unsigned char* const xbase = p;  // X_0, X_1
  p += 2 * L::X_B;
  unsigned char* const rbase = p;  // R_0, R_1
  p += 2 * L::ROW_B;
  auto xb = [&](int b) { return xbase + b * L::X_B; };
  auto rb = [&](int b) { return reinterpret_cast<float*>(rbase + b * L::ROW_B); };
  float* w2s = reinterpret_cast<float*>(p); p += 3 * kH * 4;
  float* b0s = reinterpret_cast<float*>(p); p += kH * 4;
  float* b1s = reinterpret_cast<float*>(p); p += kH * 4;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(p);  // [0], [1]: F1 of buffer 0 / 1; [2]: F2
  uint32_t* taddr_s = reinterpret_cast<uint32_t*>(p + 24);

  // ---- weights -> shared memory: BF16-rounded (the stored head), held as FP16 ----
  bool range_ok = true;
  for (int e = t; e < kH * S::IN_PAD; e += kThreads) {
    const int rr = e / S::IN_PAD, c = e % S::IN_PAD;
    const float v = __bfloat162float(__float2bfloat16_rn(c < S::IN ? a.w[0][rr * S::IN + c] : 0.f));
    range_ok &= !(fabsf(v) > kF16Max);  // NaN passes (propagates as in float32)
    *reinterpret_cast<__half*>(smem + tc::core_off(rr, c, S::IN_PAD)) = __float2half_rn(v);
  }
  for (int e = t; e < kH * kH; e += kThreads) {
    const int rr = e / kH, c = e % kH;
    const float v = __bfloat162float(__float2bfloat16_rn(a.w[1][e]));
    range_ok &= !(fabsf(v) > kF16Max);
    *reinterpret_cast<__half*>(smem + L::W0_B + tc::core_off(rr, c, kH)) = __float2half_rn(v);
  }
  for (int e = t; e < 3 * kH; e += kThreads) w2s[e] = __bfloat162float(__float2bfloat16_rn(a.w[2][e]));
  if (t < kH) {
    b0s[t] = a.b[0] ? a.b[0][t] : 0.f;
    b1s[t] = a.b[1] ? a.b[1][t] : 0.f;
  }
  tc::fence_smem_to_async();
  if (t == 0) {
    for (int i = 0; i < 3; ++i) tc::mbar_init(tc::smem_u32(mbar + i), 1);
    tc::fence_mbar_init();
  }
  __syncthreads();
  if (warp == 0) tc::tmem_alloc(tc::smem_u32(taddr_s), 256u);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *taddr_s;
  const uint32_t lane_off = (uint32_t)(quad * 32) << 16;

  uint32_t ph = 0;  // bit m: the parity of mbarrier m's next phase
  bool ok = true;
  auto wait_mma = [&](int m) {
    const bool done = tc::mbar_wait(tc::smem_u32(mbar + m), (ph >> m) & 1u, kPolls);
    ph ^= 1u << m;
    ok = __syncthreads_and(done) != 0;
    tc::fence_after_sync();
    return ok;
  };

  const int64_t n_tiles = ceil_div(a.n, kTile);
  const int64_t stride = gridDim.x;
  // the CTA's tiles: blockIdx.x + i * gridDim.x, i = 0, 1, ...
  auto tile_at = [&](int64_t i) { return (int64_t)blockIdx.x + i * stride; };
  // Staging of tile `tile`'s rows into R (a warp per row): features 1..C, the direction, the row
  // index. First the row indices (into registers), later the rows themselves as asynchronous
  // 4-byte copies (cp.async; completed by cp_async_wait_all before the rows are read).
  constexpr int kRowsPerWarp = kTile / (kThreads / 32);
  auto stage_idx = [&](int64_t tile, int32_t* pix, int32_t* pray) {
#pragma unroll
    for (int i = 0; i < kRowsPerWarp; ++i) {
      const int64_t row = tile * kTile + warp * kRowsPerWarp + i;
      const bool valid = row < a.n;
      pix[i] = valid ? a.app_idx[row] : -1;
      pray[i] = valid ? a.app_ray[row] : -1;
    }
  };
  auto stage_rows = [&](const int32_t* pix, const int32_t* pray, float* R) {
#pragma unroll
    for (int i = 0; i < kRowsPerWarp; ++i) {
      float* row = R + (warp * kRowsPerWarp + i) * L::RS;
      if (lane < C) {
        const bool v = pix[i] >= 0;
        cp_async4(row + lane, v ? a.feat + (int64_t)pix[i] * a.feat_stride + 1 + lane : a.feat, v);
      }
      if (lane < 3) {
        const bool v = pray[i] >= 0;
        cp_async4(row + C + lane, v ? a.rays + (int64_t)pray[i] * 6 + 3 + lane : a.rays, v);
      }
      if (lane == 0) row[C + 3] = __int_as_float(pix[i]);
    }
    cp_async_commit();
  };
  // X (FP16) of the rows in R -> buffer X: thread = row (warp & 3) * 32 + lane, its 8-column
  // chunks warp / 4, + 4, + 8, ... (one 16-byte store each); the FP16 range check of the raw inputs
  auto build = [&](const float* R, uint32_t X) {
    const int rr = quad * 32 + lane;
    const float* fr = R + rr * L::RS;
    float m = 0.f;
    build_row<C, F, V, true, 0>(part, X, 0u, rr, fr, fr + C, &m);
    range_ok &= !(m > kF16Max);  // NaN passes (propagates as in float32)
  };
  auto issue_f1 = [&](int b) {  // by thread 0, after the barrier that published X_b
    tc::fence_after_sync();
    const uint32_t id = tc::idesc_f16kind(128, kH, false, false, false);
    const uint32_t sx = tc::smem_u32(xb(b));
#pragma unroll 1
    for (int s = 0; s < S::IN_PAD / 16; ++s)
      tc::mma_f16kind(tmem + 128 * b, desc_k(sx, S::IN_PAD, s), desc_k(sW0, S::IN_PAD, s), id, s > 0);
    tc::mma_commit(tc::smem_u32(mbar + b));
  };

  // ---- prologue: tiles 0 and 1 staged and built, their F1 issued ----
  for (int b = 0; b < 2; ++b) {
    if (tile_at(b) < n_tiles) {
      int32_t pix[kRowsPerWarp], pray[kRowsPerWarp];
      stage_idx(tile_at(b), pix, pray);
      stage_rows(pix, pray, rb(b));
    }
  }
  cp_async_wait_all();
  __syncthreads();
  for (int b = 0; b < 2; ++b) {
    if (tile_at(b) < n_tiles) {
      build(rb(b), tc::smem_u32(xb(b)));
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0) issue_f1(b);
    }
  }

  for (int64_t i = 0; tile_at(i) < n_tiles && ok; ++i) {
    const int b = (int)(i & 1);
    const uint32_t sx = tc::smem_u32(xb(b));
    const uint32_t tS = tmem + 128 * b;
    // this row's sample index, read before R_b is restaged with tile i + 2; the row indices of
    // tile i + 2 are loaded meanwhile
    const int32_t sidx = part == 0 ? __float_as_int(rb(b)[r * L::RS + C + 3]) : -1;
    const bool next2 = tile_at(i + 2) < n_tiles;
    int32_t pix[kRowsPerWarp], pray[kRowsPerWarp];
    if (next2) stage_idx(tile_at(i + 2), pix, pray);
    // ---- H0 = relu(S + b0) -> X_b as FP16 [128 x 128] (F1 has consumed X) ----
    if (!wait_mma(b)) break;
    {
      float v[32];
      tc::tmem_ld32(tS + lane_off + part * 32, v);
      const float4* bv = reinterpret_cast<const float4*>(b0s + part * 32);
      float hmax = 0.f;
#pragma unroll
      for (int j4 = 0; j4 < 8; ++j4) {
        const float4 bb = bv[j4];
        v[4 * j4] = fmaxf(v[4 * j4] + bb.x, 0.f);
        v[4 * j4 + 1] = fmaxf(v[4 * j4 + 1] + bb.y, 0.f);
        v[4 * j4 + 2] = fmaxf(v[4 * j4 + 2] + bb.z, 0.f);
        v[4 * j4 + 3] = fmaxf(v[4 * j4 + 3] + bb.w, 0.f);
        hmax = fmaxf(hmax, fmaxf(fmaxf(v[4 * j4], v[4 * j4 + 1]), fmaxf(v[4 * j4 + 2], v[4 * j4 + 3])));
      }
      range_ok &= !(hmax > kF16Max);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const float* q = v + 8 * g;
        st_shared_v4(sx + tc::core_off(r, part * 32 + 8 * g, kH), tc::pack2_f16(q[0], q[1]), tc::pack2_f16(q[2], q[3]),
                     tc::pack2_f16(q[4], q[5]), tc::pack2_f16(q[6], q[7]));
      }
    }
    tc::fence_smem_to_async();
    tc::fence_before_sync();
    __syncthreads();
    // ---- F2: S = H0 W1^T ----
    if (t == 0) {
      tc::fence_after_sync();
      const uint32_t id = tc::idesc_f16kind(128, kH, false, false, false);
#pragma unroll 1
      for (int s = 0; s < kH / 16; ++s) tc::mma_f16kind(tS, desc_k(sx, kH, s), desc_k(sW1, kH, s), id, s > 0);
      tc::mma_commit(tc::smem_u32(mbar + 2));
    }
    // ---- the rows of tile i + 2 -> R_b, asynchronously (R_b's rows were consumed when X(i) was
    // built, its indices and range read above, before the barrier of the F1 wait) ----
    if (next2) stage_rows(pix, pray, rb(b));
    // ---- y = relu(S + b1) W2^T: the slice's partial sums, summed over the 4 slices ----
    if (!wait_mma(2)) break;
    float4* yp = reinterpret_cast<float4*>(xb(b));  // [4 slices][128 rows]; H0 is consumed
    {
      float h1[32];
      float y0 = 0.f, y1 = 0.f, y2 = 0.f;
      tc::tmem_ld32(tS + lane_off + part * 32, h1);
      const float4* b1v = reinterpret_cast<const float4*>(b1s + part * 32);
      const float4* w2v = reinterpret_cast<const float4*>(w2s + part * 32);  // rows kH / 4 float4 apart
#pragma unroll
      for (int j4 = 0; j4 < 8; ++j4) {
        const float4 bb = b1v[j4], wa = w2v[j4], wb = w2v[kH / 4 + j4], wc = w2v[kH / 2 + j4];
        const float bq[4] = {bb.x, bb.y, bb.z, bb.w}, u0[4] = {wa.x, wa.y, wa.z, wa.w};
        const float u1[4] = {wb.x, wb.y, wb.z, wb.w}, u2[4] = {wc.x, wc.y, wc.z, wc.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const float h = fmaxf(h1[4 * j4 + q] + bq[q], 0.f);
          y0 += h * u0[q];
          y1 += h * u1[q];
          y2 += h * u2[q];
        }
      }
      yp[part * kTile + r] = make_float4(y0, y1, y2, 0.f);
    }
    cp_async_wait_all();  // this thread's copies of tile i + 2's rows (published by the barrier)
    tc::fence_before_sync();
    __syncthreads();  // every slice's partials are written, R_b holds tile i + 2's rows
    if (sidx >= 0) {
      float4 ys = yp[r];
#pragma unroll
      for (int q = 1; q < 4; ++q) {
        const float4 o = yp[q * kTile + r];
        ys.x += o.x; ys.y += o.y; ys.z += o.z;
      }
      a.rgb_out[(int64_t)sidx * 3] = 1.f / (1.f + expf(-ys.x));
      a.rgb_out[(int64_t)sidx * 3 + 1] = 1.f / (1.f + expf(-ys.y));
      a.rgb_out[(int64_t)sidx * 3 + 2] = 1.f / (1.f + expf(-ys.z));
    }
    __syncthreads();  // the partials are read before X(i + 2) overwrites them
    // ---- X(i + 2) -> X_b, then its F1 -> S_b (S_b was read above) ----
    if (next2) {
      build(rb(b), sx);
      tc::fence_smem_to_async();
      tc::fence_before_sync();
      __syncthreads();
      if (t == 0) issue_f1(b);
    }
  }

  if (!ok) {
    if (t == 0 && a.status) atomicExch(a.status, FF_ERR_LIMIT);
    for (int m = 0; m < 3; ++m) (void)tc::mbar_wait(tc::smem_u32(mbar + m), (ph >> m) & 1u, kPolls);
  }
  if (!range_ok && a.status) atomicCAS(a.status, 0, FF_ERR_SIZE);
  cp_async_wait_all();  // no copy in flight when the CTA ends (after an early exit)
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, 256u);
}

template <int C, int F, int V>
cudaError_t launch_fwd16(const HeadArgs& a, cudaStream_t s) {
  constexpr int smem = Fwd16<C, F, V>::smem();
  static_assert(smem <= 227 * 1024, "shared memory per CTA");
  auto kern = head_fwd16_kernel<C, F, V>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int64_t tiles = ceil_div(a.n, kTile);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count()));
  kern<<<blocks, kThreads, smem, s>>>(a);
  return cudaGetLastError();
}

template <int C, int F, int V>
cudaError_t launch_tc(const HeadArgs& a, cudaStream_t s) {
  constexpr int smem = Shape<C, F, V>::smem();
  static_assert(smem <= 227 * 1024, "shared memory per CTA");
  auto kern = head_tc_kernel<C, F, V>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const int64_t tiles = ceil_div(a.n, kTile);
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)sm_count()));
  kern<<<blocks, kThreads, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t dispatch_fwd16(const FFRenderMlp& h, const HeadArgs& a, cudaStream_t s) {
  if (h.fea_pe == 2 && h.view_pe == 6) {
    if (h.in_channels == 27) return launch_fwd16<27, 2, 6>(a, s);
    if (h.in_channels == 31) return launch_fwd16<31, 2, 6>(a, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t dispatch_tc_bwd(const FFRenderMlp& h, const HeadArgs& a, cudaStream_t s) {
  if (h.fea_pe == 2 && h.view_pe == 6) {
    if (h.in_channels == 27) return launch_tc<27, 2, 6>(a, s);
    if (h.in_channels == 31) return launch_tc<31, 2, 6>(a, s);
  }
  return cudaErrorInvalidValue;
}

HeadArgs head_args(const FFRenderMlp& h, const float* feat, int feat_stride, const float* rays,
                   const int32_t* app_idx, const int32_t* app_ray, int64_t n, int32_t* status) {
  HeadArgs a = {};
  for (int l = 0; l < 3; ++l) a.w[l] = h.weight[l];
  a.b[0] = h.bias[0];
  a.b[1] = h.bias[1];
  a.feat = feat;
  a.feat_stride = feat_stride;
  a.rays = rays;
  a.app_idx = app_idx;
  a.app_ray = app_ray;
  a.n = n;
  a.status = status;
  return a;
}

}  // namespace

const char* render_head_tc_unsupported(const FFRenderMlp& h) {
  if (h.n_layers != 3 || h.hidden_dim != kH) return "the tensor-core head needs num_layers = 3 and hidden_dim = 128";
  if (h.fea_pe != 2 || h.view_pe != 6) return "the tensor-core head needs fea_pe = 2 and view_pe = 6";
  if (h.in_channels != 27 && h.in_channels != 31)
    return "the tensor-core head needs in_channels 27 or 31 (model.out_dim 28 or 32)";
  return nullptr;
}

cudaError_t launch_render_head_tc_forward(const FFRenderMlp& h, const float* feat, int feat_stride, const float* rays,
                                          const int32_t* app_idx, const int32_t* app_ray, int64_t n, float* rgb_rows,
                                          int32_t* status, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  HeadArgs a = head_args(h, feat, feat_stride, rays, app_idx, app_ray, n, status);
  a.rgb_out = rgb_rows;
  return dispatch_fwd16(h, a, s);
}

cudaError_t launch_render_head_tc_backward(const FFRenderMlp& h, const float* feat, int feat_stride, const float* rays,
                                           const int32_t* app_idx, const int32_t* app_ray, int64_t n,
                                           const float* grad_rgb_rows, float* grad_feat, const FFMlpGrad& g,
                                           int32_t* status, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  HeadArgs a = head_args(h, feat, feat_stride, rays, app_idx, app_ray, n, status);
  a.grad_rgb = grad_rgb_rows;
  a.grad_feat = grad_feat;
  for (int l = 0; l < 3; ++l) a.gw[l] = g.weight[l];
  a.gb[0] = g.bias[0];
  a.gb[1] = g.bias[1];
  return dispatch_tc_bwd(h, a, s);
}

}  // namespace ffgb
