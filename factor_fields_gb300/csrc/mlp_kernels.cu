// Drop-in float32 MLP head: MLPMixer.forward (models/FactorFields.py:144-159) and its backward.
//
// Persistent blocks of 256 threads keep every layer's weights in shared memory for their whole
// lifetime and walk tiles of P points. Activations live in shared memory TRANSPOSED,
// [feature][point], so that a thread's 4 consecutive points are one 128-bit load and a warp's
// loads cover 512 contiguous bytes (no bank conflicts); weight reads are warp broadcasts.
// All feature dimensions are padded to multiples of 8 with zeros.
//
// Backward recomputes the forward for the tile (nothing is saved from the forward launch),
// then runs the layers in reverse: weight gradients are reduced over the tile's points into
// block-private shared-memory accumulators (each entry owned by one thread, no atomics) and
// flushed to global memory with one atomicAdd per entry per block at the end.
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kThreads = 256;

__host__ __device__ __forceinline__ int pad8(int d) { return (d + 7) & ~7; }

struct MlpDims {
  int L;
  int d[FF_MAX_MLP_LAYERS + 1];  // d[0] = in, d[L] = out
};

__host__ __device__ inline MlpDims mlp_dims(const FFMlp& m) {
  MlpDims r;
  r.L = m.n_layers;
  for (int l = 0; l <= r.L; ++l) r.d[l] = (l == 0) ? m.in_dim : (l == r.L ? m.out_dim : m.hidden_dim);
  return r;
}

// Weight + bias floats of layer l in shared memory: [pad8(out)][pad8(in)] + pad8(out).
__host__ __device__ inline int layer_floats(const MlpDims& md, int l) {
  return pad8(md.d[l + 1]) * pad8(md.d[l]) + pad8(md.d[l + 1]);
}

__device__ void load_weights(const FFMlp& m, const MlpDims& md, float* w_s) {
  float* p = w_s;
  for (int l = 0; l < md.L; ++l) {
    const int din = md.d[l], dout = md.d[l + 1], ip = pad8(din), op = pad8(dout);
    for (int e = threadIdx.x; e < op * ip; e += blockDim.x) {
      const int j = e / ip, k = e % ip;
      p[e] = (j < dout && k < din) ? m.weight[l][(int64_t)j * din + k] : 0.f;
    }
    for (int j = threadIdx.x; j < op; j += blockDim.x) p[op * ip + j] = (m.bias[l] && j < dout) ? m.bias[l][j] : 0.f;
    p += op * ip + op;
  }
}

// act_out[j][p] = relu?(b[j] + sum_k W[j][k] act_in[k][p]) for j < dout; rows [dout, pad8) = 0.
template <int P>
__device__ void layer_forward(const float* __restrict__ W, int din, int dout, const float* __restrict__ act_in,
                              float* __restrict__ act_out, bool relu) {
  const int ip = pad8(din), op = pad8(dout);
  const float* bias = W + op * ip;
  constexpr int PG = P / 4;
  const int units = PG * (op / 8);
  for (int u = threadIdx.x; u < units; u += blockDim.x) {
    const int pg = u % PG, jg = u / PG;
    float acc[8][4];
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const float b = bias[jg * 8 + jj];
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[jj][q] = b;
    }
    for (int k = 0; k < ip; k += 4) {
      float a[4][4];
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float4 t = *reinterpret_cast<const float4*>(act_in + (k + kk) * P + pg * 4);
        a[kk][0] = t.x; a[kk][1] = t.y; a[kk][2] = t.z; a[kk][3] = t.w;
      }
#pragma unroll
      for (int jj = 0; jj < 8; ++jj) {
        const float4 w = *reinterpret_cast<const float4*>(W + (jg * 8 + jj) * ip + k);
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[jj][q] += w.x * a[0][q] + w.y * a[1][q] + w.z * a[2][q] + w.w * a[3][q];
      }
    }
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const int j = jg * 8 + jj;
      float4 o;
      if (j < dout) {
        o = make_float4(acc[jj][0], acc[jj][1], acc[jj][2], acc[jj][3]);
        if (relu) o = make_float4(fmaxf(o.x, 0.f), fmaxf(o.y, 0.f), fmaxf(o.z, 0.f), fmaxf(o.w, 0.f));
      } else {
        o = make_float4(0.f, 0.f, 0.f, 0.f);
      }
      *reinterpret_cast<float4*>(act_out + j * P + pg * 4) = o;
    }
  }
}

// Load rows [i0, i0+P) of a row-major [n, d] global matrix into smem transposed [pad8(d)][P].
template <int P>
__device__ void load_tile_T(const float* __restrict__ g, int64_t n, int d, int64_t i0, float* __restrict__ s) {
  const int dp = pad8(d);
  for (int e = threadIdx.x; e < dp * P; e += blockDim.x) {
    const int p = e % P, k = e / P;
    const int64_t i = i0 + p;
    s[k * P + p] = (k < d && i < n) ? g[i * d + k] : 0.f;
  }
}

template <int P>
__device__ void store_tile_T(float* __restrict__ g, int64_t n, int d, int64_t i0, const float* __restrict__ s) {
  for (int e = threadIdx.x; e < d * P; e += blockDim.x) {
    const int p = e % P, k = e / P;
    const int64_t i = i0 + p;
    if (i < n) g[i * d + k] = s[k * P + p];
  }
}

template <int P>
__global__ void __launch_bounds__(kThreads) mlp_forward_kernel(const FFMlp m, const float* __restrict__ x, int64_t n,
                                                               float* __restrict__ out) {
  extern __shared__ __align__(16) float smem[];
  const MlpDims md = mlp_dims(m);
  int wfl = 0, maxd = 0;
  for (int l = 0; l < md.L; ++l) wfl += layer_floats(md, l);
  for (int l = 0; l <= md.L; ++l) maxd = max(maxd, pad8(md.d[l]));
  float* w_s = smem;
  float* bufA = smem + wfl;
  float* bufB = bufA + maxd * P;
  load_weights(m, md, w_s);
  for (int64_t i0 = (int64_t)blockIdx.x * P; i0 < n; i0 += (int64_t)gridDim.x * P) {
    __syncthreads();
    load_tile_T<P>(x, n, md.d[0], i0, bufA);
    __syncthreads();
    const float* W = w_s;
    float* cur = bufA;
    float* nxt = bufB;
    for (int l = 0; l < md.L; ++l) {
      layer_forward<P>(W, md.d[l], md.d[l + 1], cur, nxt, l != md.L - 1);
      W += layer_floats(md, l);
      __syncthreads();
      float* t = cur; cur = nxt; nxt = t;
    }
    store_tile_T<P>(out, n, md.d[md.L], i0, cur);
  }
}

// dW[j][k] += sum_p g[j][p] a[k][p]; db[j] += sum_p g[j][p]. Units of 4x4 entries; each thread
// starts its point loop at a lane-dependent offset so the warp's 128-bit loads hit distinct banks.
template <int P>
__device__ void accumulate_wgrad(const float* __restrict__ g, const float* __restrict__ a, int din, int dout,
                                 float* __restrict__ dW) {
  const int ip = pad8(din), op = pad8(dout);
  float* db = dW + op * ip;
  const int jgs = op / 4, kgs = ip / 4;
  const int units = jgs * kgs;
  const int p0 = (threadIdx.x * 4) % P;
  for (int u = threadIdx.x; u < units; u += blockDim.x) {
    const int jg = u / kgs, kg = u % kgs;
    float acc[4][4] = {};
    float bsum[4] = {};
    for (int s = 0; s < P; s += 4) {
      const int p = (p0 + s) % P;
      float gv[4][4], av[4][4];
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
        const float4 t = *reinterpret_cast<const float4*>(g + (jg * 4 + jj) * P + p);
        gv[jj][0] = t.x; gv[jj][1] = t.y; gv[jj][2] = t.z; gv[jj][3] = t.w;
      }
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const float4 t = *reinterpret_cast<const float4*>(a + (kg * 4 + kk) * P + p);
        av[kk][0] = t.x; av[kk][1] = t.y; av[kk][2] = t.z; av[kk][3] = t.w;
      }
#pragma unroll
      for (int jj = 0; jj < 4; ++jj) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          acc[jj][kk] += gv[jj][0] * av[kk][0] + gv[jj][1] * av[kk][1] + gv[jj][2] * av[kk][2] + gv[jj][3] * av[kk][3];
        if (kg == 0) bsum[jj] += gv[jj][0] + gv[jj][1] + gv[jj][2] + gv[jj][3];
      }
    }
#pragma unroll
    for (int jj = 0; jj < 4; ++jj) {
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) dW[(jg * 4 + jj) * ip + kg * 4 + kk] += acc[jj][kk];
      if (kg == 0) db[jg * 4 + jj] += bsum[jj];
    }
  }
}

// gin[k][p] = sum_j W[j][k] g[j][p], masked by (act[k][p] > 0) when mask != nullptr.
template <int P>
__device__ void layer_backward_input(const float* __restrict__ W, int din, int dout, const float* __restrict__ g,
                                     const float* __restrict__ mask, float* __restrict__ gin) {
  const int ip = pad8(din);
  constexpr int PG = P / 4;
  const int units = PG * (ip / 8);
  for (int u = threadIdx.x; u < units; u += blockDim.x) {
    const int pg = u % PG, kg = u / PG;
    float acc[8][4] = {};
    for (int j = 0; j < dout; ++j) {
      const float4 gv = *reinterpret_cast<const float4*>(g + j * P + pg * 4);
      const float4 w0 = *reinterpret_cast<const float4*>(W + j * ip + kg * 8);
      const float4 w1 = *reinterpret_cast<const float4*>(W + j * ip + kg * 8 + 4);
      const float wk[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
      for (int kk = 0; kk < 8; ++kk) {
        acc[kk][0] += wk[kk] * gv.x; acc[kk][1] += wk[kk] * gv.y;
        acc[kk][2] += wk[kk] * gv.z; acc[kk][3] += wk[kk] * gv.w;
      }
    }
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
      const int k = kg * 8 + kk;
      float4 o = make_float4(acc[kk][0], acc[kk][1], acc[kk][2], acc[kk][3]);
      if (k >= din) {
        o = make_float4(0.f, 0.f, 0.f, 0.f);
      } else if (mask) {
        const float4 a = *reinterpret_cast<const float4*>(mask + k * P + pg * 4);
        o.x = a.x > 0.f ? o.x : 0.f; o.y = a.y > 0.f ? o.y : 0.f;
        o.z = a.z > 0.f ? o.z : 0.f; o.w = a.w > 0.f ? o.w : 0.f;
      }
      *reinterpret_cast<float4*>(gin + k * P + pg * 4) = o;
    }
  }
}

template <int P>
__global__ void __launch_bounds__(kThreads) mlp_backward_kernel(const FFMlp m, const float* __restrict__ x, int64_t n,
                                                                const float* __restrict__ grad_out,
                                                                float* __restrict__ grad_x, const FFMlpGrad gr) {
  extern __shared__ __align__(16) float smem[];
  const MlpDims md = mlp_dims(m);
  int wfl = 0, maxd = 0, actf = 0;
  for (int l = 0; l < md.L; ++l) {
    wfl += layer_floats(md, l);
    actf += pad8(md.d[l]) * P;
  }
  for (int l = 0; l <= md.L; ++l) maxd = max(maxd, pad8(md.d[l]));
  float* w_s = smem;
  float* dw_s = w_s + wfl;
  float* act = dw_s + wfl;  // act_l = input of layer l, l = 0..L-1
  float* gA = act + actf;
  float* gB = gA + maxd * P;
  load_weights(m, md, w_s);
  for (int e = threadIdx.x; e < wfl; e += blockDim.x) dw_s[e] = 0.f;
  for (int64_t i0 = (int64_t)blockIdx.x * P; i0 < n; i0 += (int64_t)gridDim.x * P) {
    __syncthreads();
    load_tile_T<P>(x, n, md.d[0], i0, act);
    load_tile_T<P>(grad_out, n, md.d[md.L], i0, gA);
    __syncthreads();
    {  // recompute the hidden activations of this tile
      const float* W = w_s;
      float* a = act;
      for (int l = 0; l + 1 < md.L; ++l) {
        layer_forward<P>(W, md.d[l], md.d[l + 1], a, a + pad8(md.d[l]) * P, true);
        W += layer_floats(md, l);
        a += pad8(md.d[l]) * P;
        __syncthreads();
      }
    }
    // reverse pass
    int woff = wfl, aoff = actf;
    float* g = gA;
    float* gn = gB;
    for (int l = md.L - 1; l >= 0; --l) {
      woff -= layer_floats(md, l);
      aoff -= pad8(md.d[l]) * P;
      const float* W = w_s + woff;
      const float* a = act + aoff;
      accumulate_wgrad<P>(g, a, md.d[l], md.d[l + 1], dw_s + woff);
      if (l > 0 || grad_x) layer_backward_input<P>(W, md.d[l], md.d[l + 1], g, l > 0 ? a : nullptr, gn);
      __syncthreads();
      float* t = g; g = gn; gn = t;
    }
    if (grad_x) store_tile_T<P>(grad_x, n, md.d[0], i0, g);
  }
  __syncthreads();
  // flush the block's weight gradients
  int woff = 0;
  for (int l = 0; l < md.L; ++l) {
    const int din = md.d[l], dout = md.d[l + 1], ip = pad8(din), op = pad8(dout);
    if (gr.weight[l])
      for (int e = threadIdx.x; e < dout * din; e += blockDim.x)
        atomicAdd(gr.weight[l] + e, dw_s[woff + (e / din) * ip + e % din]);
    if (gr.bias[l] && m.bias[l])
      for (int j = threadIdx.x; j < dout; j += blockDim.x) atomicAdd(gr.bias[l] + j, dw_s[woff + op * ip + j]);
    woff += layer_floats(md, l);
  }
}

int64_t smem_for(const MlpDims& md, bool backward, int P) {
  int64_t wfl = 0, maxd = 0, actf = 0;
  for (int l = 0; l < md.L; ++l) {
    wfl += layer_floats(md, l);
    actf += (int64_t)pad8(md.d[l]) * P;
  }
  for (int l = 0; l <= md.L; ++l) maxd = std::max<int64_t>(maxd, pad8(md.d[l]));
  const int64_t floats = backward ? (2 * wfl + actf + 2 * maxd * P) : (wfl + 2 * maxd * P);
  return floats * 4;
}

constexpr int64_t kSmemLimit = 227 * 1024;

template <int P>
cudaError_t run_forward(const FFMlp& m, const float* x, int64_t n, float* out, int64_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(mlp_forward_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int per_sm = std::max<int64_t>(1, std::min<int64_t>(4, (kSmemLimit) / std::max<int64_t>(smem, 1)));
  const int64_t want = ceil_div(n, P);
  const int blocks = (int)std::min<int64_t>(want, (int64_t)sm_count() * per_sm);
  mlp_forward_kernel<P><<<blocks, kThreads, smem, s>>>(m, x, n, out);
  return cudaGetLastError();
}

template <int P>
cudaError_t run_backward(const FFMlp& m, const float* x, int64_t n, const float* go, float* gx, const FFMlpGrad& g,
                         int64_t smem, cudaStream_t s) {
  cudaError_t e = cudaFuncSetAttribute(mlp_backward_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int per_sm = std::max<int64_t>(1, std::min<int64_t>(4, (kSmemLimit) / std::max<int64_t>(smem, 1)));
  const int64_t want = ceil_div(n, P);
  const int blocks = (int)std::min<int64_t>(want, (int64_t)sm_count() * per_sm);
  mlp_backward_kernel<P><<<blocks, kThreads, smem, s>>>(m, x, n, go, gx, g);
  return cudaGetLastError();
}

}  // namespace

int64_t mlp_smem_bytes(const FFMlp& m, bool backward, int* tile_points) {
  const MlpDims md = mlp_dims(m);
  for (int P : {128, 64, 32}) {
    const int64_t b = smem_for(md, backward, P);
    if (b <= kSmemLimit) {
      if (tile_points) *tile_points = P;
      return b;
    }
  }
  return -1;
}

cudaError_t launch_mlp_forward(const FFMlp& m, const float* x, int64_t n, float* out, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int P = 0;
  const int64_t smem = mlp_smem_bytes(m, false, &P);
  if (smem < 0) return cudaErrorInvalidConfiguration;
  if (P == 128) return run_forward<128>(m, x, n, out, smem, s);
  if (P == 64) return run_forward<64>(m, x, n, out, smem, s);
  return run_forward<32>(m, x, n, out, smem, s);
}

cudaError_t launch_mlp_backward(const FFMlp& m, const float* x, int64_t n, const float* grad_out, float* grad_x,
                                const FFMlpGrad& g, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  int P = 0;
  const int64_t smem = mlp_smem_bytes(m, true, &P);
  if (smem < 0) return cudaErrorInvalidConfiguration;
  if (P == 128) return run_backward<128>(m, x, n, grad_out, grad_x, g, smem, s);
  if (P == 64) return run_backward<64>(m, x, n, grad_out, grad_x, g, smem, s);
  return run_backward<32>(m, x, n, grad_out, grad_x, g, smem, s);
}

}  // namespace ffgb
