// MLPRender_Fea colour head (models/FactorFields.py:162-203), float32 drop-in path.
//
//   rgb = sigmoid(MLP([feat, dir, PE(feat, fea_pe), PE(dir, view_pe)]))        (:188-203)
//   PE(x, F) = [sin(x_d 2^f) for d, f] ++ [cos(x_d 2^f) for d, f], index d * F + f  (:74-79)
//   MLP: Linear + ReLU per hidden layer, the last Linear without bias, then a sigmoid.
//
// It runs on the samples whose compositing weight passed the threshold (the reference's
// feat[app_mask, 1:] and viewdirs[ray_valid_new], :879-885), listed by ff_app_emit as
// (live-sample index, ray index) pairs. The drop-in spells the reference's op sequence out
// kernel by kernel, through a caller workspace: the input rows X (positional encoding), one
// float32 GEMM per layer (bias, ReLU / sigmoid fused into its epilogue), and for the backward
// the recomputed forward followed by the transposed GEMMs: dW_l += G_l^T A_l (split over the
// samples, atomically accumulated), db_l += G_l^T 1, G_{l-1} = (G_l W_l) * [A_l > 0], and the
// chain rule through the positional encoding into dL/dfeat.
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

// One strided float32 GEMM: C(m, n) (op)= act(sum_k A(m, k) B(k, n) + bias[n]).
// A(m, k) = A[a_row(m) * sam + k * sak], B(k, n) = B[k * sbk + n * sbn],
// C(m, n) = C[c_row(m) * scm + n * scn], with a_row / c_row the optional row lists.
struct Gemm {
  int64_t M, N, K;
  const float* A;
  int64_t sam, sak;
  const int32_t* a_rows;
  const float* B;
  int64_t sbk, sbn;
  float* C;
  int64_t scm, scn;
  const int32_t* c_rows;
  const float* bias;  // [N] or NULL
  int act;            // 0 none, 1 relu, 2 sigmoid
  const float* mask;  // C(m, n) = 0 where mask[m * smm + n] <= 0 (NULL: none)
  int64_t smm;
  int atomic;         // C += value (split-K over blockIdx.z); act / mask must be off
  int64_t k_chunk;
};

constexpr int kBM = 64, kBN = 64, kBK = 16;

__global__ void __launch_bounds__(256) gemm_f32_kernel(const Gemm g) {
  __shared__ float As[kBK][kBM + 4];
  __shared__ float Bs[kBK][kBN + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * kBM, n0 = (int64_t)blockIdx.x * kBN;
  const int64_t kb = (int64_t)blockIdx.z * g.k_chunk;
  const int64_t ke = min(g.K, kb + g.k_chunk);
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int64_t k0 = kb; k0 < ke; k0 += kBK) {
    // A tile: consecutive threads walk k when A is row-major in k (sak == 1), else m
    for (int e = tid; e < kBM * kBK; e += 256) {
      const int mm = g.sak == 1 ? e / kBK : e % kBM, kk = g.sak == 1 ? e % kBK : e / kBM;
      const int64_t m = m0 + mm, k = k0 + kk;
      float v = 0.f;
      if (m < g.M && k < ke) {
        const int64_t row = g.a_rows ? (int64_t)g.a_rows[m] : m;
        v = g.A[row * g.sam + k * g.sak];
      }
      As[kk][mm] = v;
    }
    for (int e = tid; e < kBK * kBN; e += 256) {
      const int nn = g.sbn == 1 ? e % kBN : e / kBK, kk = g.sbn == 1 ? e / kBN : e % kBK;
      const int64_t k = k0 + kk, n = n0 + nn;
      Bs[kk][nn] = (k < ke && n < g.N) ? g.B[k * g.sbk + n * g.sbn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] += a[i] * b[j];
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t m = m0 + ty * 4 + i;
    if (m >= g.M) continue;
    const int64_t row = g.c_rows ? (int64_t)g.c_rows[m] : m;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t n = n0 + tx * 4 + j;
      if (n >= g.N) continue;
      float v = acc[i][j];
      if (g.bias && blockIdx.z == 0) v += g.bias[n];
      float* c = g.C + row * g.scm + n * g.scn;
      if (g.atomic) {
        atomicAdd(c, v);
      } else {
        if (g.act == 1) v = fmaxf(v, 0.f);
        else if (g.act == 2) v = 1.f / (1.f + expf(-v));
        if (g.mask && !(g.mask[m * g.smm + n] > 0.f)) v = 0.f;
        *c = v;
      }
    }
  }
}

cudaError_t gemm(const Gemm& g0, cudaStream_t s) {
  if (g0.M == 0 || g0.N == 0) return cudaSuccess;
  Gemm g = g0;
  int64_t splits = 1;
  if (g.atomic) {
    // split the reduction so that about 4 blocks per SM are busy
    const int64_t tiles = ceil_div(g.M, kBM) * ceil_div(g.N, kBN);
    splits = std::max<int64_t>(1, std::min<int64_t>(ceil_div(g.K, 256), ceil_div((int64_t)sm_count() * 4, tiles)));
  }
  g.k_chunk = ceil_div(ceil_div(g.K, splits), kBK) * kBK;
  if (g.k_chunk == 0) g.k_chunk = kBK;
  splits = std::max<int64_t>(1, ceil_div(g.K, g.k_chunk));
  const dim3 grid((unsigned)ceil_div(g.N, kBN), (unsigned)ceil_div(g.M, kBM), (unsigned)splits);
  gemm_f32_kernel<<<grid, 256, 0, s>>>(g);
  return cudaGetLastError();
}

struct PeDims {
  int C, F, V, in, ldx;
};

__host__ __device__ inline PeDims pe_dims(const FFRenderMlp& h) {
  PeDims d;
  d.C = h.in_channels;
  d.F = h.fea_pe;
  d.V = h.view_pe;
  d.in = 3 + d.C + 2 * d.V * 3 + 2 * d.F * d.C;
  d.ldx = (d.in + 3) & ~3;
  return d;
}

// X[i][k]: the head's input row of app sample i (reference order), zero padding to ldx.
__global__ void pe_forward_kernel(const PeDims d, const float* __restrict__ feat, int feat_stride, int feat_off,
                                  const float* __restrict__ rays, const int32_t* __restrict__ app_idx,
                                  const int32_t* __restrict__ app_ray, int64_t n, float* __restrict__ X) {
  const int64_t total = n * d.ldx;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / d.ldx;
    int k = (int)(e % d.ldx);
    const float* f = feat + (int64_t)app_idx[i] * feat_stride + feat_off;
    const float* dir = rays + (int64_t)app_ray[i] * 6 + 3;
    float v = 0.f;
    if (k < d.C) {
      v = f[k];
    } else if ((k -= d.C) < 3) {
      v = dir[k];
    } else if ((k -= 3) < 2 * d.C * d.F) {
      const bool cosine = k >= d.C * d.F;
      const int j = cosine ? k - d.C * d.F : k;
      const float x = f[j / d.F] * (float)(1 << (j % d.F));  // positions * 2^f, exact
      v = cosine ? cosf(x) : sinf(x);
    } else if ((k -= 2 * d.C * d.F) < 6 * d.V) {
      const bool cosine = k >= 3 * d.V;
      const int j = cosine ? k - 3 * d.V : k;
      const float x = dir[j / d.V] * (float)(1 << (j % d.V));
      v = cosine ? cosf(x) : sinf(x);
    }
    X[e] = v;
  }
}

// dL/dfeat[c] = dX[c] + sum_f 2^f (dX[sin c f] cos(x 2^f) - dX[cos c f] sin(x 2^f)), written to
// grad_feat[app_idx[i]][feat_off + c] (overwritten).
__global__ void pe_backward_kernel(const PeDims d, const float* __restrict__ feat, int feat_stride, int feat_off,
                                   const int32_t* __restrict__ app_idx, int64_t n, const float* __restrict__ dX,
                                   float* __restrict__ grad_feat) {
  const int64_t total = n * d.C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / d.C;
    const int c = (int)(e % d.C);
    const int64_t row = (int64_t)app_idx[i] * feat_stride + feat_off;
    const float x = feat[row + c];
    const float* g = dX + i * d.ldx;
    float v = g[c];
    for (int f = 0; f < d.F; ++f) {
      const float s = (float)(1 << f), xf = x * s;
      v += s * (g[d.C + 3 + c * d.F + f] * cosf(xf) - g[d.C + 3 + d.C * d.F + c * d.F + f] * sinf(xf));
    }
    grad_feat[row + c] = v;
  }
}

// dY = dL/drgb * rgb * (1 - rgb) for the app samples (grad_rgb rows at app_idx).
__global__ void sigmoid_backward_kernel(const float* __restrict__ rgb, const float* __restrict__ grad_rgb,
                                        const int32_t* __restrict__ app_idx, int64_t n, float* __restrict__ dY) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n * 3; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / 3;
    const int o = (int)(e % 3);
    const float y = rgb[e];
    dY[e] = grad_rgb[(int64_t)app_idx[i] * 3 + o] * y * (1.f - y);
  }
}

__global__ void set_one_kernel(float* p) {
  if (threadIdx.x == 0) *p = 1.f;
}

int elem_blocks(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), (int64_t)sm_count() * 8)); }

struct HeadWs {
  float *X, *H[FF_MAX_MLP_LAYERS], *Y, *dY, *G0, *G1, *dX, *one;
};

int layer_in(const FFRenderMlp& h, const PeDims& d, int l) { return l == 0 ? d.in : h.hidden_dim; }
int layer_out(const FFRenderMlp& h, int l) { return l == h.n_layers - 1 ? 3 : h.hidden_dim; }

int64_t head_ws_floats(const FFRenderMlp& h, int64_t n, HeadWs* w, float* base) {
  const PeDims d = pe_dims(h);
  const int64_t hid = ((int64_t)h.hidden_dim + 3) & ~3;
  int64_t off = 0;
  auto take = [&](int64_t floats) {
    float* p = base ? base + off : nullptr;
    off += (floats + 63) & ~int64_t(63);  // 256-byte aligned pieces
    return p;
  };
  HeadWs ws;
  ws.X = take(n * d.ldx);
  for (int l = 0; l < FF_MAX_MLP_LAYERS; ++l) ws.H[l] = (l + 1 < h.n_layers) ? take(n * hid) : nullptr;
  ws.Y = take(n * 3);
  ws.dY = take(n * 3);
  ws.G0 = take(n * std::max<int64_t>(hid, 3));
  ws.G1 = take(n * std::max<int64_t>(hid, 3));
  ws.dX = take(n * d.ldx);
  ws.one = take(1);
  if (w) *w = ws;
  return off;
}

int64_t ld_of(const FFRenderMlp& h, const PeDims& d, int l) {
  // row stride of layer l's input activation buffer
  return l == 0 ? d.ldx : (((int64_t)h.hidden_dim + 3) & ~3);
}

// Forward through the layers: X (built), H_l, and Y (rgb after the sigmoid, [n, 3]) or the rgb rows
// of out_rows (c_rows = app_idx) when y_out is given.
cudaError_t head_forward_layers(const FFRenderMlp& h, const PeDims& d, const HeadWs& w, int64_t n, float* y_out,
                                const int32_t* y_rows, cudaStream_t s) {
  for (int l = 0; l < h.n_layers; ++l) {
    const bool last = l == h.n_layers - 1;
    Gemm g = {};
    g.M = n;
    g.N = layer_out(h, l);
    g.K = layer_in(h, d, l);
    g.A = l == 0 ? w.X : w.H[l - 1];
    g.sam = ld_of(h, d, l);
    g.sak = 1;
    g.B = h.weight[l];
    g.sbk = 1;
    g.sbn = g.K;  // B(k, n) = W[n][k]
    if (last) {
      g.C = y_out ? y_out : w.Y;
      g.c_rows = y_out ? y_rows : nullptr;
      g.scm = 3;
    } else {
      g.C = w.H[l];
      g.scm = ld_of(h, d, l + 1);
    }
    g.scn = 1;
    g.bias = h.bias[l];
    g.act = last ? 2 : 1;
    const cudaError_t e = gemm(g, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

int64_t render_head_workspace_bytes(const FFRenderMlp& h, int64_t n) { return head_ws_floats(h, n, nullptr, nullptr) * 4; }

cudaError_t launch_render_head_forward(const FFRenderMlp& h, const float* feat, int feat_stride, int feat_off,
                                       const float* rays, const int32_t* app_idx, const int32_t* app_ray, int64_t n,
                                       float* rgb_rows, void* workspace, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const PeDims d = pe_dims(h);
  HeadWs w;
  head_ws_floats(h, n, &w, static_cast<float*>(workspace));
  pe_forward_kernel<<<elem_blocks(n * d.ldx), 256, 0, s>>>(d, feat, feat_stride, feat_off, rays, app_idx, app_ray, n,
                                                          w.X);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return head_forward_layers(h, d, w, n, rgb_rows, app_idx, s);
}

cudaError_t launch_render_head_backward(const FFRenderMlp& h, const float* feat, int feat_stride, int feat_off,
                                        const float* rays, const int32_t* app_idx, const int32_t* app_ray, int64_t n,
                                        const float* grad_rgb_rows, float* grad_feat, const FFMlpGrad& gr,
                                        void* workspace, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const PeDims d = pe_dims(h);
  HeadWs w;
  head_ws_floats(h, n, &w, static_cast<float*>(workspace));
  pe_forward_kernel<<<elem_blocks(n * d.ldx), 256, 0, s>>>(d, feat, feat_stride, feat_off, rays, app_idx, app_ray, n,
                                                          w.X);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if ((e = head_forward_layers(h, d, w, n, nullptr, nullptr, s)) != cudaSuccess) return e;
  sigmoid_backward_kernel<<<elem_blocks(n * 3), 256, 0, s>>>(w.Y, grad_rgb_rows, app_idx, n, w.dY);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  set_one_kernel<<<1, 32, 0, s>>>(w.one);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  const float* G = w.dY;
  int64_t ldg = 3;
  float* bufs[2] = {w.G0, w.G1};
  for (int l = h.n_layers - 1; l >= 0; --l) {
    const int64_t din = layer_in(h, d, l), dout = layer_out(h, l);
    const float* Aact = l == 0 ? w.X : w.H[l - 1];
    const int64_t lda = ld_of(h, d, l);
    if (gr.weight[l]) {  // dW_l[j][k] += sum_i G[i][j] A[i][k]
      Gemm g = {};
      g.M = dout; g.N = din; g.K = n;
      g.A = G; g.sam = 1; g.sak = ldg;
      g.B = Aact; g.sbk = lda; g.sbn = 1;
      g.C = gr.weight[l]; g.scm = din; g.scn = 1;
      g.atomic = 1;
      if ((e = gemm(g, s)) != cudaSuccess) return e;
    }
    if (gr.bias[l] && h.bias[l]) {  // db_l[j] += sum_i G[i][j]
      Gemm g = {};
      g.M = dout; g.N = 1; g.K = n;
      g.A = G; g.sam = 1; g.sak = ldg;
      g.B = w.one; g.sbk = 0; g.sbn = 0;
      g.C = gr.bias[l]; g.scm = 1; g.scn = 1;
      g.atomic = 1;
      if ((e = gemm(g, s)) != cudaSuccess) return e;
    }
    // G_{l-1}[i][k] = sum_j G[i][j] W_l[j][k], masked by the layer input's ReLU (hidden layers)
    float* out = l == 0 ? w.dX : bufs[l & 1];
    const int64_t ldo = l == 0 ? d.ldx : ld_of(h, d, l);
    Gemm g = {};
    g.M = n; g.N = din; g.K = dout;
    g.A = G; g.sam = ldg; g.sak = 1;
    g.B = h.weight[l]; g.sbk = din; g.sbn = 1;
    g.C = out; g.scm = ldo; g.scn = 1;
    if (l > 0) {
      g.mask = Aact;
      g.smm = lda;
    }
    if ((e = gemm(g, s)) != cudaSuccess) return e;
    G = out;
    ldg = ldo;
  }
  pe_backward_kernel<<<elem_blocks(n * d.C), 256, 0, s>>>(d, feat, feat_stride, feat_off, app_idx, n, w.dX,
                                                          grad_feat);
  return cudaGetLastError();
}

}  // namespace ffgb
