// Occupancy-volume maintenance (updateAlphaMask, models/FactorFields.py:757-793): from the dense
// alpha volume [D][H][W] (z, y, x) to the occupancy bitfield the ray marcher reads.
//
//   pool      3x3x3 max-pool (stride 1, padding 1: out-of-volume neighbours ignored, NaN
//             propagates like ATen's max_pool3d) of alpha clamped to [0, 1], then >= threshold
//   label     connected components of the occupied voxels, 6-connectivity (skimage
//             remove_small_objects with connectivity=1, :774): lock-free union-find. Each voxel
//             unites with its occupied -x, -y, -z neighbours; a root is always hooked under the
//             smaller root (parent[v] <= v, so no cycles), find() halves paths.
//   size      voxels per component (atomics on the root)
//   filter    keep the voxels of components with at least min_size voxels (the reference removes
//             the smaller ones), pack 32 voxels per word (bit k of word w = voxel 32 w + k),
//             optional 0/1 float volume, and the index bounding box of the kept voxels
//
// The result is unique whatever order the unions happen in. Every loop that retries
// (find, unite) has an iteration limit; running out sets a status word instead of spinning.
#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {

constexpr int kOccThreads = 256;
constexpr int kFindLimit = 1 << 22;   // path steps in one find (a path is at most V long)
constexpr int kUniteLimit = 1 << 16;  // CAS retries in one unite
constexpr int kNone = -1;

struct Vol {
  int d, h, w;
  int64_t n;
};

__device__ __forceinline__ float clamp01(float a) { return a != a ? a : fminf(fmaxf(a, 0.f), 1.f); }

__global__ void __launch_bounds__(kOccThreads) occ_pool_kernel(const float* __restrict__ alpha, const Vol v,
                                                               float threshold, int32_t* __restrict__ parent) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % v.w), y = (int)((i / v.w) % v.h), z = (int)(i / ((int64_t)v.w * v.h));
    float m = -INFINITY;
    bool nan = false;
    for (int dz = -1; dz <= 1; ++dz) {
      const int zz = z + dz;
      if (zz < 0 || zz >= v.d) continue;
      for (int dy = -1; dy <= 1; ++dy) {
        const int yy = y + dy;
        if (yy < 0 || yy >= v.h) continue;
        for (int dx = -1; dx <= 1; ++dx) {
          const int xx = x + dx;
          if (xx < 0 || xx >= v.w) continue;
          const float a = clamp01(alpha[((int64_t)zz * v.h + yy) * v.w + xx]);
          nan = nan || (a != a);
          m = fmaxf(m, a);
        }
      }
    }
    parent[i] = (!nan && m >= threshold) ? (int32_t)i : kNone;
  }
}

__device__ __forceinline__ int32_t find_root(int32_t* parent, int32_t a, int* status) {
  for (int it = 0; it < kFindLimit; ++it) {
    const int32_t p = parent[a];
    if (p == a) return a;
    const int32_t g = parent[p];
    if (g != p) parent[a] = g;  // path halving; g <= p < a keeps parent[v] <= v
    a = g;
  }
  atomicExch(status, 1);
  return a;
}

__device__ __forceinline__ void unite(int32_t* parent, int32_t a, int32_t b, int* status) {
  for (int it = 0; it < kUniteLimit; ++it) {
    a = find_root(parent, a, status);
    b = find_root(parent, b, status);
    if (a == b) return;
    if (a < b) {
      const int32_t t = a;
      a = b;
      b = t;
    }
    if (atomicCAS(parent + a, a, b) == a) return;  // hooked the larger root under the smaller
  }
  atomicExch(status, 2);
}

__global__ void __launch_bounds__(kOccThreads) occ_unite_kernel(int32_t* __restrict__ parent, const Vol v,
                                                                int* status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (parent[i] == kNone) continue;
    const int x = (int)(i % v.w), y = (int)((i / v.w) % v.h), z = (int)(i / ((int64_t)v.w * v.h));
    if (x > 0 && parent[i - 1] != kNone) unite(parent, (int32_t)i, (int32_t)(i - 1), status);
    if (y > 0 && parent[i - v.w] != kNone) unite(parent, (int32_t)i, (int32_t)(i - v.w), status);
    if (z > 0 && parent[i - (int64_t)v.w * v.h] != kNone)
      unite(parent, (int32_t)i, (int32_t)(i - (int64_t)v.w * v.h), status);
  }
}

__global__ void __launch_bounds__(kOccThreads) occ_size_kernel(int32_t* __restrict__ parent, const Vol v,
                                                               int32_t* __restrict__ size, int* status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.n; i += (int64_t)gridDim.x * blockDim.x) {
    if (parent[i] == kNone) continue;
    const int32_t r = find_root(parent, (int32_t)i, status);
    atomicAdd(size + r, 1);
  }
}

// Warp per 32 consecutive voxels: ballot -> one bitfield word.
__global__ void __launch_bounds__(kOccThreads) occ_filter_kernel(int32_t* __restrict__ parent, const Vol v,
                                                                 const int32_t* __restrict__ size, int min_size,
                                                                 int32_t* __restrict__ bits, float* __restrict__ vol,
                                                                 int32_t* __restrict__ bbox, int* status) {
  const int lane = threadIdx.x & 31;
  const int64_t words = ceil_div(v.n, 32);
  const int64_t wstep = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; w < words; w += wstep) {
    const int64_t i = w * 32 + lane;
    bool keep = false;
    if (i < v.n && parent[i] != kNone) {
      keep = min_size <= 1 || size[find_root(parent, (int32_t)i, status)] >= min_size;
    }
    const unsigned word = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) bits[w] = (int32_t)word;
    if (i < v.n && vol) vol[i] = keep ? 1.f : 0.f;
    if (keep) {
      const int x = (int)(i % v.w), y = (int)((i / v.w) % v.h), z = (int)(i / ((int64_t)v.w * v.h));
      atomicMin(bbox + 0, x); atomicMin(bbox + 1, y); atomicMin(bbox + 2, z);
      atomicMax(bbox + 3, x); atomicMax(bbox + 4, y); atomicMax(bbox + 5, z);
    }
  }
}

__global__ void occ_init_kernel(int32_t* __restrict__ bbox, int* status) {
  if (threadIdx.x < 3) bbox[threadIdx.x] = 0x7fffffff;
  else if (threadIdx.x < 6) bbox[threadIdx.x] = -1;
  else if (threadIdx.x == 6) *status = 0;
}

int occ_blocks(int64_t n) {
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kOccThreads), (int64_t)sm_count() * 16));
}

}  // namespace

int64_t occupancy_workspace_bytes(int64_t voxels) { return 2 * ((voxels * 4 + 255) & ~int64_t(255)) + 256; }

cudaError_t launch_occupancy_mask(const float* alpha, int d, int h, int w, float threshold, int min_size,
                                  int32_t* bits, float* vol, int32_t* bbox, void* workspace, int* status_host,
                                  cudaStream_t st) {
  const Vol v{d, h, w, (int64_t)d * h * w};
  unsigned char* ws = static_cast<unsigned char*>(workspace);
  int32_t* parent = reinterpret_cast<int32_t*>(ws);
  int32_t* size = reinterpret_cast<int32_t*>(ws + ((v.n * 4 + 255) & ~int64_t(255)));
  int* status = reinterpret_cast<int*>(ws + 2 * ((v.n * 4 + 255) & ~int64_t(255)));
  occ_init_kernel<<<1, 32, 0, st>>>(bbox, status);
  const int blocks = occ_blocks(v.n);
  occ_pool_kernel<<<blocks, kOccThreads, 0, st>>>(alpha, v, threshold, parent);
  if (min_size > 1) {
    cudaError_t e = cudaMemsetAsync(size, 0, v.n * 4, st);
    if (e != cudaSuccess) return e;
    occ_unite_kernel<<<blocks, kOccThreads, 0, st>>>(parent, v, status);
    occ_size_kernel<<<blocks, kOccThreads, 0, st>>>(parent, v, size, status);
  }
  occ_filter_kernel<<<occ_blocks(ceil_div(v.n, 32) * 32), kOccThreads, 0, st>>>(parent, v, size, min_size, bits, vol,
                                                                                bbox, status);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cudaMemcpyAsync(status_host, status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return e;
  return cudaStreamSynchronize(st);
}

}  // namespace ffgb
