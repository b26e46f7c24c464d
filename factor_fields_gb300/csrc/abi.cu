// extern "C" entry points of libffgb.so (declared in include/ff_native.h): argument
// validation, error reporting and dispatch to the kernel launchers.
#include <atomic>
#include <cstdio>
#include <string>

#include "ff_common.cuh"
#include "ff_internal.h"

namespace ffgb {

namespace {
thread_local std::string g_last_error;
}

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

// SM count per device ordinal, looked up on first use. The cache entries are atomics: two
// threads that race on the first lookup both store the same value.
int sm_count() {
  static std::atomic<int> cached[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  int v = cached[dev].load(std::memory_order_relaxed);
  if (v == 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 148;
    cached[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

static int cuda_status(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return FF_OK;
  return set_error(FF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

static bool aligned(const void* p, int bytes) { return (reinterpret_cast<uintptr_t>(p) % bytes) == 0; }

// Validates an FFField; returns FF_OK or an error code with ff_last_error set.
// need_grids false: the descriptor alone (entries that touch no grid values)
static int validate_field(const FFField* f, const void* basis, const void* coeff, bool need_grids = true) {
  if (!f) return set_error(FF_ERR_ARG, "field descriptor is NULL");
  if (!(f->basis_dim == 2 || f->basis_dim == 3)) return set_error(FF_ERR_ARG, "basis_dim must be 2 or 3");
  if (!(f->coord_dim == f->basis_dim || (f->basis_dim == 2 && f->coord_dim == 3)))
    return set_error(FF_ERR_UNSUPPORTED, "coord_dim must equal basis_dim (or be 3 with a 2-D basis: 'images' mode)");
  if (f->n_levels < 1 || f->n_levels > FF_MAX_LEVELS) return set_error(FF_ERR_ARG, "n_levels out of range 1..8");
  if (f->mapping != FF_MAP_SAWTOOTH && f->mapping != FF_MAP_TRIANGLE)
    return set_error(FF_ERR_UNSUPPORTED, "basis_mapping must be sawtooth or triangle");
  if ((f->basis_interp != FF_INTERP_LINEAR && f->basis_interp != FF_INTERP_NEAREST) ||
      (f->coeff_interp != FF_INTERP_LINEAR && f->coeff_interp != FF_INTERP_NEAREST))
    return set_error(FF_ERR_ARG, "interpolation mode must be linear or nearest");
  if (f->param_dtype != FF_F32 && f->param_dtype != FF_BF16) return set_error(FF_ERR_ARG, "param_dtype must be F32 or BF16");
  const int es = f->param_dtype == FF_F32 ? 4 : 2;
  if (need_grids && (!basis || !coeff)) return set_error(FF_ERR_ARG, "basis/coeff pointer is NULL");
  if (need_grids && (!aligned(basis, 16) || !aligned(coeff, 16)))
    return set_error(FF_ERR_ALIGN, "basis/coeff must be 16-byte aligned");
  int sum = 0;
  for (int l = 0; l < f->n_levels; ++l) {
    const int c = f->level_channels[l], v = f->level_vec[l];
    if (c < 1 || f->level_reso[l] < 1 || f->level_stride[l] < c) return set_error(FF_ERR_ARG, "bad level channels/reso/stride");
    if (!(v == 1 || v == 2 || v == 4) || c % v || f->level_stride[l] % v || f->level_offset[l] % v || sum % v ||
        f->coeff_stride % v)
      return set_error(FF_ERR_ALIGN, "level_vec does not divide channels/stride/offset of level " + std::to_string(l));
    if (f->level_scale[l] <= 0.f) return set_error(FF_ERR_ARG, "level_scale must be > 0");
    int64_t cells = 1;
    for (int k = 0; k < f->basis_dim; ++k) cells *= f->level_reso[l];
    if (cells > (1ll << 31) / 8 || cells * f->level_stride[l] >= (1ll << 31))  // 32-bit corner offsets
      return set_error(FF_ERR_SIZE, "basis level too large");
    sum += c;
  }
  if (sum != f->n_feat) return set_error(FF_ERR_ARG, "n_feat != sum(level_channels)");
  if (f->coeff_stride < f->n_feat) return set_error(FF_ERR_ARG, "coeff_stride < n_feat");
  int64_t cells = 1;
  for (int k = 0; k < f->coord_dim; ++k) {
    if (f->coeff_reso[k] < 1) return set_error(FF_ERR_ARG, "coeff_reso must be >= 1");
    cells *= f->coeff_reso[k];
  }
  if (cells > (1ll << 31) / 8 || cells * f->coeff_stride >= (1ll << 31))
    return set_error(FF_ERR_SIZE, "coefficient grid too large");
  (void)es;
  return FF_OK;
}

static int validate_mlp(const FFMlp* m) {
  if (!m) return set_error(FF_ERR_ARG, "mlp descriptor is NULL");
  if (m->n_layers < 1 || m->n_layers > FF_MAX_MLP_LAYERS) return set_error(FF_ERR_UNSUPPORTED, "n_layers must be 1..4");
  if (m->in_dim < 1 || m->out_dim < 1 || (m->n_layers > 1 && m->hidden_dim < 1))
    return set_error(FF_ERR_ARG, "bad MLP dims");
  for (int l = 0; l < m->n_layers; ++l)
    if (!m->weight[l]) return set_error(FF_ERR_ARG, "MLP weight pointer is NULL");
  return FF_OK;
}

}  // namespace ffgb

using namespace ffgb;

extern "C" {

int ff_abi_version(void) { return FF_ABI_VERSION; }

const char* ff_last_error(void) { return g_last_error.c_str(); }

int64_t ff_struct_size(int32_t which) {
  switch (which) {
    case 0: return (int64_t)sizeof(FFField);
    case 1: return (int64_t)sizeof(FFMlp);
    case 2: return (int64_t)sizeof(FFMlpGrad);
    case 3: return (int64_t)sizeof(FFRender);
    case 4: return (int64_t)sizeof(FFProposal);
    case 5: return (int64_t)sizeof(FFAdamParam);
    case 6: return (int64_t)sizeof(FFRenderMlp);
    default: return -1;
  }
}

int ff_device_info(int32_t* sms, int32_t* cc) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetDevice");
  int ma = 0, mi = 0;
  cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, dev);
  if (sms) *sms = sm_count();
  if (cc) *cc = ma * 10 + mi;
  return FF_OK;
}

int ff_field_forward(const FFField* f, const void* basis, const void* coeff, const float* x, int64_t n, float* feats,
                     float* coeff_out, float* basis_out, void* stream) {
  int rc = validate_field(f, basis, coeff);
  if (rc) return rc;
  if (n < 0 || (n > 0 && !x)) return set_error(FF_ERR_ARG, "bad points pointer or count");
  return cuda_status(launch_field_forward(*f, basis, coeff, x, n, feats, coeff_out, basis_out, (cudaStream_t)stream),
                     "ff_field_forward launch");
}

int ff_field_backward(const FFField* f, const void* basis, const void* coeff, const float* x, int64_t n,
                      const float* grad_feats, const float* grad_coeff_out, const float* grad_basis_out,
                      float* grad_basis, float* grad_coeff_grid, void* stream) {
  int rc = validate_field(f, basis, coeff);
  if (rc) return rc;
  if (n < 0 || (n > 0 && !x)) return set_error(FF_ERR_ARG, "bad points pointer or count");
  if ((grad_basis && !aligned(grad_basis, 16)) || (grad_coeff_grid && !aligned(grad_coeff_grid, 16)))
    return set_error(FF_ERR_ALIGN, "gradient buffers must be 16-byte aligned");
  return cuda_status(launch_field_backward(*f, basis, coeff, x, n, grad_feats, grad_coeff_out, grad_basis_out,
                                           grad_basis, grad_coeff_grid, (cudaStream_t)stream),
                     "ff_field_backward launch");
}

int ff_mlp_forward(const FFMlp* m, const float* x, int64_t n, float* out, void* stream) {
  int rc = validate_mlp(m);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!x || !out))) return set_error(FF_ERR_ARG, "bad x/out pointer or count");
  if (mlp_smem_bytes(*m, false, nullptr) < 0) return set_error(FF_ERR_UNSUPPORTED, "MLP too large for shared memory");
  return cuda_status(launch_mlp_forward(*m, x, n, out, (cudaStream_t)stream), "ff_mlp_forward launch");
}

int ff_mlp_backward(const FFMlp* m, const float* x, int64_t n, const float* grad_out, float* grad_x, const FFMlpGrad* g,
                    void* stream) {
  int rc = validate_mlp(m);
  if (rc) return rc;
  if (n < 0 || (n > 0 && (!x || !grad_out))) return set_error(FF_ERR_ARG, "bad x/grad_out pointer or count");
  if (mlp_smem_bytes(*m, true, nullptr) < 0) return set_error(FF_ERR_UNSUPPORTED, "MLP too large for shared memory");
  FFMlpGrad none = {};
  return cuda_status(launch_mlp_backward(*m, x, n, grad_out, grad_x, g ? *g : none, (cudaStream_t)stream),
                     "ff_mlp_backward launch");
}

static int validate_render(const FFRender* r, const float* rays, int64_t n) {
  if (!r) return set_error(FF_ERR_ARG, "render descriptor is NULL");
  if (n < 0 || (n > 0 && !rays)) return set_error(FF_ERR_ARG, "bad rays pointer or count");
  if (r->n_samples < 1 || r->n_samples > (1 << 20)) return set_error(FF_ERR_ARG, "n_samples must be 1..2^20");
  if (!(r->step > 0.f)) return set_error(FF_ERR_ARG, "step must be > 0");
  if (r->density_act != 0 && r->density_act != 1) return set_error(FF_ERR_ARG, "density_act must be 0 or 1");
  if (r->occ_bits) {
    int64_t cells = 1;
    for (int k = 0; k < 3; ++k) {
      if (r->occ_reso[k] < 1) return set_error(FF_ERR_ARG, "occupancy resolution must be >= 1");
      cells *= r->occ_reso[k];
    }
    if (cells > (1ll << 31)) return set_error(FF_ERR_SIZE, "occupancy volume too large");
  }
  return FF_OK;
}

static int validate_fused(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, const float* x,
                          int64_t n) {
  int rc = validate_field(f, basis, coeff);
  if (rc) return rc;
  rc = validate_mlp(m);
  if (rc) return rc;
  if (const char* why = fused_unsupported(*f, *m)) return set_error(FF_ERR_UNSUPPORTED, why);
  if (n < 0 || (n > 0 && !x)) return set_error(FF_ERR_ARG, "bad points pointer or count");
  return FF_OK;
}

int ff_field_mlp_forward(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, const float* x,
                         int64_t n, float* out, void* stream) {
  int rc = validate_fused(f, basis, coeff, m, x, n);
  if (rc) return rc;
  if (n > 0 && !out) return set_error(FF_ERR_ARG, "out is NULL");
  return cuda_status(launch_fused_forward(*f, basis, coeff, *m, x, n, out, (cudaStream_t)stream),
                     "ff_field_mlp_forward launch");
}

int ff_field_render_fixed(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, const FFRender* r,
                          const float* rays, const float* xyz, const float* zd, int64_t n_rays, int32_t n_fine,
                          float* rgb, float* depth, void* stream) {
  if (n_fine != 32 && n_fine != 64 && n_fine != 128)
    return set_error(FF_ERR_UNSUPPORTED, "ff_field_render_fixed: n_fine must be 32, 64 or 128");
  if (n_rays < 0 || n_rays > (int64_t(1) << 40)) return set_error(FF_ERR_ARG, "bad ray count");
  int rc = validate_fused(f, basis, coeff, m, xyz, n_rays * n_fine);
  if (rc) return rc;
  if (m->out_dim != 28 || f->coord_dim != 3)
    return set_error(FF_ERR_UNSUPPORTED,
                     "ff_field_render_fixed composites 3-D points with a 28-wide head (density + degree-2 SH colour)");
  rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!zd || !rgb)) return set_error(FF_ERR_ARG, "zd/rgb are NULL");
  if (!aligned(zd, 8)) return set_error(FF_ERR_ALIGN, "zd must be 8-byte aligned");
  return cuda_status(launch_fused_render_fixed(*f, basis, coeff, *m, *r, rays, xyz, zd, n_rays, n_fine, rgb, depth,
                                               (cudaStream_t)stream),
                     "ff_field_render_fixed launch");
}

int ff_field_mlp_backward(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, const float* x,
                          int64_t n, const float* grad_out, float* grad_basis, float* grad_coeff_grid,
                          const FFMlpGrad* g, void* stream) {
  int rc = validate_fused(f, basis, coeff, m, x, n);
  if (rc) return rc;
  if (n > 0 && !grad_out) return set_error(FF_ERR_ARG, "grad_out is NULL");
  if (!grad_basis || !grad_coeff_grid || !aligned(grad_basis, 16) || !aligned(grad_coeff_grid, 16))
    return set_error(FF_ERR_ARG, "grid gradient buffers must be non-NULL and 16-byte aligned");
  FFMlpGrad none = {};
  return cuda_status(launch_fused_backward(*f, basis, coeff, *m, x, n, grad_out, grad_basis, grad_coeff_grid,
                                           g ? *g : none, (cudaStream_t)stream),
                     "ff_field_mlp_backward launch");
}

int ff_field_mlp_forward_counted(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                 const float* x, int64_t n_max, const int64_t* n_dev, float* out, void* stream) {
  int rc = validate_fused(f, basis, coeff, m, x, n_max);
  if (rc) return rc;
  if (n_max > 0 && (!out || !n_dev)) return set_error(FF_ERR_ARG, "out / n_dev is NULL");
  if (!aligned(n_dev, 8)) return set_error(FF_ERR_ALIGN, "n_dev must be 8-byte aligned");
  return cuda_status(launch_fused_forward(*f, basis, coeff, *m, x, n_max, out, (cudaStream_t)stream, n_dev),
                     "ff_field_mlp_forward_counted launch");
}

int ff_field_mlp_backward_counted(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                  const float* x, int64_t n_max, const int64_t* n_dev, const float* grad_out,
                                  float* grad_basis, float* grad_coeff_grid, const FFMlpGrad* g, void* stream) {
  int rc = validate_fused(f, basis, coeff, m, x, n_max);
  if (rc) return rc;
  if (n_max > 0 && (!grad_out || !n_dev)) return set_error(FF_ERR_ARG, "grad_out / n_dev is NULL");
  if (!aligned(n_dev, 8)) return set_error(FF_ERR_ALIGN, "n_dev must be 8-byte aligned");
  if (!grad_basis || !grad_coeff_grid || !aligned(grad_basis, 16) || !aligned(grad_coeff_grid, 16))
    return set_error(FF_ERR_ARG, "grid gradient buffers must be non-NULL and 16-byte aligned");
  FFMlpGrad none = {};
  return cuda_status(launch_fused_backward(*f, basis, coeff, *m, x, n_max, grad_out, grad_basis, grad_coeff_grid,
                                           g ? *g : none, (cudaStream_t)stream, n_dev),
                     "ff_field_mlp_backward_counted launch");
}

int ff_field_fit_step(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, const float* x,
                      const float* target, int64_t n, int32_t loss_kind, float loss_scale, float* loss_sum,
                      float* grad_basis, float* grad_coeff_grid, const FFMlpGrad* g, void* stream) {
  int rc = validate_fused(f, basis, coeff, m, x, n);
  if (rc) return rc;
  if (n > 0 && !target) return set_error(FF_ERR_ARG, "target is NULL");
  if (loss_kind != FF_LOSS_L1 && loss_kind != FF_LOSS_MSE) return set_error(FF_ERR_ARG, "loss_kind must be L1 or MSE");
  if (!grad_basis || !grad_coeff_grid || !aligned(grad_basis, 16) || !aligned(grad_coeff_grid, 16))
    return set_error(FF_ERR_ARG, "grid gradient buffers must be non-NULL and 16-byte aligned");
  FFMlpGrad none = {};
  return cuda_status(launch_fused_fit(*f, basis, coeff, *m, x, target, n, loss_kind, loss_scale, loss_sum,
                                      grad_basis, grad_coeff_grid, g ? *g : none, (cudaStream_t)stream),
                     "ff_field_fit_step launch");
}

int64_t ff_field_fit_binned_workspace_bytes(const FFField* f, int64_t n, int32_t out_dim) {
  if (!f || n < 0 || out_dim < 1 || f->coord_dim < 2 || f->coord_dim > 3) return FF_ERR_ARG;
  const int64_t keys = fit_bin_keys(*f);
  if (keys < 1 || keys > (int64_t(1) << 30)) return FF_ERR_UNSUPPORTED;
  return fit_bin_workspace_bytes(*f, n, out_dim);
}

// Checks shared by the binned fit entries: the binning half (x, target, zeroing targets) and the
// fit half (loss, gradient buffers); both need a large enough, aligned workspace.
static int validate_fit_bin(const FFField* f, const FFMlp* m, const float* x, const float* target, int64_t n,
                            float* grad_basis, float* grad_coeff_grid, int32_t flags, const void* workspace,
                            int64_t workspace_bytes) {
  int rc = validate_mlp(m);
  if (rc) return rc;
  if (n < 0 || (n > 0 && !x)) return set_error(FF_ERR_ARG, "bad points pointer or count");
  if (n > 0 && !target) return set_error(FF_ERR_ARG, "target is NULL");
  if (flags & ~(FF_FIT_ZERO_GRADS | FF_FIT_HOST_BATCH)) return set_error(FF_ERR_ARG, "unknown flags");
  if ((flags & FF_FIT_ZERO_GRADS) &&
      (!grad_basis || !grad_coeff_grid || !aligned(grad_basis, 16) || !aligned(grad_coeff_grid, 16)))
    return set_error(FF_ERR_ARG, "grid gradient buffers must be non-NULL and 16-byte aligned");
  const int64_t need = ff_field_fit_binned_workspace_bytes(f, n, m->out_dim);
  if (need < 0) return set_error((int)need, "coefficient grid too large to bin by cell");
  if (!workspace) return set_error(FF_ERR_ARG, "workspace is NULL");
  if (workspace_bytes < need) return set_error(FF_ERR_SIZE, "workspace smaller than ff_field_fit_binned_workspace_bytes");
  if (!aligned(workspace, 256)) return set_error(FF_ERR_ALIGN, "workspace must be 256-byte aligned");
  return FF_OK;
}

static int validate_fit_on_bins(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, int64_t n,
                                int32_t loss_kind, float* grad_basis, float* grad_coeff_grid, int32_t flags,
                                const void* workspace, int64_t workspace_bytes) {
  int rc = validate_fused(f, basis, coeff, m, static_cast<const float*>(workspace), n);
  if (rc) return rc;
  if (loss_kind != FF_LOSS_L1 && loss_kind != FF_LOSS_MSE) return set_error(FF_ERR_ARG, "loss_kind must be L1 or MSE");
  if (!grad_basis || !grad_coeff_grid || !aligned(grad_basis, 16) || !aligned(grad_coeff_grid, 16))
    return set_error(FF_ERR_ARG, "grid gradient buffers must be non-NULL and 16-byte aligned");
  if (flags & ~(FF_FIT_MEAN_LOSS | FF_FIT_LEVEL0_SHARED)) return set_error(FF_ERR_ARG, "unknown flags");
  const int64_t need = ff_field_fit_binned_workspace_bytes(f, n, m->out_dim);
  if (need < 0) return set_error((int)need, "coefficient grid too large to bin by cell");
  if (!workspace) return set_error(FF_ERR_ARG, "workspace is NULL");
  if (workspace_bytes < need) return set_error(FF_ERR_SIZE, "workspace smaller than ff_field_fit_binned_workspace_bytes");
  if (!aligned(workspace, 256)) return set_error(FF_ERR_ALIGN, "workspace must be 256-byte aligned");
  return FF_OK;
}

int ff_field_fit_step_binned(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, const float* x,
                             const float* target, int64_t n, int32_t loss_kind, float loss_scale, float* loss_sum,
                             float* grad_basis, float* grad_coeff_grid, const FFMlpGrad* g, int32_t flags,
                             void* workspace, int64_t workspace_bytes, void* stream) {
  if (flags & ~(FF_FIT_ZERO_GRADS | FF_FIT_MEAN_LOSS | FF_FIT_LEVEL0_SHARED | FF_FIT_HOST_BATCH))
    return set_error(FF_ERR_ARG, "unknown flags");
  int rc = validate_fit_on_bins(f, basis, coeff, m, n, loss_kind, grad_basis, grad_coeff_grid,
                                flags & (FF_FIT_MEAN_LOSS | FF_FIT_LEVEL0_SHARED), workspace, workspace_bytes);
  if (rc) return rc;
  rc = validate_fit_bin(f, m, x, target, n, grad_basis, grad_coeff_grid, flags & (FF_FIT_ZERO_GRADS | FF_FIT_HOST_BATCH),
                        workspace, workspace_bytes);
  if (rc) return rc;
  if ((flags & FF_FIT_HOST_BATCH) &&
      cuda_status(fit_bin_stage_host(*f, &x, &target, m->out_dim, n, workspace, (cudaStream_t)stream),
                  "ff_field_fit_step_binned host batch copy"))
    return FF_ERR_CUDA;
  FFMlpGrad none = {};
  return cuda_status(launch_fused_fit_binned(*f, basis, coeff, *m, x, target, n, loss_kind, loss_scale, loss_sum,
                                             grad_basis, grad_coeff_grid, g ? *g : none, workspace,
                                             (flags & FF_FIT_ZERO_GRADS) != 0,
                                             (flags & FF_FIT_MEAN_LOSS) ? loss_scale : 1.f,
                                             (flags & FF_FIT_LEVEL0_SHARED) != 0, (cudaStream_t)stream),
                     "ff_field_fit_step_binned launch");
}

int ff_field_fit_bin(const FFField* f, const FFMlp* m, const float* x, const float* target, int64_t n,
                     float* loss_sum, float* grad_basis, float* grad_coeff_grid, const FFMlpGrad* g, int32_t flags,
                     void* workspace, int64_t workspace_bytes, void* stream) {
  int rc = validate_field(f, nullptr, nullptr, /*need_grids=*/false);
  if (rc) return rc;
  rc = validate_fit_bin(f, m, x, target, n, grad_basis, grad_coeff_grid, flags, workspace, workspace_bytes);
  if (rc) return rc;
  if ((flags & FF_FIT_HOST_BATCH) &&
      cuda_status(fit_bin_stage_host(*f, &x, &target, m->out_dim, n, workspace, (cudaStream_t)stream),
                  "ff_field_fit_bin host batch copy"))
    return FF_ERR_CUDA;
  FFMlpGrad none = {};
  return cuda_status(launch_fit_bin_phase(*f, *m, x, target, n, loss_sum, grad_basis, grad_coeff_grid, g ? *g : none,
                                          workspace, (flags & FF_FIT_ZERO_GRADS) != 0, (cudaStream_t)stream),
                     "ff_field_fit_bin launch");
}

int ff_field_fit_step_on_bins(const FFField* f, const void* basis, const void* coeff, const FFMlp* m, int64_t n,
                              int32_t loss_kind, float loss_scale, float* loss_sum, float* grad_basis,
                              float* grad_coeff_grid, const FFMlpGrad* g, int32_t flags, const void* workspace,
                              int64_t workspace_bytes, void* stream) {
  int rc = validate_fit_on_bins(f, basis, coeff, m, n, loss_kind, grad_basis, grad_coeff_grid, flags, workspace,
                                workspace_bytes);
  if (rc) return rc;
  FFMlpGrad none = {};
  return cuda_status(launch_fit_on_bins(*f, basis, coeff, *m, n, loss_kind, loss_scale, loss_sum, grad_basis,
                                        grad_coeff_grid, g ? *g : none, workspace,
                                        (flags & FF_FIT_MEAN_LOSS) ? loss_scale : 1.f,
                                        (flags & FF_FIT_LEVEL0_SHARED) != 0, (cudaStream_t)stream),
                     "ff_field_fit_step_on_bins launch");
}

int ff_zero_f32(float* const* ptrs, const int64_t* counts, int32_t n_buffers, void* stream) {
  if (n_buffers < 0 || (n_buffers > 0 && (!ptrs || !counts))) return set_error(FF_ERR_ARG, "bad buffer list");
  for (int b = 0; b < n_buffers; ++b)
    if (counts[b] < 0 || (counts[b] > 0 && !ptrs[b])) return set_error(FF_ERR_ARG, "NULL buffer or negative count");
  return cuda_status(launch_zero_buffers(ptrs, counts, n_buffers, (cudaStream_t)stream), "ff_zero_f32 launch");
}

static int validate_adam(const FFAdamParam* params, int32_t n_params, float beta1, float beta2, float eps,
                         int32_t flags, bool host_schedule) {
  if (n_params < 0 || (n_params > 0 && !params)) return set_error(FF_ERR_ARG, "bad parameter list");
  if (flags & ~FF_ADAM_ZERO_GRAD) return set_error(FF_ERR_ARG, "unknown flags");
  if (!(beta1 >= 0.f && beta1 < 1.f && beta2 >= 0.f && beta2 < 1.f && eps >= 0.f))
    return set_error(FF_ERR_ARG, "betas must be in [0, 1) and eps >= 0");
  for (int b = 0; b < n_params; ++b) {
    const FFAdamParam& q = params[b];
    if (q.n < 0 || (q.n > 0 && (!q.param || !q.grad || !q.exp_avg || !q.exp_avg_sq)))
      return set_error(FF_ERR_ARG, "parameter " + std::to_string(b) + ": NULL buffer or negative size");
    if (host_schedule && q.n > 0 && q.step < 1) return set_error(FF_ERR_ARG, "step must be >= 1");
    if (q.param_bf16 && !aligned(q.param_bf16, 2)) return set_error(FF_ERR_ALIGN, "param_bf16 misaligned");
  }
  return FF_OK;
}

int ff_adam_step(const FFAdamParam* params, int32_t n_params, float beta1, float beta2, float eps, int32_t flags,
                 void* stream) {
  const int rc = validate_adam(params, n_params, beta1, beta2, eps, flags, true);
  if (rc) return rc;
  return cuda_status(launch_adam(params, n_params, beta1, beta2, eps, (flags & FF_ADAM_ZERO_GRAD) != 0,
                                 (cudaStream_t)stream),
                     "ff_adam_step launch");
}

int ff_adam_step_scheduled(const FFAdamParam* params, int32_t n_params, float beta1, float beta2, float eps,
                           int32_t flags, const double* lr, const int64_t* step, void* stream) {
  const int rc = validate_adam(params, n_params, beta1, beta2, eps, flags, false);
  if (rc) return rc;
  if (n_params > 0 && (!lr || !step)) return set_error(FF_ERR_ARG, "lr and step must be device pointers");
  if (!aligned(lr, 8) || !aligned(step, 8)) return set_error(FF_ERR_ALIGN, "lr and step must be 8-byte aligned");
  return cuda_status(launch_adam(params, n_params, beta1, beta2, eps, (flags & FF_ADAM_ZERO_GRAD) != 0,
                                 (cudaStream_t)stream, lr, step),
                     "ff_adam_step_scheduled launch");
}

int64_t ff_image_metrics_workspace_bytes(int32_t height, int32_t width, int32_t channels) {
  if (height < 11 || width < 11 || channels < 1 || (int64_t)height * width * channels >= (1ll << 31)) return FF_ERR_ARG;
  return image_metrics_workspace_bytes(height, width, channels);
}

int ff_image_metrics(const float* img0, const float* img1, int32_t height, int32_t width, int32_t channels,
                     float max_val, double* mse_ssim, void* workspace, int64_t workspace_bytes, void* stream) {
  const int64_t need = ff_image_metrics_workspace_bytes(height, width, channels);
  if (need < 0) return set_error(FF_ERR_ARG, "images need height, width >= 11 and channels >= 1");
  if (!img0 || !img1 || !mse_ssim || !workspace) return set_error(FF_ERR_ARG, "NULL argument");
  if (workspace_bytes < need) return set_error(FF_ERR_SIZE, "workspace smaller than ff_image_metrics_workspace_bytes");
  if (!aligned(workspace, 8)) return set_error(FF_ERR_ALIGN, "workspace must be 8-byte aligned");
  return cuda_status(launch_image_metrics(img0, img1, height, width, channels, max_val, workspace, mse_ssim,
                                          (cudaStream_t)stream),
                     "ff_image_metrics");
}

int64_t ff_occupancy_workspace_bytes(int32_t depth, int32_t height, int32_t width) {
  const int64_t v = (int64_t)depth * height * width;
  if (depth < 1 || height < 1 || width < 1 || v >= (1ll << 31)) return FF_ERR_ARG;
  return occupancy_workspace_bytes(v);
}

int ff_occupancy_mask(const float* alpha, int32_t depth, int32_t height, int32_t width, float threshold,
                      int32_t min_size, int32_t* bits, float* volume, int32_t* bbox, void* workspace,
                      int64_t workspace_bytes, void* stream) {
  const int64_t need = ff_occupancy_workspace_bytes(depth, height, width);
  if (need < 0) return set_error(FF_ERR_ARG, "bad occupancy volume dimensions");
  if (!alpha || !bits || !bbox || !workspace) return set_error(FF_ERR_ARG, "alpha/bits/bbox/workspace are NULL");
  if (workspace_bytes < need) return set_error(FF_ERR_SIZE, "workspace smaller than ff_occupancy_workspace_bytes");
  if (!aligned(workspace, 256)) return set_error(FF_ERR_ALIGN, "workspace must be 256-byte aligned");
  int status = 0;
  int rc = cuda_status(launch_occupancy_mask(alpha, depth, height, width, threshold, min_size, bits, volume, bbox,
                                             workspace, &status, (cudaStream_t)stream),
                       "ff_occupancy_mask");
  if (rc) return rc;
  if (status) return set_error(FF_ERR_LIMIT, "ff_occupancy_mask: a union-find loop hit its iteration limit");
  return FF_OK;
}

int ff_march_count(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays, int32_t* counts,
                   float* t_min, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && !counts) return set_error(FF_ERR_ARG, "counts is NULL");
  return cuda_status(launch_march_count(*r, rays, jitter, n_rays, counts, t_min, (cudaStream_t)stream),
                     "ff_march_count launch");
}

int64_t ff_scan_workspace_bytes(int64_t n) { return n < 0 ? -1 : scan_workspace_bytes(n); }

int ff_scan_counts(const int32_t* counts, int64_t n, int64_t* offsets, void* workspace, int64_t workspace_bytes,
                   void* stream) {
  if (n < 0 || !offsets || (n > 0 && (!counts || !workspace))) return set_error(FF_ERR_ARG, "bad scan arguments");
  if (workspace_bytes < scan_workspace_bytes(n)) return set_error(FF_ERR_SIZE, "scan workspace too small");
  if (!aligned(workspace, 8) || !aligned(offsets, 8)) return set_error(FF_ERR_ALIGN, "scan buffers must be 8-byte aligned");
  return cuda_status(launch_scan(counts, n, offsets, workspace, (cudaStream_t)stream), "ff_scan_counts launch");
}

int64_t ff_scan_noalloc_max_counts(void) { return scan_noalloc_max_counts(); }

int ff_scan_counts_noalloc(const int32_t* counts, int64_t n, int64_t* offsets, void* stream) {
  if (n < 0 || !offsets || (n > 0 && !counts)) return set_error(FF_ERR_ARG, "bad scan arguments");
  if (n > scan_noalloc_max_counts())
    return set_error(FF_ERR_SIZE, "ff_scan_counts_noalloc: " + std::to_string(n) + " counts exceed its fixed scratch (" +
                                      std::to_string(scan_noalloc_max_counts()) +
                                      " counts); use ff_scan_counts with a workspace");
  if (!aligned(offsets, 8)) return set_error(FF_ERR_ALIGN, "offsets must be 8-byte aligned");
  return cuda_status(launch_scan_noalloc(counts, n, offsets, (cudaStream_t)stream), "ff_scan_counts_noalloc");
}

int ff_filter_rays(const FFRender* r, const float* rays, int64_t n_rays, int32_t n_samples, int32_t bbox_only,
                   uint8_t* keep, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && !keep) return set_error(FF_ERR_ARG, "keep is NULL");
  if (!bbox_only && (n_samples < 1 || !r->occ_bits))
    return set_error(FF_ERR_ARG, "ff_filter_rays needs n_samples >= 1 and an occupancy bitfield (or bbox_only)");
  return cuda_status(launch_filter_rays(*r, rays, n_rays, n_samples, bbox_only, keep, (cudaStream_t)stream),
                     "ff_filter_rays launch");
}

int ff_march_emit(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays, const int64_t* offsets,
                  float* xyz, int32_t* sample_idx, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!offsets || !xyz || !sample_idx)) return set_error(FF_ERR_ARG, "emit outputs are NULL");
  return cuda_status(launch_march_emit(*r, rays, jitter, n_rays, offsets, xyz, sample_idx, (cudaStream_t)stream),
                     "ff_march_emit launch");
}

int ff_composite_forward(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                         const int64_t* offsets, const int32_t* sample_idx, const float* feat, int32_t feat_stride,
                         const int32_t* white_bg, float* rgb, float* depth, float* acc, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 28) return set_error(FF_ERR_UNSUPPORTED, "the SH-2 colour head needs feat_stride >= 28");
  if (n_rays > 0 && (!offsets || !rgb)) return set_error(FF_ERR_ARG, "offsets/rgb are NULL");
  return cuda_status(launch_composite_forward(*r, rays, jitter, n_rays, offsets, sample_idx, feat, feat_stride,
                                              white_bg, rgb, depth, acc, nullptr, nullptr, (cudaStream_t)stream),
                     "ff_composite_forward launch");
}

int ff_composite_backward(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                          const int64_t* offsets, const int32_t* sample_idx, const float* feat, int32_t feat_stride,
                          const int32_t* white_bg, const float* grad_rgb, float* grad_feat, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 28) return set_error(FF_ERR_UNSUPPORTED, "the SH-2 colour head needs feat_stride >= 28");
  if (n_rays > 0 && (!offsets || !grad_rgb || !grad_feat)) return set_error(FF_ERR_ARG, "backward buffers are NULL");
  return cuda_status(launch_composite_backward(*r, rays, jitter, n_rays, offsets, sample_idx, feat, feat_stride,
                                               white_bg, grad_rgb, grad_feat, nullptr, (cudaStream_t)stream),
                     "ff_composite_backward launch");
}

int ff_composite_forward_zd(const FFRender* r, const float* rays, int64_t n_rays, const int64_t* offsets,
                            const float* zd, const float* feat, int32_t feat_stride, float* rgb, float* depth,
                            float* w_out, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 28) return set_error(FF_ERR_UNSUPPORTED, "the SH-2 colour head needs feat_stride >= 28");
  if (n_rays > 0 && (!offsets || !rgb || !zd)) return set_error(FF_ERR_ARG, "offsets/zd/rgb are NULL");
  return cuda_status(launch_composite_forward(*r, rays, nullptr, n_rays, offsets, nullptr, feat, feat_stride, nullptr,
                                              rgb, depth, nullptr, zd, w_out, (cudaStream_t)stream),
                     "ff_composite_forward_zd launch");
}

int ff_composite_backward_zd(const FFRender* r, const float* rays, int64_t n_rays, const int64_t* offsets,
                             const float* zd, const float* feat, int32_t feat_stride, const float* grad_rgb,
                             float* grad_feat, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 28) return set_error(FF_ERR_UNSUPPORTED, "the SH-2 colour head needs feat_stride >= 28");
  if (n_rays > 0 && (!offsets || !grad_rgb || !grad_feat || !zd)) return set_error(FF_ERR_ARG, "buffers are NULL");
  return cuda_status(launch_composite_backward(*r, rays, nullptr, n_rays, offsets, nullptr, feat, feat_stride,
                                               nullptr, grad_rgb, grad_feat, zd, (cudaStream_t)stream),
                     "ff_composite_backward_zd launch");
}

int ff_composite_weights(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                         const int64_t* offsets, const int32_t* sample_idx, const float* feat, int32_t feat_stride,
                         float* w_out, int32_t* app_counts, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 1) return set_error(FF_ERR_ARG, "feat_stride must be >= 1");
  if (n_rays > 0 && (!offsets || !sample_idx || !feat || !w_out || !app_counts))
    return set_error(FF_ERR_ARG, "ff_composite_weights: a buffer is NULL");
  return cuda_status(launch_composite_weights(*r, rays, jitter, n_rays, offsets, sample_idx, feat, feat_stride, w_out,
                                              app_counts, (cudaStream_t)stream),
                     "ff_composite_weights launch");
}

int ff_app_emit(int64_t n_rays, const int64_t* offsets, const float* w, float weight_thres, const int64_t* app_offsets,
                int32_t* app_idx, int32_t* app_ray, void* stream) {
  if (n_rays < 0 || (n_rays > 0 && (!offsets || !w || !app_offsets || !app_idx || !app_ray)))
    return set_error(FF_ERR_ARG, "ff_app_emit: bad arguments");
  return cuda_status(launch_app_emit(n_rays, offsets, w, weight_thres, app_offsets, app_idx, app_ray,
                                     (cudaStream_t)stream),
                     "ff_app_emit launch");
}

static int validate_render_head(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                                const int32_t* app_idx, const int32_t* app_ray, int64_t n) {
  if (!h) return set_error(FF_ERR_ARG, "render head descriptor is NULL");
  if (h->n_layers < 1 || h->n_layers > FF_MAX_MLP_LAYERS) return set_error(FF_ERR_ARG, "n_layers must be 1..4");
  if (h->in_channels < 1 || h->hidden_dim < 1 || h->view_pe < 0 || h->fea_pe < 0 || h->view_pe > 24 || h->fea_pe > 24)
    return set_error(FF_ERR_ARG, "bad render head dimensions");
  const int64_t in = 3 + (int64_t)h->in_channels + 6 * (int64_t)h->view_pe + 2 * (int64_t)h->fea_pe * h->in_channels;
  if (h->in_dim != in) return set_error(FF_ERR_ARG, "in_dim must be 3 + C + 6 view_pe + 2 fea_pe C");
  for (int l = 0; l < h->n_layers; ++l) {
    if (!h->weight[l]) return set_error(FF_ERR_ARG, "a render head weight is NULL");
    if (l == h->n_layers - 1 && h->bias[l]) return set_error(FF_ERR_ARG, "the last layer has no bias");
  }
  if (feat_stride < h->in_channels + 1) return set_error(FF_ERR_ARG, "feat_stride must be >= in_channels + 1");
  if (n < 0 || (n > 0 && (!feat || !rays || !app_idx || !app_ray))) return set_error(FF_ERR_ARG, "bad head inputs");
  return FF_OK;
}

int64_t ff_render_head_workspace_bytes(const FFRenderMlp* h, int64_t n_app) {
  if (!h || n_app < 0 || h->n_layers < 1 || h->n_layers > FF_MAX_MLP_LAYERS) return -1;
  return render_head_workspace_bytes(*h, n_app);
}

int ff_render_head_forward(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                           const int32_t* app_idx, const int32_t* app_ray, int64_t n_app, float* rgb_sample,
                           void* workspace, int64_t workspace_bytes, void* stream) {
  int rc = validate_render_head(h, feat, feat_stride, rays, app_idx, app_ray, n_app);
  if (rc) return rc;
  if (n_app > 0 && !rgb_sample) return set_error(FF_ERR_ARG, "rgb_sample is NULL");
  if (workspace_bytes < render_head_workspace_bytes(*h, n_app) || (n_app > 0 && !workspace))
    return set_error(FF_ERR_SIZE, "render head workspace too small");
  if (!aligned(workspace, 256)) return set_error(FF_ERR_ALIGN, "workspace must be 256-byte aligned");
  return cuda_status(launch_render_head_forward(*h, feat, feat_stride, 1, rays, app_idx, app_ray, n_app, rgb_sample,
                                                workspace, (cudaStream_t)stream),
                     "ff_render_head_forward launch");
}

int ff_render_head_backward(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                            const int32_t* app_idx, const int32_t* app_ray, int64_t n_app, const float* grad_rgb_sample,
                            float* grad_feat, const FFMlpGrad* g, void* workspace, int64_t workspace_bytes,
                            void* stream) {
  int rc = validate_render_head(h, feat, feat_stride, rays, app_idx, app_ray, n_app);
  if (rc) return rc;
  if (n_app > 0 && (!grad_rgb_sample || !grad_feat)) return set_error(FF_ERR_ARG, "backward buffers are NULL");
  if (workspace_bytes < render_head_workspace_bytes(*h, n_app) || (n_app > 0 && !workspace))
    return set_error(FF_ERR_SIZE, "render head workspace too small");
  if (!aligned(workspace, 256)) return set_error(FF_ERR_ALIGN, "workspace must be 256-byte aligned");
  FFMlpGrad none = {};
  return cuda_status(launch_render_head_backward(*h, feat, feat_stride, 1, rays, app_idx, app_ray, n_app,
                                                 grad_rgb_sample, grad_feat, g ? *g : none, workspace,
                                                 (cudaStream_t)stream),
                     "ff_render_head_backward launch");
}

int ff_render_head_forward_tc(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                              const int32_t* app_idx, const int32_t* app_ray, int64_t n_app, float* rgb_sample,
                              int32_t* status, void* stream) {
  int rc = validate_render_head(h, feat, feat_stride, rays, app_idx, app_ray, n_app);
  if (rc) return rc;
  if (const char* why = render_head_tc_unsupported(*h)) return set_error(FF_ERR_UNSUPPORTED, why);
  if (n_app > 0 && !rgb_sample) return set_error(FF_ERR_ARG, "rgb_sample is NULL");
  return cuda_status(launch_render_head_tc_forward(*h, feat, feat_stride, rays, app_idx, app_ray, n_app, rgb_sample,
                                                   status, (cudaStream_t)stream),
                     "ff_render_head_forward_tc launch");
}

int ff_render_head_backward_tc(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                               const int32_t* app_idx, const int32_t* app_ray, int64_t n_app,
                               const float* grad_rgb_sample, float* grad_feat, const FFMlpGrad* g, int32_t* status,
                               void* stream) {
  int rc = validate_render_head(h, feat, feat_stride, rays, app_idx, app_ray, n_app);
  if (rc) return rc;
  if (const char* why = render_head_tc_unsupported(*h)) return set_error(FF_ERR_UNSUPPORTED, why);
  if (n_app > 0 && (!grad_rgb_sample || !grad_feat)) return set_error(FF_ERR_ARG, "backward buffers are NULL");
  FFMlpGrad none = {};
  return cuda_status(launch_render_head_tc_backward(*h, feat, feat_stride, rays, app_idx, app_ray, n_app,
                                                    grad_rgb_sample, grad_feat, g ? *g : none, status,
                                                    (cudaStream_t)stream),
                     "ff_render_head_backward_tc launch");
}

int ff_composite_forward_rgb(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                             const int64_t* offsets, const int32_t* sample_idx, const float* feat, int32_t feat_stride,
                             const float* rgb_sample, const int32_t* white_bg, float* rgb, float* depth, float* acc,
                             void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 1) return set_error(FF_ERR_ARG, "feat_stride must be >= 1");
  if (n_rays > 0 && (!offsets || !rgb || !sample_idx)) return set_error(FF_ERR_ARG, "offsets/sample_idx/rgb are NULL");
  return cuda_status(launch_composite_forward_rgb(*r, rays, jitter, n_rays, offsets, sample_idx, feat, feat_stride,
                                                  rgb_sample, white_bg, rgb, depth, acc, (cudaStream_t)stream),
                     "ff_composite_forward_rgb launch");
}

int ff_composite_backward_rgb(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                              const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                              int32_t feat_stride, const float* rgb_sample, const int32_t* white_bg,
                              const float* grad_rgb, float* grad_feat, float* grad_rgb_sample, void* stream) {
  int rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (feat_stride < 1) return set_error(FF_ERR_ARG, "feat_stride must be >= 1");
  if (n_rays > 0 && (!offsets || !sample_idx || !grad_rgb || !grad_feat || !grad_rgb_sample))
    return set_error(FF_ERR_ARG, "backward buffers are NULL");
  return cuda_status(launch_composite_backward_rgb(*r, rays, jitter, n_rays, offsets, sample_idx, feat, feat_stride,
                                                   rgb_sample, white_bg, grad_rgb, grad_feat, grad_rgb_sample,
                                                   (cudaStream_t)stream),
                     "ff_composite_backward_rgb launch");
}

static int validate_proposal(const FFProposal* p, const float* rays, int64_t n) {
  if (!p) return set_error(FF_ERR_ARG, "proposal descriptor is NULL");
  if (n < 0 || (n > 0 && !rays)) return set_error(FF_ERR_ARG, "bad rays pointer or count");
  if (p->reso < 2 || (int64_t)p->reso * p->reso * p->reso > (1ll << 30)) return set_error(FF_ERR_ARG, "bad proposal reso");
  if (p->n_bins < 32 || p->n_bins > 128 || p->n_bins % 32)
    return set_error(FF_ERR_UNSUPPORTED, "n_bins must be 32, 64, 96 or 128");
  if (p->n_fine < 1 || p->n_fine > 128) return set_error(FF_ERR_UNSUPPORTED, "n_fine must be 1..128");
  if (p->param_dtype != FF_F32 && p->param_dtype != FF_BF16) return set_error(FF_ERR_ARG, "bad param_dtype");
  return FF_OK;
}

int ff_proposal_encode(const FFProposal* p, const void* grid, const float* rays, int64_t n_rays, float* feat,
                       void* stream) {
  int rc = validate_proposal(p, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!grid || !feat)) return set_error(FF_ERR_ARG, "grid/feat are NULL");
  if (!aligned(grid, 16) || !aligned(feat, 16)) return set_error(FF_ERR_ALIGN, "grid/feat must be 16-byte aligned");
  return cuda_status(launch_proposal_encode(*p, grid, rays, n_rays, feat, (cudaStream_t)stream),
                     "ff_proposal_encode launch");
}

int ff_proposal_resample(const FFProposal* p, const float* rays, int64_t n_rays, const float* o_prop,
                         const float* jitter, const float* u, float* w_prop, float* xyz, float* zd, int32_t* bin_of,
                         void* stream) {
  int rc = validate_proposal(p, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!xyz || !zd)) return set_error(FF_ERR_ARG, "xyz/zd are NULL");
  return cuda_status(launch_proposal_resample(*p, rays, n_rays, o_prop, jitter, u, w_prop, xyz, zd, bin_of,
                                              (cudaStream_t)stream),
                     "ff_proposal_resample launch");
}

int ff_proposal_resample_occupied(const FFProposal* p, const FFRender* r, const float* rays, int64_t n_rays,
                                  const float* o_prop, const float* jitter, int32_t* counts, int64_t* offsets,
                                  void* workspace, int64_t workspace_bytes, float* xyz, float* zd, void* stream) {
  int rc = validate_proposal(p, rays, n_rays);
  if (rc) return rc;
  rc = validate_render(r, rays, n_rays);
  if (rc) return rc;
  if (!r->occ_bits) return set_error(FF_ERR_ARG, "ff_proposal_resample_occupied needs an occupancy volume (occ_bits)");
  if (!offsets) return set_error(FF_ERR_ARG, "offsets is NULL");
  if (n_rays > 0 && (!counts || !xyz || !zd)) return set_error(FF_ERR_ARG, "buffers are NULL");
  if (workspace_bytes < scan_workspace_bytes(n_rays) || (n_rays > 0 && !workspace))
    return set_error(FF_ERR_ARG, "workspace smaller than ff_scan_workspace_bytes(n_rays)");
  return cuda_status(launch_proposal_resample_occupied(*p, *r, rays, n_rays, o_prop, jitter, counts, offsets, workspace,
                                                       xyz, zd, (cudaStream_t)stream),
                     "ff_proposal_resample_occupied launch");
}

int ff_proposal_loss(const FFProposal* p, const float* rays, int64_t n_rays, const float* o_prop,
                     const float* w_field, const int32_t* bin_of, float loss_scale, float* loss_sum, float* grad_o,
                     void* stream) {
  int rc = validate_proposal(p, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!o_prop || !w_field || !bin_of || !grad_o)) return set_error(FF_ERR_ARG, "buffers are NULL");
  return cuda_status(launch_proposal_loss(*p, rays, n_rays, o_prop, w_field, bin_of, loss_scale, loss_sum, grad_o,
                                          (cudaStream_t)stream),
                     "ff_proposal_loss launch");
}

int ff_proposal_scatter(const FFProposal* p, const float* rays, int64_t n_rays, const float* grad_feat,
                        float* grad_grid, void* stream) {
  int rc = validate_proposal(p, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!grad_feat || !grad_grid)) return set_error(FF_ERR_ARG, "buffers are NULL");
  if (!aligned(grad_grid, 16) || !aligned(grad_feat, 16)) return set_error(FF_ERR_ALIGN, "buffers must be 16-byte aligned");
  return cuda_status(launch_proposal_scatter(*p, rays, n_rays, grad_feat, grad_grid, (cudaStream_t)stream),
                     "ff_proposal_scatter launch");
}

static int validate_head(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays, int64_t n) {
  int rc = validate_proposal(p, rays, n);
  if (rc) return rc;
  if (!m) return set_error(FF_ERR_ARG, "mlp is NULL");
  if (m->n_layers != 2 || m->in_dim != 8 || m->hidden_dim != 64 || m->out_dim != 1)
    return set_error(FF_ERR_UNSUPPORTED, "the proposal head is an 8 -> 64 -> 1 MLP");
  if (m->bias[1]) return set_error(FF_ERR_UNSUPPORTED, "the proposal head's last layer has no bias");
  if (n > 0 && (!grid || !m->weight[0] || !m->weight[1])) return set_error(FF_ERR_ARG, "grid/weights are NULL");
  if (!aligned(grid, 16)) return set_error(FF_ERR_ALIGN, "grid must be 16-byte aligned");
  return FF_OK;
}

int ff_proposal_head_forward(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays,
                             int64_t n_rays, float* o_prop, void* stream) {
  int rc = validate_head(p, grid, m, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && !o_prop) return set_error(FF_ERR_ARG, "o_prop is NULL");
  return cuda_status(launch_proposal_head_forward(*p, grid, *m, rays, n_rays, o_prop, (cudaStream_t)stream),
                     "ff_proposal_head_forward launch");
}

int ff_proposal_head_infer(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays, int64_t n_rays,
                           float* o_prop, void* stream) {
  int rc = validate_head(p, grid, m, rays, n_rays);
  if (rc) return rc;
  if (p->param_dtype != FF_BF16) return set_error(FF_ERR_UNSUPPORTED, "ff_proposal_head_infer reads a BF16 grid");
  if (n_rays > 0 && !o_prop) return set_error(FF_ERR_ARG, "o_prop is NULL");
  return cuda_status(launch_proposal_head_infer(*p, grid, *m, rays, n_rays, o_prop, (cudaStream_t)stream),
                     "ff_proposal_head_infer launch");
}

int ff_proposal_head_backward(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays,
                              int64_t n_rays, const float* grad_o, float* grad_grid, const FFMlpGrad* g,
                              void* stream) {
  int rc = validate_head(p, grid, m, rays, n_rays);
  if (rc) return rc;
  if (n_rays > 0 && (!grad_o || !grad_grid)) return set_error(FF_ERR_ARG, "grad_o/grad_grid are NULL");
  if (!aligned(grad_grid, 16)) return set_error(FF_ERR_ALIGN, "grad_grid must be 16-byte aligned");
  FFMlpGrad none = {};
  return cuda_status(launch_proposal_head_backward(*p, grid, *m, rays, n_rays, grad_o, grad_grid, g ? *g : none,
                                                   (cudaStream_t)stream),
                     "ff_proposal_head_backward launch");
}

}  // extern "C"
