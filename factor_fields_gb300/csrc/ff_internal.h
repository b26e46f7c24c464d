// Host-side launchers shared between the kernel translation units and the C-ABI layer.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "../../include/ff_native.h"

namespace ffgb {

// Records an error message for ff_last_error() and returns the code.
int set_error(int code, const std::string& msg);
int check_launch(const char* what);  // reads cudaGetLastError after a launch
int sm_count();                      // SMs of the current device (cached per device)

// field_kernels.cu
cudaError_t launch_field_forward(const FFField& f, const void* basis, const void* coeff, const float* x,
                                 int64_t n, float* feats, float* coeff_out, float* basis_out,
                                 cudaStream_t s);
cudaError_t launch_field_backward(const FFField& f, const void* basis, const void* coeff, const float* x,
                                  int64_t n, const float* grad_feats, const float* grad_coeff_out,
                                  const float* grad_basis_out, float* grad_basis, float* grad_coeff_grid,
                                  cudaStream_t s);

// mlp_kernels.cu
// Returns the dynamic shared memory an MLP launch needs, or -1 if the shape cannot fit.
int64_t mlp_smem_bytes(const FFMlp& m, bool backward, int* tile_points);
cudaError_t launch_mlp_forward(const FFMlp& m, const float* x, int64_t n, float* out, cudaStream_t s);
cudaError_t launch_mlp_backward(const FFMlp& m, const float* x, int64_t n, const float* grad_out,
                                float* grad_x, const FFMlpGrad& g, cudaStream_t s);

// fused_kernels.cu
const char* fused_unsupported(const FFField& f, const FFMlp& m);  // nullptr when supported
// n_dev (optional): a device count; the launch is sized for n points and processes min(n, *n_dev)
cudaError_t launch_fused_forward(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                 const float* x, int64_t n, float* out, cudaStream_t st,
                                 const int64_t* n_dev = nullptr);
cudaError_t launch_fused_backward(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                  const float* x, int64_t n, const float* grad_out, float* grad_basis,
                                  float* grad_coeff, const FFMlpGrad& g, cudaStream_t st,
                                  const int64_t* n_dev = nullptr);
cudaError_t launch_fused_fit(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                             const float* x, const float* target, int64_t n, int loss_kind, float loss_scale,
                             float* loss_sum, float* grad_basis, float* grad_coeff, const FFMlpGrad& g,
                             cudaStream_t st);

// launch_fused_fit on point rows x_stride / t_stride floats apart (binned, packed batches)
cudaError_t launch_fused_fit_rows(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                  const float* x, int64_t x_stride, const float* target, int64_t t_stride, int64_t n,
                                  int loss_kind, float loss_scale, float* loss_sum, float* grad_basis,
                                  float* grad_coeff, const FFMlpGrad& g, float loss_mul, cudaStream_t st);
cudaError_t launch_fused_fit_binned(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                    const float* x, const float* target, int64_t n, int loss_kind, float loss_scale,
                                    float* loss_sum, float* grad_basis, float* grad_coeff, const FFMlpGrad& g,
                                    void* workspace, bool zero_grads, float loss_mul, bool level0_shared,
                                    cudaStream_t st);
// fused_render_kernels.cu: field forward + compositing of rays with exactly nf samples each
cudaError_t launch_fused_render_fixed(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                      const FFRender& r, const float* rays, const float* xyz, const float* zd,
                                      int64_t n_rays, int nf, float* rgb, float* depth, cudaStream_t st);
// its two halves: binning (with the gradient zeroing) and the fit kernel on the binned rows
cudaError_t launch_fit_bin_phase(const FFField& f, const FFMlp& m, const float* x, const float* target, int64_t n,
                                 float* loss_sum, float* grad_basis, float* grad_coeff, const FFMlpGrad& g,
                                 void* workspace, bool zero_grads, cudaStream_t st);
cudaError_t launch_fit_on_bins(const FFField& f, const void* basis, const void* coeff, const FFMlp& m, int64_t n,
                               int loss_kind, float loss_scale, float* loss_sum, float* grad_basis, float* grad_coeff,
                               const FFMlpGrad& g, const void* workspace, float loss_mul, bool level0_shared,
                               cudaStream_t st, bool after_bin = false);

// fit_bin_kernels.cu
int64_t fit_bin_keys(const FFField& f);
int64_t fit_bin_workspace_bytes(const FFField& f, int64_t n, int out_dim);
// FF_FIT_HOST_BATCH: copies (x, target) from host memory into the workspace on the stream and
// points *x, *target at the copies
cudaError_t fit_bin_stage_host(const FFField& f, const float** x, const float** target, int out_dim, int64_t n,
                               void* workspace, cudaStream_t st);
// Gradient buffers the binning pass zeroes (NULL entries skipped): the grid gradients (16-byte
// aligned, sizes from the descriptor) and up to 4 small float buffers with explicit sizes.
struct FitZero {
  float* grad_basis;
  float* grad_coeff;
  float* other[4];
  int64_t other_n[4];
};
int64_t field_basis_elems(const FFField& f);  // elements of the flat basis buffer
// Bins the batch (3 kernels: bin, alloc, permute) into the workspace's rows: per binned point
// its coordinates then its targets; fit_bin_rows locates them, *stride_out floats per row
// (coord_dim + out_dim rounded up to 4).
cudaError_t launch_fit_bin(const FFField& f, const float* x, const float* target, int out_dim, int64_t n,
                           void* workspace, const FitZero* zero, cudaStream_t st);
const float* fit_bin_rows(const FFField& f, int64_t n, int out_dim, const void* workspace, int64_t* stride_out);

// util_kernels.cu
constexpr int kMaxZeroBuffers = 8;  // buffers per zeroing launch (more: several launches)
cudaError_t launch_zero_buffers(float* const* ptrs, const int64_t* counts, int n_buffers, cudaStream_t st);

// optim_kernels.cu
cudaError_t launch_adam(const FFAdamParam* prm, int n, float beta1, float beta2, float eps, bool zero_grad,
                        cudaStream_t st, const double* lr_dev = nullptr, const int64_t* step_dev = nullptr);

// metrics_kernels.cu
int64_t image_metrics_workspace_bytes(int h, int w, int c);
cudaError_t launch_image_metrics(const float* a, const float* b, int h, int w, int c, float max_val,
                                 void* workspace, double* out_host, cudaStream_t st);

// occupancy_kernels.cu
int64_t occupancy_workspace_bytes(int64_t voxels);
cudaError_t launch_occupancy_mask(const float* alpha, int d, int h, int w, float threshold, int min_size,
                                  int32_t* bits, float* vol, int32_t* bbox, void* workspace, int* status_host,
                                  cudaStream_t st);

// render_kernels.cu
int64_t scan_workspace_bytes(int64_t n);
cudaError_t launch_march_count(const FFRender& r, const float* rays, const float* jitter, int64_t n, int32_t* counts,
                               float* t_min, cudaStream_t s);
cudaError_t launch_scan(const int32_t* counts, int64_t n, int64_t* offsets, void* workspace, cudaStream_t s);
int64_t scan_noalloc_max_counts();
cudaError_t launch_scan_noalloc(const int32_t* counts, int64_t n, int64_t* offsets, cudaStream_t s);
cudaError_t launch_filter_rays(const FFRender& r, const float* rays, int64_t n, int n_samples, int bbox_only,
                               uint8_t* keep, cudaStream_t s);
cudaError_t launch_march_emit(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                              const int64_t* offsets, float* xyz, int32_t* sample_idx, cudaStream_t s);
cudaError_t launch_composite_forward(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                     const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                     int feat_stride, const int32_t* white_bg, float* rgb, float* depth, float* acc,
                                     const float* zd, float* w_out, cudaStream_t s);
cudaError_t launch_composite_backward(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                      const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                      int feat_stride, const int32_t* white_bg, const float* grad_rgb,
                                      float* grad_feat, const float* zd, cudaStream_t s);

cudaError_t launch_composite_forward_rgb(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                         const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                         int feat_stride, const float* rgb_sample, const int32_t* white_bg, float* rgb,
                                         float* depth, float* acc, cudaStream_t s);
cudaError_t launch_composite_backward_rgb(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                          const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                          int feat_stride, const float* rgb_sample, const int32_t* white_bg,
                                          const float* grad_rgb, float* grad_feat, float* grad_rgb_sample,
                                          cudaStream_t s);
cudaError_t launch_composite_weights(const FFRender& r, const float* rays, const float* jitter, int64_t n,
                                     const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                     int feat_stride, float* w_out, int32_t* app_counts, cudaStream_t s);
cudaError_t launch_app_emit(int64_t n, const int64_t* offsets, const float* w, float thres, const int64_t* app_offsets,
                            int32_t* app_idx, int32_t* app_ray, cudaStream_t s);

// render_head_kernels.cu (MLPRender_Fea, float32 drop-in); features are channels 1..C of feat rows
int64_t render_head_workspace_bytes(const FFRenderMlp& h, int64_t n);
cudaError_t launch_render_head_forward(const FFRenderMlp& h, const float* feat, int feat_stride, int feat_off,
                                       const float* rays, const int32_t* app_idx, const int32_t* app_ray, int64_t n,
                                       float* rgb_rows, void* workspace, cudaStream_t s);
cudaError_t launch_render_head_backward(const FFRenderMlp& h, const float* feat, int feat_stride, int feat_off,
                                        const float* rays, const int32_t* app_idx, const int32_t* app_ray, int64_t n,
                                        const float* grad_rgb_rows, float* grad_feat, const FFMlpGrad& gr,
                                        void* workspace, cudaStream_t s);

// render_head_tc.cu (MLPRender_Fea on tcgen05 tensor cores)
const char* render_head_tc_unsupported(const FFRenderMlp& h);  // nullptr when supported
cudaError_t launch_render_head_tc_forward(const FFRenderMlp& h, const float* feat, int feat_stride, const float* rays,
                                          const int32_t* app_idx, const int32_t* app_ray, int64_t n, float* rgb_rows,
                                          int32_t* status, cudaStream_t s);
cudaError_t launch_render_head_tc_backward(const FFRenderMlp& h, const float* feat, int feat_stride, const float* rays,
                                           const int32_t* app_idx, const int32_t* app_ray, int64_t n,
                                           const float* grad_rgb_rows, float* grad_feat, const FFMlpGrad& g,
                                           int32_t* status, cudaStream_t s);

// proposal_kernels.cu
cudaError_t launch_proposal_head_forward(const FFProposal& p, const void* grid, const FFMlp& m, const float* rays,
                                         int64_t n, float* o_out, cudaStream_t s);
cudaError_t launch_proposal_head_infer(const FFProposal& p, const void* grid, const FFMlp& m, const float* rays,
                                       int64_t n, float* o_out, cudaStream_t s);
cudaError_t launch_proposal_head_backward(const FFProposal& p, const void* grid, const FFMlp& m, const float* rays,
                                          int64_t n, const float* g_o, float* grad_grid, const FFMlpGrad& gr,
                                          cudaStream_t s);
cudaError_t launch_proposal_encode(const FFProposal& p, const void* grid, const float* rays, int64_t n, float* feat,
                                   cudaStream_t s);
cudaError_t launch_proposal_scatter(const FFProposal& p, const float* rays, int64_t n, const float* grad_feat,
                                    float* grad_grid, cudaStream_t s);
cudaError_t launch_proposal_resample(const FFProposal& p, const float* rays, int64_t n, const float* o_prop,
                                     const float* jitter, const float* u, float* w_prop, float* xyz, float* zd,
                                     int32_t* bin_of, cudaStream_t s);
cudaError_t launch_proposal_resample_occupied(const FFProposal& p, const FFRender& r, const float* rays, int64_t n,
                                              const float* o_prop, const float* jitter, int32_t* counts,
                                              int64_t* offsets, void* workspace, float* xyz, float* zd,
                                              cudaStream_t s);
cudaError_t launch_proposal_loss(const FFProposal& p, const float* rays, int64_t n, const float* o_prop,
                                 const float* w_field, const int32_t* bin_of, float loss_scale, float* loss_sum,
                                 float* grad_o, cudaStream_t s);

}  // namespace ffgb
