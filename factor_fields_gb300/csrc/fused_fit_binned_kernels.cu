// Fused field + MLP head: the fit step on a batch binned by coefficient cell
// (ff_field_fit_step_binned = ff_field_fit_bin + ff_field_fit_step_on_bins): binning with the
// gradient zeroing (fit_bin_kernels.cu), then the kFitBinned kernel on the binned rows.
#include "fused_impl.cuh"

namespace ffgb {

cudaError_t launch_fit_bin_phase(const FFField& f, const FFMlp& m, const float* x, const float* target, int64_t n,
                                 float* loss_sum, float* grad_basis, float* grad_coeff, const FFMlpGrad& g,
                                 void* workspace, bool zero_grads, cudaStream_t st) {
  FitZero z = {};
  if (zero_grads) {
    z.grad_basis = grad_basis;
    z.grad_coeff = grad_coeff;
    z.other[0] = g.weight[0];
    z.other_n[0] = (int64_t)m.hidden_dim * m.in_dim;
    z.other[1] = g.bias[0];
    z.other_n[1] = m.hidden_dim;
    z.other[2] = g.weight[1];
    z.other_n[2] = (int64_t)m.out_dim * m.hidden_dim;
    z.other[3] = loss_sum;
    z.other_n[3] = 1;
  }
  if (n == 0 && !zero_grads) return cudaSuccess;  // nothing to bin; with n == 0 the zeroing still happens
  return launch_fit_bin(f, x, target, m.out_dim, n, workspace, zero_grads ? &z : nullptr, st);
}

cudaError_t launch_fit_on_bins(const FFField& f, const void* basis, const void* coeff, const FFMlp& m, int64_t n,
                               int loss_kind, float loss_scale, float* loss_sum, float* grad_basis, float* grad_coeff,
                               const FFMlpGrad& g, const void* workspace, float loss_mul, bool level0_shared,
                               cudaStream_t st, bool after_bin) {
  if (n == 0) return cudaSuccess;
  int64_t stride = 0;
  const float* rows = fit_bin_rows(f, n, m.out_dim, workspace, &stride);
  if (f.param_dtype != FF_BF16)  // float32 grids: the per-point fit on the binned rows
    return launch_fused_fit_rows(f, basis, coeff, m, rows, stride, rows + f.coord_dim, stride, n, loss_kind,
                                 loss_scale, loss_sum, grad_basis, grad_coeff, g, loss_mul, st);
  FusedArgs a = make_args(f, basis, coeff, m, rows, n);
  a.x_stride = stride;  // packed rows: coordinates, then the targets
  a.target = rows + f.coord_dim;
  a.t_stride = stride;
  a.packed_rows = (f.coord_dim == 3 && m.out_dim == 1 && stride == 4) ? 1 : 0;
  a.loss_kind = loss_kind;
  a.loss_scale = loss_scale;
  a.loss_sum = loss_sum;
  a.loss_mul = loss_mul;
  a.grad_basis = grad_basis;
  a.grad_coeff = grad_coeff;
  a.grad_w0 = g.weight[0];
  a.grad_b0 = g.bias[0];
  a.grad_w1 = g.weight[1];
  a.level0_shared = level0_shared ? 1 : 0;
  a.programmatic = after_bin ? 1 : 0;
  return dispatch_bf16<kFitBinned>(a, st);
}

cudaError_t launch_fused_fit_binned(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                    const float* x, const float* target, int64_t n, int loss_kind, float loss_scale,
                                    float* loss_sum, float* grad_basis, float* grad_coeff, const FFMlpGrad& g,
                                    void* workspace, bool zero_grads, float loss_mul, bool level0_shared,
                                    cudaStream_t st) {
  cudaError_t e = launch_fit_bin_phase(f, m, x, target, n, loss_sum, grad_basis, grad_coeff, g, workspace, zero_grads,
                                       st);
  if (e != cudaSuccess) return e;
  return launch_fit_on_bins(f, basis, coeff, m, n, loss_kind, loss_scale, loss_sum, grad_basis, grad_coeff, g,
                            workspace, loss_mul, level0_shared, st, /*after_bin=*/true);
}

}  // namespace ffgb
