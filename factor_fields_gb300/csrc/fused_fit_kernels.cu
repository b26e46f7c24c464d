// Fused field + MLP head: the fit step (ff_field_fit_step).
#include "fused_impl.cuh"

namespace ffgb {

cudaError_t launch_fused_fit_rows(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                  const float* x, int64_t x_stride, const float* target, int64_t t_stride, int64_t n,
                                  int loss_kind, float loss_scale, float* loss_sum, float* grad_basis,
                                  float* grad_coeff, const FFMlpGrad& g, float loss_mul, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, x, n);
  a.x_stride = x_stride;
  a.target = target;
  a.t_stride = t_stride;
  a.loss_kind = loss_kind;
  a.loss_scale = loss_scale;
  a.loss_sum = loss_sum;
  a.loss_mul = loss_mul;
  a.grad_basis = grad_basis;
  a.grad_coeff = grad_coeff;
  a.grad_w0 = g.weight[0];
  a.grad_b0 = g.bias[0];
  a.grad_w1 = g.weight[1];
  return dispatch<kFit>(a, st);
}

cudaError_t launch_fused_fit(const FFField& f, const void* basis, const void* coeff, const FFMlp& m, const float* x,
                             const float* target, int64_t n, int loss_kind, float loss_scale, float* loss_sum,
                             float* grad_basis, float* grad_coeff, const FFMlpGrad& g, cudaStream_t st) {
  return launch_fused_fit_rows(f, basis, coeff, m, x, f.coord_dim, target, m.out_dim, n, loss_kind, loss_scale,
                               loss_sum, grad_basis, grad_coeff, g, 1.f, st);
}

}  // namespace ffgb
