// Fused field + MLP head: the backward (ff_field_mlp_backward).
#include "fused_impl.cuh"

namespace ffgb {

cudaError_t launch_fused_backward(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                  const float* x, int64_t n, const float* grad_out, float* grad_basis,
                                  float* grad_coeff, const FFMlpGrad& g, cudaStream_t st, const int64_t* n_dev) {
  if (n == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, x, n);
  a.n_dev = n_dev;
  a.grad_out = grad_out;
  a.grad_basis = grad_basis;
  a.grad_coeff = grad_coeff;
  a.grad_w0 = g.weight[0];
  a.grad_b0 = g.bias[0];
  a.grad_w1 = g.weight[1];
  return dispatch<kBwd>(a, st);
}

}  // namespace ffgb
