// Fused field + MLP head: support check and the forward (ff_field_mlp_forward).
#include "fused_impl.cuh"

namespace ffgb {

const char* fused_unsupported(const FFField& f, const FFMlp& m) {
  if (f.n_levels != 6) return "the fused path needs 6 basis levels with basis_dims [4,4,4,2,2,2]";
  for (int l = 0; l < 6; ++l)
    if (f.level_channels[l] != kLevelC[l] || f.level_vec[l] != kLevelC[l] || f.level_stride[l] != kLevelC[l])
      return "the fused path needs basis_dims [4,4,4,2,2,2] stored unpadded";
  if (f.n_feat != kF || f.coeff_stride % 8) return "the fused path needs 18 features and coeff_stride % 8 == 0";
  if (m.n_layers != 2 || m.hidden_dim != kHid || m.in_dim != kF)
    return "the fused path needs an MLPMixer with num_layers=2, hidden_dim=64, in_dim=18";
  if (m.out_dim < 1 || m.out_dim > 32) return "the fused path needs 1 <= out_dim <= 32";
  if (!m.bias[0] || m.bias[1]) return "the fused path needs a bias on layer 0 and none on layer 1 (MLPMixer)";
  return nullptr;
}

cudaError_t launch_fused_forward(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                 const float* x, int64_t n, float* out, cudaStream_t st, const int64_t* n_dev) {
  if (n == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, x, n);
  a.out = out;
  a.n_dev = n_dev;
  return dispatch<kFwd>(a, st);
}

}  // namespace ffgb
