// Fused field + MLP head with the compositing in its epilogue (ff_field_render_fixed): the
// rendering of rays that carry exactly n_fine samples each (the proposal sampler's rendering
// samples), without the per-sample feature rows ever reaching memory.
#include "fused_impl.cuh"

namespace ffgb {

cudaError_t launch_fused_render_fixed(const FFField& f, const void* basis, const void* coeff, const FFMlp& m,
                                      const FFRender& r, const float* rays, const float* xyz, const float* zd,
                                      int64_t n_rays, int nf, float* rgb, float* depth, cudaStream_t st) {
  if (n_rays == 0) return cudaSuccess;
  FusedArgs a = make_args(f, basis, coeff, m, xyz, n_rays * nf);
  a.rd = r;
  a.rays = rays;
  a.zd = zd;
  a.nf = nf;
  a.rgb = rgb;
  a.depth = depth;
  const bool bf = f.param_dtype == FF_BF16;
  // the 28-wide head (density + 27 SH coefficients): four 8-wide output tiles
  if (f.basis_dim == 3 && f.coord_dim == 3)
    return bf ? launch_one<kRender, 3, 3, 4, __nv_bfloat16>(a, st) : launch_one<kRender, 3, 3, 4, float>(a, st);
  if (f.basis_dim == 2 && f.coord_dim == 3)
    return bf ? launch_one<kRender, 2, 3, 4, __nv_bfloat16>(a, st) : launch_one<kRender, 2, 3, 4, float>(a, st);
  return cudaErrorInvalidValue;
}

}  // namespace ffgb
