/*
 * ff_native.h — C ABI of the GB300 (sm_103a) Factor Fields field-evaluation and ray-rendering
 * library (libffgb.so).
 *
 * Conventions for every entry point:
 *   - Pointers named x, out, grad_* ... are DEVICE pointers owned by the caller. The library
 *     allocates no device memory; where an operation needs scratch space the caller passes it
 *     (see each function) and ff_*_workspace_bytes() says how much.
 *   - Work is enqueued on `stream` (a cudaStream_t passed as void*; NULL = legacy default
 *     stream) and returns without synchronising.
 *   - The return value is FF_OK (0) or a negative FF_ERR_* code; ff_last_error() returns a
 *     thread-local description of the most recent failure on the calling thread.
 *   - Gradient outputs are ACCUMULATED (+=) in float32, like autograd's .grad: zero them first.
 *   - Launches are stream-ordered: two calls on different streams are independent unless they
 *     write the same output buffers (ff_scan_counts_noalloc excepted: its calls share one
 *     library-owned array). The library's only process-wide state is a per-device cache of
 *     launch parameters (SM count, occupancy, kernel attributes) and, for
 *     ff_scan_counts_noalloc, the device address of its array; the caches are filled on first
 *     use with atomic or mutex-guarded writes, so concurrent host threads are safe. They are
 *     keyed by device ordinal and assume the device's primary context (the one the CUDA runtime
 *     and torch use); they are not cleared by cudaDeviceReset.
 *   - Two entry points synchronise the stream before returning because they read a small
 *     result back to the host: ff_occupancy_mask (a status word) and ff_image_metrics (the two
 *     metrics). Every other entry point only enqueues work.
 *
 * Every entry point replaces a specific piece of the reference's PyTorch code
 * (autonomousvision/factor-fields); the citation is given beside each declaration.
 */
#ifndef FF_NATIVE_H
#define FF_NATIVE_H

#include <stdint.h>

#if defined(__GNUC__)
#define FF_API __attribute__((visibility("default")))
#else
#define FF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define FF_ABI_VERSION 1
#define FF_MAX_LEVELS 8
#define FF_MAX_MLP_LAYERS 4

enum {
  FF_OK = 0,
  FF_ERR_ARG = -1,         /* bad pointer / size / enum value */
  FF_ERR_UNSUPPORTED = -2, /* a shape or mode this library does not implement */
  FF_ERR_ALIGN = -3,       /* a pointer is not aligned as documented */
  FF_ERR_CUDA = -4,        /* a CUDA runtime call failed (see ff_last_error) */
  FF_ERR_SIZE = -5,        /* a size exceeds a documented maximum */
  FF_ERR_LIMIT = -6        /* a bounded device loop ran out of iterations (result not valid) */
};

enum { FF_MAP_SAWTOOTH = 0, FF_MAP_TRIANGLE = 1 };
enum { FF_INTERP_LINEAR = 0, FF_INTERP_NEAREST = 1 };
enum { FF_F32 = 0, FF_BF16 = 1 };
enum { FF_LOSS_L1 = 0, FF_LOSS_MSE = 1 };
/* ff_field_fit_step_binned flags */
enum { FF_FIT_ZERO_GRADS = 1, FF_FIT_MEAN_LOSS = 2, FF_FIT_LEVEL0_SHARED = 4, FF_FIT_HOST_BATCH = 8 };

/*
 * Description of one grid/grid factor field (models/FactorFields.py:262-309 setup_params,
 * :397-409 init_basis, :311-317 init_coef). Filled in by the host from the model config.
 *
 * Storage (channels-last, all offsets/strides in ELEMENTS of param_dtype):
 *   basis level l : [R_l]^basis_dim cells x level_stride[l] channels, starting at
 *                   level_offset[l]; cell (x, y[, z]) is at ((z*R + y)*R + x).
 *   coefficients  : [coeff_reso.z][coeff_reso.y][coeff_reso.x] cells x coeff_stride channels.
 *   The float32 gradient buffers use exactly the same element offsets and strides.
 * Alignment: basis/coeff base pointers 16-byte aligned; level_offset[l]*elem_size and
 * level_stride[l]*elem_size multiples of the vector width used for level l (vec_l below).
 */
typedef struct FFField {
  int32_t basis_dim;     /* 2 or 3: dims of the basis grids (in_dim of the reference) */
  int32_t coord_dim;     /* 2 or 3: dims of the input points and of the coefficient grid */
  int32_t n_levels;      /* 1..FF_MAX_LEVELS */
  int32_t mapping;       /* FF_MAP_*: basis_mapping (:11-33) */
  int32_t basis_interp;  /* FF_INTERP_*: cfg.model.basis_mode */
  int32_t coeff_interp;  /* FF_INTERP_*: cfg.model.coef_mode */
  int32_t param_dtype;   /* FF_F32 or FF_BF16: element type of basis and coeff */
  int32_t n_feat;        /* sum(basis_dims) == coefficient channels */
  int32_t level_channels[FF_MAX_LEVELS];
  int32_t level_stride[FF_MAX_LEVELS];
  int32_t level_vec[FF_MAX_LEVELS];  /* 1, 2 or 4: channels per vector access on level l, valid
                                        for the basis level AND its coefficient channel segment */
  int32_t level_reso[FF_MAX_LEVELS];
  int64_t level_offset[FF_MAX_LEVELS];
  float level_scale[FF_MAX_LEVELS];  /* max(aabb size) / freq_bands[l] in float32 (:12-13) */
  float map_origin[3];               /* aabb[0] over the basis dims (:15, :20) */
  int32_t coeff_reso[3];             /* x (W), y (H), z (D) */
  int32_t coeff_stride;              /* channels per coefficient cell (>= n_feat) */
  float coeff_origin[3];             /* aabb[0] over coord dims (:635-637) */
  float coeff_inv_size[3];           /* 2 / (aabb[1] - aabb[0]) in float32 (:636) */
  /* Reciprocals used by the fused kernels' division-free mapping (the drop-in kernels divide
   * exactly as the reference does): float32 nearest to 1/scale and 2/scale. */
  float level_inv_scale[FF_MAX_LEVELS];
  float level_inv_half[FF_MAX_LEVELS];
} FFField;

/* MLPMixer (models/FactorFields.py:113-159): Linear+ReLU per layer, no ReLU after the last.
 * weight[i] is row-major [out_i, in_i] float32 (torch layout); bias[i] may be NULL. */
typedef struct FFMlp {
  int32_t n_layers; /* 1..FF_MAX_MLP_LAYERS */
  int32_t in_dim;
  int32_t hidden_dim;
  int32_t out_dim;
  const float* weight[FF_MAX_MLP_LAYERS];
  const float* bias[FF_MAX_MLP_LAYERS];
} FFMlp;

/* Accumulated (+=) float32 gradients of an FFMlp; NULL entries are skipped. */
typedef struct FFMlpGrad {
  float* weight[FF_MAX_MLP_LAYERS];
  float* bias[FF_MAX_MLP_LAYERS];
} FFMlpGrad;

/* ---- library ------------------------------------------------------------------------- */
FF_API int ff_abi_version(void);
FF_API const char* ff_last_error(void);
/* sizeof of the ABI structs, for binding checks: 0 FFField, 1 FFMlp, 2 FFMlpGrad, 3 FFRender,
 * 4 FFProposal, 5 FFAdamParam, 6 FFRenderMlp. */
FF_API int64_t ff_struct_size(int32_t which);
/* Number of SMs of the current device and the compute capability (major*10+minor). */
FF_API int ff_device_info(int32_t* sm_count, int32_t* cc);

/* ---- field: drop-in (unfused, float32 math) ------------------------------------------ */

/* get_coding (models/FactorFields.py:523-527) = get_coeff (:425-434) * get_basis (:467-513)
 * for basis_type=coeff_type='grid'. x: [n, coord_dim] float32. Outputs (each optional, NULL
 * to skip): feats = basis*coeff [n, n_feat], coeff [n, n_feat], basis [n, n_feat], float32. */
FF_API int ff_field_forward(const FFField* f, const void* basis, const void* coeff, const float* x,
                     int64_t n, float* feats, float* coeff_out, float* basis_out, void* stream);

/* Backward of ff_field_forward: the grid_sample backward scatter of F.grid_sample (:433, :488)
 * and of the product (:527). Incoming gradients of the three outputs, each [n, n_feat] and
 * each optional (NULL = zero): grad_feats, grad_coeff_out, grad_basis_out. grad_basis /
 * grad_coeff_grid: float32 buffers laid out like the parameters (NULL = not wanted). */
FF_API int ff_field_backward(const FFField* f, const void* basis, const void* coeff, const float* x,
                             int64_t n, const float* grad_feats, const float* grad_coeff_out,
                             const float* grad_basis_out, float* grad_basis, float* grad_coeff_grid,
                             void* stream);

/* ---- MLP: drop-in float32 -------------------------------------------------------------- */

/* MLPMixer.forward (models/FactorFields.py:144-159), dropout off. x [n, in_dim] -> out [n, out_dim]. */
FF_API int ff_mlp_forward(const FFMlp* m, const float* x, int64_t n, float* out, void* stream);

/* Backward of ff_mlp_forward: grad_x [n, in_dim] (optional, overwritten) and accumulated
 * weight/bias gradients. */
FF_API int ff_mlp_backward(const FFMlp* m, const float* x, int64_t n, const float* grad_out, float* grad_x,
                    const FFMlpGrad* g, void* stream);

/* ---- field + MLP fused (the fast path; BF16 or float32 grids, BF16 tensor-core MLP) ---- */
/* Requirements (else FF_ERR_UNSUPPORTED): basis_dims = [4,4,4,2,2,2] stored unpadded, and an
 * MLPMixer with num_layers = 2, hidden_dim = 64, in_dim = 18, out_dim <= 32, bias on layer 0
 * only. MLP weights are read as float32 and rounded to BF16 inside the kernel. */

/* linear_mat(get_coding(x)[0]) (models/FactorFields.py:523-527 then :144-159) in one launch:
 * out [n, out_dim] float32. */
FF_API int ff_field_mlp_forward(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                const float* x, int64_t n, float* out, void* stream);

/* Backward of ff_field_mlp_forward given grad_out [n, out_dim]: accumulates the grid
 * gradients (as ff_field_backward) and the MLP weight/bias gradients. Recomputes the forward. */
FF_API int ff_field_mlp_backward(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                 const float* x, int64_t n, const float* grad_out, float* grad_basis,
                                 float* grad_coeff_grid, const FFMlpGrad* g, void* stream);

/* ff_field_mlp_forward / _backward for a point count known only on the device: the launch is
 * sized for n_max points and processes the first min(n_max, *n_dev) of them (n_dev: device
 * int64, e.g. the last entry of ff_scan_counts' offsets: the number of live ray samples), so a
 * render step needs no host read of the live-sample count. Rows past the count are not touched. */
FF_API int ff_field_mlp_forward_counted(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                        const float* x, int64_t n_max, const int64_t* n_dev, float* out,
                                        void* stream);
FF_API int ff_field_mlp_backward_counted(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                         const float* x, int64_t n_max, const int64_t* n_dev,
                                         const float* grad_out, float* grad_basis, float* grad_coeff_grid,
                                         const FFMlpGrad* g, void* stream);

/* One regression step of the notebooks' field fit (scripts/2D_regression.ipynb cell 4,
 * scripts/sdf_regression.ipynb cell 2) up to the optimizer: forward, loss against target
 * [n, out_dim] (FF_LOSS_L1: mean |o - t|, FF_LOSS_MSE: mean (o - t)^2; gradients scaled by
 * loss_scale, normally 1 / (n * out_dim)), and the full backward, in ONE launch.
 * loss_sum (optional, device float) accumulates sum |o - t| or sum (o - t)^2. */
FF_API int ff_field_fit_step(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                             const float* x, const float* target, int64_t n, int32_t loss_kind,
                             float loss_scale, float* loss_sum, float* grad_basis, float* grad_coeff_grid,
                             const FFMlpGrad* g, void* stream);

/* ff_field_fit_step on the batch binned by coefficient cell first (inside the call: bin with
 * atomic ranks, a contiguous row range per cell, permute), so that points sharing coefficient
 * corners sit in the same warp and their coefficient gradients are summed on chip before the
 * atomics. Same loss and gradients as ff_field_fit_step up to float32 summation order.
 * flags: FF_FIT_ZERO_GRADS zeroes grad_basis (the whole flat basis), grad_coeff_grid (this
 * coefficient grid), the MLP gradients in g and *loss_sum first, in the binning pass (the step's
 * zero_grad without a launch of its own); otherwise they are accumulated into (+=).
 * FF_FIT_MEAN_LOSS: *loss_sum accumulates loss_scale * sum of the per-element losses (with
 * loss_scale = 1 / (n * out_dim) the mean loss itself) instead of the plain sum.
 * FF_FIT_LEVEL0_SHARED (BF16 grids, 2-D basis whose level 0 has 4 channels and at most 32^2
 * cells; without effect otherwise): each block of the fit kernel accumulates its level-0 basis
 * gradients in shared memory and adds them to grad_basis once, one float4 atomic per touched
 * cell, instead of one global atomic per point and corner. Same gradients up to float32
 * summation order.
 * FF_FIT_HOST_BATCH: x and target are host memory (page-locked, e.g. cudaHostAlloc or a pinned
 * torch tensor, for an asynchronous copy; pageable memory works but its copy is synchronous
 * and cannot be captured in a CUDA graph). The call copies them into the workspace
 * (cudaMemcpyAsync on the stream, in stream order before the binning) and bins from there, so a
 * captured step holds its own host-to-device copies. The host memory is read when the copies
 * run, not during the call.
 * workspace: device memory of at least ff_field_fit_binned_workspace_bytes(f, n, out_dim)
 * bytes, 256-byte aligned, not shared with a call in flight. */
FF_API int64_t ff_field_fit_binned_workspace_bytes(const FFField* f, int64_t n, int32_t out_dim);
FF_API int ff_field_fit_step_binned(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                    const float* x, const float* target, int64_t n, int32_t loss_kind,
                                    float loss_scale, float* loss_sum, float* grad_basis, float* grad_coeff_grid,
                                    const FFMlpGrad* g, int32_t flags, void* workspace, int64_t workspace_bytes,
                                    void* stream);

/* The two halves of ff_field_fit_step_binned, one call each (the same launches in the same
 * order), for callers that time the fit kernel apart from the binning or bin a batch once for
 * several steps. ff_field_fit_bin: bins (x, target) into the workspace; flags: FF_FIT_ZERO_GRADS,
 * FF_FIT_HOST_BATCH (grad_basis, grad_coeff_grid, g and loss_sum are touched only by that zeroing; the grids' values
 * are not read, so f alone describes them). ff_field_fit_step_on_bins: the fit on the rows that the
 * last ff_field_fit_bin call on this workspace wrote for the same f, n and m->out_dim, in stream
 * order; flags: FF_FIT_MEAN_LOSS, FF_FIT_LEVEL0_SHARED. */
FF_API int ff_field_fit_bin(const FFField* f, const FFMlp* m, const float* x, const float* target, int64_t n,
                            float* loss_sum, float* grad_basis, float* grad_coeff_grid, const FFMlpGrad* g,
                            int32_t flags, void* workspace, int64_t workspace_bytes, void* stream);
FF_API int ff_field_fit_step_on_bins(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                     int64_t n, int32_t loss_kind, float loss_scale, float* loss_sum,
                                     float* grad_basis, float* grad_coeff_grid, const FFMlpGrad* g, int32_t flags,
                                     const void* workspace, int64_t workspace_bytes, void* stream);

/* Zero n_buffers float32 device buffers (ptrs[b], counts[b] elements; the two arrays are host
 * memory, read during the call) in one launch per 8 buffers: a training step's gradient
 * zeroing (optimizer.zero_grad) and loss accumulator reset without one fill per tensor. */
FF_API int ff_zero_f32(float* const* ptrs, const int64_t* counts, int32_t n_buffers, void* stream);

/* ---- optimizer --------------------------------------------------------------------------- */
/* One parameter of ff_adam_step: float32 param, grad, Adam moments (exp_avg, exp_avg_sq, zeroed
 * before the first step), optional BF16 copy of the param to refresh (NULL: none), element
 * count, the step number t >= 1 after this update, and the learning rate. */
typedef struct FFAdamParam {
  float* param;
  float* grad;
  float* exp_avg;
  float* exp_avg_sq;
  void* param_bf16;
  int64_t n;
  int64_t step;
  float lr;
  float reserved;
} FFAdamParam;
enum { FF_ADAM_ZERO_GRAD = 1 };
/* torch.optim.Adam's update (amsgrad=False, weight_decay=0) of n_params parameters in one
 * launch per 8 parameters (params is host memory, read during the call): moments, param, the
 * BF16 copy, and with FF_ADAM_ZERO_GRAD the gradient set to 0 (the next step's zero_grad). */
FF_API int ff_adam_step(const FFAdamParam* params, int32_t n_params, float beta1, float beta2, float eps,
                        int32_t flags, void* stream);
/* ff_adam_step with the schedule in device memory, for a training step captured in a CUDA graph
 * (a replay reads the current values; the launch arguments hold only pointers): lr[b] (float64)
 * is parameter b's learning rate and *step (int64, >= 1 when the kernels run) the step number t
 * after this update, shared by all n_params parameters; the entries' lr and step fields are not
 * read. The bias corrections 1 - beta^t are formed on the device in float32 (beta^t =
 * exp2(t log2 beta)): the step size is within a few ulp of ff_adam_step's, which forms them in
 * double precision as torch.optim.Adam does. The caller advances *step (and decays lr) on the
 * stream before the call. */
FF_API int ff_adam_step_scheduled(const FFAdamParam* params, int32_t n_params, float beta1, float beta2, float eps,
                                  int32_t flags, const double* lr, const int64_t* step, void* stream);

/* ---- evaluation metrics (renderer.py:30-98, utils.py:110-156) ------------------------------ */
/* Mean squared error and SSIM of two [height][width][channels] float32 device images, SSIM as
 * the reference's rgb_ssim (11-tap Gaussian, sigma 1.5, 'valid' window, k1 0.01, k2 0.03,
 * max_val). mse_ssim: HOST double[2] = {mse, ssim}. Synchronises the stream. */
FF_API int64_t ff_image_metrics_workspace_bytes(int32_t height, int32_t width, int32_t channels);
FF_API int ff_image_metrics(const float* img0, const float* img1, int32_t height, int32_t width, int32_t channels,
                            float max_val, double* mse_ssim, void* workspace, int64_t workspace_bytes, void* stream);

/* ---- occupancy-volume maintenance (updateAlphaMask, models/FactorFields.py:757-793) -------- */
/* From the dense alpha volume [depth][height][width] (z, y, x; float32): clamp to [0, 1], 3x3x3
 * max-pool (stride 1, padding 1), >= threshold, then drop the 6-connected components with fewer
 * than min_size voxels (skimage remove_small_objects, connectivity=1; min_size <= 1 keeps
 * all). Outputs: bits [ceil(V / 32)] int32 (bit k of word w = voxel 32 w + k, the layout
 * FFRender.alpha_bits reads), volume [V] 0/1 float32 (optional), bbox [6] int32 = x, y, z
 * minimum then maximum voxel index of the kept voxels (x_min > x_max when none is kept).
 * Synchronises the stream before returning (it reads a status word back): not for graph
 * capture. FF_ERR_LIMIT if a bounded union-find loop ran out (results invalid). */
FF_API int64_t ff_occupancy_workspace_bytes(int32_t depth, int32_t height, int32_t width);
FF_API int ff_occupancy_mask(const float* alpha, int32_t depth, int32_t height, int32_t width, float threshold,
                             int32_t min_size, int32_t* bits, float* volume, int32_t* bbox, void* workspace,
                             int64_t workspace_bytes, void* stream);

/* ---- rendering (bounded scenes): march, compact, composite ------------------------------ */

/* Renderer constants (models/FactorFields.py:586-602, :693-699, :843-898; configs/nerf.yaml
 * renderer keys). rays are [n_rays, 6] float32 (origin, direction). */
typedef struct FFRender {
  float aabb_min[3];
  float aabb_max[3];
  float step;             /* stepSize, float32 as the reference computes it (:697) */
  int32_t n_samples;      /* samples per ray (N_samples > 0, else nSamples) */
  float distance_scale;   /* renderer.distance_scale (25) */
  float density_shift;    /* renderer.density_shift (-10) */
  int32_t density_act;    /* 0 softplus, 1 relu (renderer.fea2denseAct) */
  float weight_thres;     /* renderer.rayMarch_weight_thres (1e-3) */
  int32_t white_bg;       /* add (1 - acc) to rgb (:890-891) */
  /* occupancy (AlphaGridMask, :91-110): NULL = no mask. Bit (z*H + y)*W + x of the 0/1 volume
   * [D][H][W]; a sample is live when the trilinear interpolation of the bits is > 0.5. */
  const uint32_t* occ_bits;
  int32_t occ_reso[3];    /* x (W), y (H), z (D) */
  float occ_origin[3];    /* mask aabb[0] */
  float occ_inv[3];       /* invgridSize = 1.0 / aabbSize * 2, float32 */
} FFRender;

/* Live samples per ray: in the aabb (sample_point, :586-602) and occupied (:865-867).
 * jitter: [n_rays] per-ray offset u added to the sample index when training (:595), or NULL.
 * counts [n_rays] int32; t_min [n_rays] float32 (optional). */
FF_API int ff_march_count(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                          int32_t* counts, float* t_min, void* stream);

/* Exclusive scan: offsets[i] = sum(counts[:i]), offsets[n] = total. Uses a caller workspace of
 * ff_scan_workspace_bytes(n) bytes (per-block partial sums). */
FF_API int64_t ff_scan_workspace_bytes(int64_t n);
FF_API int ff_scan_counts(const int32_t* counts, int64_t n, int64_t* offsets, void* workspace,
                          int64_t workspace_bytes, void* stream);

/* ff_scan_counts for callers that cannot allocate device memory — a host engine that owns
 * every device buffer and hands this library only inputs and outputs, or code running under an
 * allocator it must not touch. It has no counterpart in the reference. Instead of a workspace
 * it uses a fixed scratch array inside the library (32 KiB per GPU, held until the process
 * exits), so it takes at most ff_scan_noalloc_max_counts() = 16,777,216 counts and returns
 * FF_ERR_SIZE beyond that. The first call on a device looks up the array's device address (in
 * the device's primary context; the address is cached per device ordinal and not refreshed
 * after cudaDeviceReset); make that first call before any stream capture. All calls share the
 * array: calls that overlap on the GPU race. It allocates nothing (no cudaMalloc / cudaFree,
 * no allocating library routine). */
FF_API int64_t ff_scan_noalloc_max_counts(void);
FF_API int ff_scan_counts_noalloc(const int32_t* counts, int64_t n, int64_t* offsets, void* stream);

/* filtering_rays (models/FactorFields.py:825-841): keep[ray] = 1 if some sample
 * z_i = t_min + step * i (i < n_samples, no jitter, inside the box or not) has a trilinear
 * occupancy value > 0 (r->occ_bits required), or with bbox_only if the ray meets r's aabb
 * (slab test t_max > t_min, unclamped); else 0. keep: [n_rays] uint8. */
FF_API int ff_filter_rays(const FFRender* r, const float* rays, int64_t n_rays, int32_t n_samples, int32_t bbox_only,
                          uint8_t* keep, void* stream);
/* Writes the live samples in ray-major order (= xyz_sampled[ray_valid] of :874): xyz [M, 3]
 * float32 and sample_idx [M] int32 (index along the ray), using the scanned offsets. */
FF_API int ff_march_emit(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                         const int64_t* offsets, float* xyz, int32_t* sample_idx, void* stream);

/* raw2alpha + colour + compositing (:82-88, :876-896) with the SH-2 colour head: feat [M,
 * feat_stride] holds the MLP output per live sample (channel 0 density feature, 1..27 the SH
 * coefficients as [3][9]). rgb [n_rays, 3], depth [n_rays], acc [n_rays] (optional).
 * white_bg: optional device int overriding r->white_bg. */
FF_API int ff_composite_forward(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                                const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                int32_t feat_stride, const int32_t* white_bg, float* rgb, float* depth,
                                float* acc, void* stream);

/* Backward of ff_composite_forward for dL/drgb [n_rays, 3]: writes dL/dfeat [M, feat_stride]
 * (channels 0..27; overwritten, not accumulated). Depth carries no gradient (:895). */
FF_API int ff_composite_backward(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                                 const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                 int32_t feat_stride, const int32_t* white_bg, const float* grad_rgb,
                                 float* grad_feat, void* stream);

/* Compositing with explicit per-sample (z, dist) pairs zd [M, 2] instead of the uniform
 * sampler's positions (for resampled rays; dist already excludes distance_scale). w_out
 * (optional) receives each sample's compositing weight. Otherwise as ff_composite_*. */
FF_API int ff_composite_forward_zd(const FFRender* r, const float* rays, int64_t n_rays, const int64_t* offsets,
                                   const float* zd, const float* feat, int32_t feat_stride, float* rgb,
                                   float* depth, float* w_out, void* stream);
FF_API int ff_composite_backward_zd(const FFRender* r, const float* rays, int64_t n_rays, const int64_t* offsets,
                                    const float* zd, const float* feat, int32_t feat_stride,
                                    const float* grad_rgb, float* grad_feat, void* stream);

/* Rendering of rays that carry exactly n_fine samples each (32, 64 or 128; ray k's samples at rows
 * [k n_fine, (k + 1) n_fine) of xyz [n_rays * n_fine, 3] and zd, e.g. ff_proposal_resample's
 * output): ff_field_mlp_forward (the fused path, 3-D points, out_dim 28: density + degree-2 SH
 * colour) and ff_composite_forward_zd with offsets k * n_fine, in one launch. The compositing
 * runs in the field kernel's epilogue, so the [n, 28] feature rows never reach memory.
 * rgb [n_rays, 3], depth [n_rays] (optional). Equals the two calls up to float32 summation order
 * of the per-ray sums (rays longer than 32 samples are summed per 32-sample chunk). Forward only:
 * the training step keeps the two calls, whose backward needs the feature rows. */
FF_API int ff_field_render_fixed(const FFField* f, const void* basis, const void* coeff, const FFMlp* m,
                                 const FFRender* r, const float* rays, const float* xyz, const float* zd,
                                 int64_t n_rays, int32_t n_fine, float* rgb, float* depth, void* stream);

/* ---- MLPRender_Fea colour head (models/FactorFields.py:162-203) ------------------------------
 * rgb = sigmoid(MLP([feat, dir, PE(feat, fea_pe), PE(dir, view_pe)])) for the samples whose
 * compositing weight passes renderer.rayMarch_weight_thres (:879-885), with
 * PE(x, F) = [sin(x_d 2^f)]_{d,f} ++ [cos(x_d 2^f)]_{d,f} (index d * F + f, :74-79), feat = the
 * field MLP's channels 1 .. C of the sample's row (feat[app_mask, 1:]) and dir = its ray's
 * direction (rays[:, 3:6], not normalised). The pipeline of FactorFields.forward with this head:
 *   ff_composite_weights -> ff_scan_counts (app counts) -> ff_app_emit -> ff_render_head_forward
 *   -> ff_composite_forward_rgb; backward: ff_composite_backward_rgb -> ff_render_head_backward
 *   -> the field / MLP backward on grad_feat. */
typedef struct FFRenderMlp {
  int32_t n_layers;     /* renderer.num_layers, 1..FF_MAX_MLP_LAYERS */
  int32_t in_channels;  /* C = feature channels (inChanel = model.out_dim - 1) */
  int32_t hidden_dim;   /* renderer.hidden_dim */
  int32_t view_pe;      /* renderer.view_pe */
  int32_t fea_pe;       /* renderer.fea_pe */
  int32_t in_dim;       /* 3 + C + 2 * view_pe * 3 + 2 * fea_pe * C (checked) */
  const float* weight[FF_MAX_MLP_LAYERS]; /* [out_l, in_l] float32 (torch layout); out = 3 for the last */
  const float* bias[FF_MAX_MLP_LAYERS];   /* [out_l] for the hidden layers; the last layer has none */
} FFRenderMlp;

/* Compositing weights without colours (the forward's transmittance scan, :82-88, :876-878):
 * w_out [M] per live sample and app_counts [n_rays] int32 = samples per ray with weight above
 * r->weight_thres. feat: as ff_composite_forward (channel 0 is the density feature). */
FF_API int ff_composite_weights(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                                const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                int32_t feat_stride, float* w_out, int32_t* app_counts, void* stream);
/* The samples with w > weight_thres in ray-major order (app_mask, :879-885): app_idx [n_app]
 * = live-sample index, app_ray [n_app] = its ray, at app_offsets (ff_scan_counts of app_counts).
 * Live-sample indices must fit in int32 (M < 2^31). */
FF_API int ff_app_emit(int64_t n_rays, const int64_t* offsets, const float* w, float weight_thres,
                       const int64_t* app_offsets, int32_t* app_idx, int32_t* app_ray, void* stream);

/* The float32 drop-in head: rgb_sample rows app_idx[i] (of a [M, 3] buffer) receive the colour
 * of app sample i. workspace: ff_render_head_workspace_bytes(h, n_app) bytes, 256-byte aligned. */
FF_API int64_t ff_render_head_workspace_bytes(const FFRenderMlp* h, int64_t n_app);
FF_API int ff_render_head_forward(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                                  const int32_t* app_idx, const int32_t* app_ray, int64_t n_app, float* rgb_sample,
                                  void* workspace, int64_t workspace_bytes, void* stream);
/* Backward for grad_rgb_sample [M, 3] (rows app_idx): writes dL/dfeat into channels 1 .. C of
 * grad_feat rows app_idx[i] (overwritten) and accumulates the weight / bias gradients g (+=). */
FF_API int ff_render_head_backward(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                                   const int32_t* app_idx, const int32_t* app_ray, int64_t n_app,
                                   const float* grad_rgb_sample, float* grad_feat, const FFMlpGrad* g,
                                   void* workspace, int64_t workspace_bytes, void* stream);

/* The same head on the tensor cores (tcgen05 MMA, FP32 accumulators in tensor memory, every
 * accumulation FP32), weights rounded to BF16 inside the kernel (the stored head). The forward
 * holds the input row (features, direction, their positional encoding) and the first hidden layer
 * as FP16 values (11 significant bits; the BF16 weights are exact in FP16). The backward
 * recomputes the forward with BF16 hi + lo pairs for those two (~16 significant bits, so its ReLU
 * decisions match float32 except within ~1e-5 of a kink) and uses BF16 gradient operands.
 * One persistent launch each way, no workspace. Requirements (else FF_ERR_UNSUPPORTED): n_layers
 * 3, hidden_dim 128, fea_pe 2, view_pe 6, in_channels 27 or 31 (model.out_dim 28 or 32).
 * status (optional, device int32, zero on entry): set to FF_ERR_LIMIT if a bounded wait inside the
 * kernel ran out, and by the forward to FF_ERR_SIZE when a weight, feature or first-layer
 * activation lies outside the FP16 range (|x| > 65504); results invalid in both cases; left
 * untouched otherwise. The backward writes grad_feat and accumulates g exactly like
 * ff_render_head_backward. */
FF_API int ff_render_head_forward_tc(const FFRenderMlp* h, const float* feat, int32_t feat_stride, const float* rays,
                                     const int32_t* app_idx, const int32_t* app_ray, int64_t n_app, float* rgb_sample,
                                     int32_t* status, void* stream);
FF_API int ff_render_head_backward_tc(const FFRenderMlp* h, const float* feat, int32_t feat_stride,
                                      const float* rays, const int32_t* app_idx, const int32_t* app_ray, int64_t n_app,
                                      const float* grad_rgb_sample, float* grad_feat, const FFMlpGrad* g,
                                      int32_t* status, void* stream);

/* ff_composite_forward with per-sample colours from a separate head: rgb_sample [M, 3] is read
 * for the samples whose weight passes the threshold (the others contribute no colour, :880-887). */
FF_API int ff_composite_forward_rgb(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                                    const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                    int32_t feat_stride, const float* rgb_sample, const int32_t* white_bg, float* rgb,
                                    float* depth, float* acc, void* stream);
/* Its backward for dL/drgb [n_rays, 3]: grad_feat rows [M, feat_stride] get dL/dfeat0 in channel 0
 * and zeros elsewhere (overwritten); grad_rgb_sample [M, 3] = dL/dcolour (w * dL/drgb above the
 * threshold, else 0). */
FF_API int ff_composite_backward_rgb(const FFRender* r, const float* rays, const float* jitter, int64_t n_rays,
                                     const int64_t* offsets, const int32_t* sample_idx, const float* feat,
                                     int32_t feat_stride, const float* rgb_sample, const int32_t* white_bg,
                                     const float* grad_rgb, float* grad_feat, float* grad_rgb_sample, void* stream);

/* ---- learned proposal sampler (no counterpart in the reference; resampling follows
 * sample_pdf, dataLoader/ray_utils.py:132-174) ------------------------------------------- */

typedef struct FFProposal {
  float aabb_min[3];
  float aabb_max[3];
  float inv_cell[3];      /* (reso - 1) / (aabb_max - aabb_min): align-corners grid mapping */
  int32_t reso;           /* grid cells per axis; the grid is [reso^3][8] channels-last */
  int32_t param_dtype;    /* FF_F32 or FF_BF16 storage of the grid */
  int32_t n_bins;         /* coarse bins per ray: 32, 64, 96 or 128 */
  int32_t n_fine;         /* resampled samples per ray: 1..128 */
  float density_shift;    /* proposal density = softplus(o + density_shift) */
  float distance_scale;   /* alpha = 1 - exp(-density * bin_len * distance_scale) */
  float uniform_mix;      /* resampling pdf = (1 - mix) * sample_pdf's pdf + mix / n_bins (0 = exact) */
  int32_t u_stratified;   /* given u: u_i lies in stratum [i / n_fine, (i + 1) / n_fine), so each
                             sample's dist is its stratum's width (else: to the next sample) */
} FFProposal;

/* Grid features at the coarse bin centres: feat [n_rays * n_bins, 8] float32. */
FF_API int ff_proposal_encode(const FFProposal* p, const void* grid, const float* rays, int64_t n_rays,
                              float* feat, void* stream);
/* From the proposal MLP's outputs o_prop [n_rays * n_bins]: proposal weights w_prop
 * [n_rays * n_bins], and n_fine samples per ray by inverse CDF: xyz [n_rays * n_fine, 3],
 * zd [n_rays * n_fine, 2] (z, the width of the sample's CDF stratum [F^-1(i / n_fine), F^-1((i+1) / n_fine)]
 * for stratified u; with u given, the distance to the next sample / the segment end), bin_of [.] int32.
 * u: optional [n_rays * n_fine] uniforms; else u_i = (i + jitter[ray]) / n_fine (jitter
 * optional, 0.5 when NULL). o_prop NULL: a flat histogram (stratified samples over the segment).
 * w_prop and bin_of (needed by ff_proposal_loss only) may be NULL: not written. */
FF_API int ff_proposal_resample(const FFProposal* p, const float* rays, int64_t n_rays, const float* o_prop,
                                const float* jitter, const float* u, float* w_prop, float* xyz, float* zd,
                                int32_t* bin_of, void* stream);
/* Rendering with the proposal through an occupancy volume: ff_proposal_resample's rendering
 * samples (u_i = (i + jitter[ray]) / n_fine, jitter optional, 0.5 when NULL; each sample's
 * distance is the width of its CDF stratum) with the samples that fail the alpha-mask test
 * left out (r->occ_bits required; AlphaGridMask.sample_alpha > 0.5, models/FactorFields.py:
 * 865-867, the test ff_march_count applies). Such samples would have zero density, hence alpha 0
 * and weight 0, and would leave the transmittance unchanged, so compositing the kept samples
 * with their own (z, dist) gives the render of all of them with the mask applied. Outputs are
 * compacted per ray in sample order: counts [n_rays] int32, offsets [n_rays + 1] int64 (an
 * exclusive scan of counts; offsets[n_rays] = M stays on the device), xyz [M, 3] and zd [M, 2]
 * in buffers sized for n_rays * n_fine rows; the kept rows equal ff_proposal_resample's rows bit
 * for bit. workspace: ff_scan_workspace_bytes(n_rays) bytes. Of r, the occupancy fields are used
 * (r must pass the same validation as for ff_march_count). */
FF_API int ff_proposal_resample_occupied(const FFProposal* p, const FFRender* r, const float* rays, int64_t n_rays,
                                         const float* o_prop, const float* jitter, int32_t* counts, int64_t* offsets,
                                         void* workspace, int64_t workspace_bytes, float* xyz, float* zd,
                                         void* stream);
/* Proposal loss sum_k max(0, m_k - w_k)^2 / (w_k + 1e-5) per ray, m_k = field weight mass in
 * bin k (w_field [n_rays * n_fine], bin_of from resample), scaled by loss_scale; loss_sum
 * (optional) accumulates the loss, grad_o [n_rays * n_bins] receives dL/do_prop. bin_of must
 * come from ff_proposal_resample with the same descriptor; entries outside [0, n_bins) are
 * ignored (they add no mass). */
FF_API int ff_proposal_loss(const FFProposal* p, const float* rays, int64_t n_rays, const float* o_prop,
                            const float* w_field, const int32_t* bin_of, float loss_scale, float* loss_sum,
                            float* grad_o, void* stream);
/* Scatter dL/dfeat [n_rays * n_bins, 8] into the float32 grid gradient [reso^3][8] (+=). */
FF_API int ff_proposal_scatter(const FFProposal* p, const float* rays, int64_t n_rays, const float* grad_feat,
                               float* grad_grid, void* stream);
/* The proposal head fused on tensor cores: bin-centre positions, the grid gather and the
 * 8 -> 64 (ReLU) -> 1 MLP m (n_layers 2, in_dim 8, hidden_dim 64, out_dim 1, no bias on the
 * last layer) in one launch, o_prop [n_rays * n_bins] out. Equals ff_proposal_encode followed
 * by ff_mlp_forward up to split-BF16 rounding (first layer: features and weights as hi + lo). */
FF_API int ff_proposal_head_forward(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays,
                                    int64_t n_rays, float* o_prop, void* stream);
/* ff_proposal_head_forward for rendering (a BF16 grid): one BF16 tensor-core pass per layer,
 * features and hidden activations rounded to BF16 and the 64 -> 1 layer on the tensor cores too,
 * about 45% fewer instructions. o_prop differs from ff_proposal_head_forward's by BF16
 * rounding (~1e-2 relative). Training keeps ff_proposal_head_forward, whose outputs the loss
 * and the backward are consistent with. */
FF_API int ff_proposal_head_infer(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays,
                                  int64_t n_rays, float* o_prop, void* stream);
/* Backward of ff_proposal_head_forward for grad_o [n_rays * n_bins]: the grid gradient
 * (float32 [reso^3][8], +=) and the MLP gradients g (+=; NULL entries skipped) in one launch.
 * Equals ff_mlp_backward followed by ff_proposal_scatter up to BF16 rounding. */
FF_API int ff_proposal_head_backward(const FFProposal* p, const void* grid, const FFMlp* m, const float* rays,
                                     int64_t n_rays, const float* grad_o, float* grad_grid, const FFMlpGrad* g,
                                     void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FF_NATIVE_H */
