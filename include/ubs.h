/*
 * ubs.h -- C ABI of the GB300 (sm_103a) Universal Beta Splatting rasteriser.
 *
 * Conventions (all entry points):
 *   - Plain device pointers and sizes; no framework types.  `stream` is a
 *     cudaStream_t passed as void* (NULL = legacy default stream).
 *   - The caller owns every buffer.  The library allocates nothing: scratch
 *     memory is a caller-provided workspace whose size comes from the matching
 *     *_workspace_bytes() query.
 *   - float32 tensors are contiguous, row-major; int tensors int32 unless
 *     stated.  Shapes are given in the comment of each function.
 *   - Return 0 (UBS_OK) on success or a negative UBS_ERR_* code; the message
 *     of the calling thread's last failure is returned by ubs_last_error().
 *   - Kernels never trap.  Device-side waits are bounded; a wait that runs out
 *     or an invalid input discovered on the device sets a status word that the
 *     synchronising entry points report as UBS_ERR_DEVICE.
 *
 * Each declaration names the reference operator it replaces
 * (paths inside RongLiu-Leo/universal-beta-splatting).
 */
#ifndef UBS_GB300_H
#define UBS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UBS_OK 0
#define UBS_ERR_INVALID (-1)     /* bad argument (shape, size, pointer)         */
#define UBS_ERR_CUDA (-2)        /* a CUDA runtime call or kernel launch failed */
#define UBS_ERR_UNSUPPORTED (-3) /* valid in the reference, not supported here  */
#define UBS_ERR_OVERFLOW (-4)    /* a caller buffer or workspace is too small   */
#define UBS_ERR_DEVICE (-5)      /* a kernel reported a device-side status      */

/* Message of the calling thread's last failure ("" if none). */
const char *ubs_last_error(void);
/* ABI version of this library (bumped on any signature change). */
int ubs_abi_version(void);
/* Number of kernels this library has launched in the process (no reference
 * counterpart; used to report launches per benchmark step). */
unsigned long long ubs_launch_count(void);
/* Kernel timing (no reference counterpart).  Between ubs_profile_start and
 * ubs_profile_stop every kernel the library launches (from any thread) is
 * bracketed by a pair of CUDA events recorded on its launching stream, from a
 * pool of max_launches pairs created by start (launches beyond the pool are
 * not timed).  stop waits for the recorded events and aggregates the
 * durations per kernel name; ubs_profile_result(i, ...) reads entry i < n.
 * Start and stop are host-side set-up: call them outside stream capture.
 * Launches captured into a CUDA graph while timing is on get their event pair
 * as external event-record nodes, recorded again by every replay: call
 * ubs_profile_sample after each replay (it waits for the events and adds the
 * durations); stop then aggregates the samples instead of taking one. */
int ubs_profile_start(int32_t max_launches);
int ubs_profile_sample(void);
int ubs_profile_stop(int32_t *n_kernels);
int ubs_profile_result(int32_t i, const char **name, int64_t *launches, double *total_ms);
/* FP32 FMA issue-rate probe (no reference counterpart): 8 CTAs of 256 threads
 * per SM run independent FMA chains; *flops receives the launch's FP32 operation
 * count so that the caller's event timing gives the measured FP32 peak used as
 * the blend kernels' roofline denominator.  Workspace: one float per thread. */
size_t ubs_fp32_probe_workspace_bytes(void);
int ubs_fp32_probe(int32_t iters, void *workspace, size_t workspace_bytes, double *flops,
                   void *stream);
/* XU (multi-function unit) issue-rate probe (no reference counterpart): the
 * same launch shape running chains of base-2 exponentials; *ops receives the
 * launch's MUFU operation count, the denominator for the blend kernels'
 * transcendental work (log2 / exp2 / reciprocal).  Workspace as the FP32
 * probe's. */
int ubs_mufu_probe(int32_t iters, void *workspace, size_t workspace_bytes, double *ops,
                   void *stream);

/* ------------------------------------------------------------------ a2 ---
 * R = I + A(a01, a02, a12): submodules/gsplat/cuda/_wrapper.py:34
 * (l_triangle_to_rotmat), kernels l_triagnle_to_rotmat_fwd.cu:8 / _bwd.cu:8.
 * l_triangle [n, row_stride] (first 3 entries of each row used), rotmats [n,3,3].
 * v_l_triangle [n, 3]. */
int ubs_l_triangle_to_rotmat_fwd(int64_t n, const float *l_triangle, int64_t row_stride,
                                 float *rotmats, void *stream);
int ubs_l_triangle_to_rotmat_bwd(int64_t n, const float *v_rotmats, float *v_l_triangle,
                                 void *stream);

/* ------------------------------------------------------------------ a3 ---
 * Sigma = L L^T from rotation, scale and lower-triangle parameters:
 * _wrapper.py:39 (rot_scale_l_triangle_to_covar), kernels
 * rot_scale_l_triangle_to_covar_fwd.cu:8 / _bwd.cu:8.
 * rot [n,3,3], scale [n,dim], l_triangle [n, dim*(dim-1)/2], rest_i/rest_j
 * device int32 [m_rest]; covar [n,dim,dim] or [n,3,3] if spatial_block.
 * 3 <= dim <= 11. */
int ubs_rot_scale_l_triangle_to_covar_fwd(int64_t n, int32_t dim, const float *rot,
                                          const float *scale, const float *l_triangle,
                                          const int32_t *rest_i, const int32_t *rest_j,
                                          int32_t m_rest, int32_t spatial_block, float *covar,
                                          void *stream);
int ubs_rot_scale_l_triangle_to_covar_bwd(int64_t n, int32_t dim, const float *rot,
                                          const float *scale, const float *l_triangle,
                                          const int32_t *rest_i, const int32_t *rest_j,
                                          int32_t m_rest, int32_t spatial_block,
                                          const float *v_covar, float *v_rot, float *v_scale,
                                          float *v_l_triangle, void *stream);

/* ------------------------------------------------------------------ a4 ---
 * Conditioning of an N-D Beta primitive on its view query: _wrapper.py:18
 * (cond_mean_convariance_opacity), kernels cond_mean_convariance_opacity_fwd.cu:107
 * / _bwd.cu:102.  means [n,dim], covars [n,dim,dim], opacities [n], betas and
 * query [n,dim-3]; out_means [n,3], out_covars [n,3,3], out_opacities [n].
 * 4 <= dim <= 11.  exact == 0 reproduces the reference backward bit-for-bit in
 * formula (including its transposed Cholesky-backward factor); exact != 0 gives
 * the true gradient of the forward. */
int ubs_cond_fwd(int64_t n, int32_t dim, const float *means, const float *covars,
                 const float *opacities, const float *betas, const float *query,
                 float *out_means, float *out_covars, float *out_opacities, void *stream);
int ubs_cond_bwd(int64_t n, int32_t dim, const float *means, const float *covars,
                 const float *opacities, const float *betas, const float *query,
                 const float *v_out_means, const float *v_out_covars,
                 const float *v_out_opacities, float *v_means, float *v_covars,
                 float *v_opacities, float *v_betas, int32_t exact, void *stream);

/* ------------------------------------------------------------------ a6 ---
 * EWA perspective projection: _wrapper.py:185 (fully_fused_projection),
 * kernels fully_fused_projection_fwd.cu:20 / _bwd.cu:20.
 * means [N,3]; covars either [N,6] (upper triangle, covar_layout = 6) or
 * [N,3,3] (covar_layout = 9); or covars == NULL and quats [N,4] + scales [N,3].
 * viewmats [C,4,4] (world-to-camera, row-major), Ks [C,3,3].
 * radii [C,N] int32, means2d [C,N,2], depths [C,N], conics [C,N,3],
 * compensations [C,N] or NULL.  Culled entries get radius 0 and zeros.
 * Backward: v_* of the outputs in, gradients out (overwritten, summed over
 * cameras); v_covars uses covar_layout (for 9 the upper triangle holds the
 * gradient of the packed entries and the strict lower triangle is zero);
 * v_viewmats [C,4,4] or NULL. */
int ubs_projection_fwd(int32_t C, int64_t N, const float *means, const float *covars,
                       int32_t covar_layout, const float *quats, const float *scales,
                       const float *viewmats, const float *Ks, int32_t width, int32_t height,
                       float eps2d, float near_plane, float far_plane, float radius_clip,
                       int32_t *radii, float *means2d, float *depths, float *conics,
                       float *compensations, void *stream);
int ubs_projection_bwd(int32_t C, int64_t N, const float *means, const float *covars,
                       int32_t covar_layout, const float *quats, const float *scales,
                       const float *viewmats, const float *Ks, int32_t width, int32_t height,
                       float eps2d, const int32_t *radii, const float *conics,
                       const float *compensations, const float *v_means2d,
                       const float *v_depths, const float *v_conics,
                       const float *v_compensations, float *v_means, float *v_covars,
                       float *v_quats, float *v_scales, float *v_viewmats, void *stream);

/* ------------------------------------------------------------- a7 / a8 ---
 * Tile intersection: _wrapper.py:286 (isect_tiles), kernel isect_tiles.cu:17-285,
 * and offsets _wrapper.py:347 (isect_offset_encode), isect_tiles.cu:287-367.
 * Step 1 (synchronises the stream, like the reference's .item()):
 *   tiles_per_gauss [C,N], isect_offsets [C,tile_height,tile_width] and the
 *   intersection count.  Workspace: ubs_isect_count_workspace_bytes().
 *   It blocks the host because the drop-in operator returns isect_ids /
 *   flatten_ids as tensors whose length is the count, so the caller must
 *   know it before it can allocate them (the reference reads it with .item()
 *   at the same point, isect_tiles.cu:181).  The fused scene render below
 *   keeps the count on the device and never synchronises.
 * Step 2: isect_ids [n_isects] int64 (cam | tile | depth bits) and
 *   flatten_ids [n_isects] int32, sorted like the reference's stable radix sort
 *   when sort != 0, else in the reference's generation order.  Workspace:
 *   ubs_isect_sort_workspace_bytes(), its own buffer (step 2 reads nothing of
 *   step 1's workspace; the counts it needs are isect_offsets).
 * Depths of visible primitives must be non-negative (the reference's key then
 * overflows into the tile field); a negative one makes step 1 fail. */
size_t ubs_isect_count_workspace_bytes(int32_t C, int64_t N, int32_t n_tiles);
size_t ubs_isect_sort_workspace_bytes(int32_t C, int64_t N, int32_t n_tiles, int64_t n_isects);
int ubs_isect_count(int32_t C, int64_t N, const float *means2d, const int32_t *radii,
                    const float *depths, int32_t tile_size, int32_t tile_width,
                    int32_t tile_height, int32_t *tiles_per_gauss, int32_t *isect_offsets,
                    int64_t *n_isects, void *workspace, size_t workspace_bytes, void *stream);
int ubs_isect_emit(int32_t C, int64_t N, const float *means2d, const int32_t *radii,
                   const float *depths, int32_t tile_size, int32_t tile_width,
                   int32_t tile_height, const int32_t *tiles_per_gauss,
                   const int32_t *isect_offsets, int64_t n_isects, int32_t sort,
                   int64_t *isect_ids, int32_t *flatten_ids, void *workspace,
                   size_t workspace_bytes, void *stream);
/* offsets [C,tile_height,tile_width] from sorted isect_ids [n_isects]. */
int ubs_isect_offset_encode(int64_t n_isects, const int64_t *isect_ids, int32_t C,
                            int32_t tile_width, int32_t tile_height, int32_t *offsets,
                            void *stream);

/* ------------------------------------------------------------ a9 / a10 ---
 * Per-tile Beta-kernel blend: _wrapper.py:366 (rasterize_to_pixels),
 * kernels rasterize_to_pixels_fwd.cu:17 / _bwd.cu:17.
 * means2d [C,N,2], conics [C,N,3], colors [C,N,channels], opacities and betas
 * [C,N], backgrounds [C,channels] or NULL, masks [C,tile_height,tile_width]
 * uint8 or NULL, isect_offsets [C,tile_height,tile_width], flatten_ids
 * [n_isects].  Forward outputs: render_colors [C,H,W,channels], render_alphas
 * [C,H,W], last_ids [C,H,W] int32 (index of the last contributing sorted
 * intersection).  Backward outputs (overwritten): v_means2d, v_conics,
 * v_colors, v_opacities, v_betas; the background gradient is left to the
 * caller, as in the reference.  channels in {1-5, 8, 9, 16, 17, 32, 33};
 * tile_size in {8, 16, 24, 32}.  Workspace: ubs_raster_workspace_bytes().
 *
 * ubs_raster_fwd / _bwd = ubs_raster_pack (gather one record per sorted
 * intersection into the workspace) + ubs_raster_fwd_packed / _bwd_packed (the
 * blend kernels, which read only the packed records and `colors` for more than
 * 4 channels).  A packed workspace may serve one forward and its backward. */
size_t ubs_raster_workspace_bytes(int64_t n_isects, int32_t channels);
int ubs_raster_fwd(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                   const float *means2d, const float *conics, const float *colors,
                   const float *opacities, const float *betas, const float *backgrounds,
                   const uint8_t *masks, int32_t width, int32_t height, int32_t tile_size,
                   int32_t tile_width, int32_t tile_height, const int32_t *isect_offsets,
                   const int32_t *flatten_ids, float *render_colors, float *render_alphas,
                   int32_t *last_ids, void *workspace, size_t workspace_bytes, void *stream);
int ubs_raster_bwd(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                   const float *means2d, const float *conics, const float *colors,
                   const float *opacities, const float *betas, const float *backgrounds,
                   const uint8_t *masks, int32_t width, int32_t height, int32_t tile_size,
                   int32_t tile_width, int32_t tile_height, const int32_t *isect_offsets,
                   const int32_t *flatten_ids, const float *render_alphas,
                   const int32_t *last_ids, const float *v_render_colors,
                   const float *v_render_alphas, float *v_means2d, float *v_conics,
                   float *v_colors, float *v_opacities, float *v_betas, void *workspace,
                   size_t workspace_bytes, void *stream);
int ubs_raster_pack(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                    const int32_t *flatten_ids, const float *means2d, const float *conics,
                    const float *opacities, const float *betas, const float *colors,
                    void *workspace, size_t workspace_bytes, void *stream);
/* count_pairs != 0 also counts contributing (pixel, intersection) pairs into
 * the workspace header (read with ubs_raster_status). */
int ubs_raster_fwd_packed(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                          const float *colors, const float *backgrounds, const uint8_t *masks,
                          int32_t width, int32_t height, int32_t tile_size, int32_t tile_width,
                          int32_t tile_height, const int32_t *isect_offsets,
                          float *render_colors, float *render_alphas, int32_t *last_ids,
                          int32_t count_pairs, void *workspace, size_t workspace_bytes,
                          void *stream);
/* zero_outputs == 0 leaves the gradient buffers as given (caller zeroed them). */
int ubs_raster_bwd_packed(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                          const float *colors, const float *backgrounds, const uint8_t *masks,
                          int32_t width, int32_t height, int32_t tile_size, int32_t tile_width,
                          int32_t tile_height, const int32_t *isect_offsets,
                          const float *render_alphas, const int32_t *last_ids,
                          const float *v_render_colors, const float *v_render_alphas,
                          float *v_means2d, float *v_conics, float *v_colors, float *v_opacities,
                          float *v_betas, int32_t zero_outputs, void *workspace,
                          size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------ optimizer ---
 * One-launch Adam step over a scene's parameter tensors, the update of
 * torch.optim.Adam(groups, eps) as the reference trains with it
 * (scene/beta_model.py:239-276, train.py:170-171): per element
 *   m = m + (1 - beta1) (g - m);  v = v beta2 + (1 - beta2) g g;
 *   p = p + step_size m / (sqrt(v) / bc2 + eps)
 * with step_size = -lr / (1 - beta1^t) and bc2 = sqrt(1 - beta2^t) read from
 * device_hyper[2 * group], [2 * group + 1] (float, on the device, so that a
 * captured launch follows the host's per-step updates of that array).
 * 1 - beta1 and 1 - beta2 are passed as the caller rounds them (torch forms
 * them in double before rounding to float).
 * The table (device memory, ubs_adam_table_bytes) lists the tensors; fill a
 * host copy with ubs_adam_table_entry and copy it to the device.  max_numel
 * and total_numel are the largest and the summed element counts. */
size_t ubs_adam_table_bytes(int32_t n_tensors);
int ubs_adam_table_entry(void *host_table, int32_t index, float *param, const float *grad,
                         float *exp_avg, float *exp_avg_sq, int64_t numel, int32_t group);
int ubs_adam_step(int32_t n_tensors, const void *device_table, const float *device_hyper,
                  int64_t max_numel, int64_t total_numel, float one_minus_beta1, float beta2,
                  float one_minus_beta2, float eps, void *stream);

/* ----------------------------------------------------------------- loss ---
 * The training loss  weight_l1 * mean|img - gt| + weight_ssim * mean(SSIM map)
 * + weight_const  over a batch of images, with its gradient w.r.t. img in the
 * same call.  SSIM as utils/loss_utils.py:26-80 defines it (11 x 11 Gaussian
 * window, sigma 1.5, zero padding, C1 = 0.01^2, C2 = 0.03^2) and as the
 * fused_ssim package evaluates it for train.py:117-121; valid_padding != 0
 * averages the map only over points at least 5 pixels from every edge
 * (fused_ssim's padding="valid").  The reference's loss is weight_l1 = 1 - l,
 * weight_ssim = -l, weight_const = l with l = lambda_dssim; fused_ssim alone
 * is (0, 1, 0).
 * Layouts are free: element (image n, channel c, row y, column x) of img sits
 * at img + n s[0] + c s[1] + y s[2] + x s[3] for its strides s (int64[4]);
 * gt and grad likewise.  grad == NULL computes the loss only.
 * out (device, float[3]) receives mean(map), mean|img - gt| and the loss.
 * Two launches with the gradient (map and derivatives; the gradient), one
 * without.  The workspace (ubs_ssim_workspace_bytes: a header, per-CTA
 * partials and three derivative planes of the batch) needs only its first 256
 * bytes zero before its first use; every call leaves them zero again, so it
 * can be reused by calls ordered on one stream (and by captured launches). */
size_t ubs_ssim_workspace_bytes(int32_t n_images, int32_t channels, int32_t height,
                                int32_t width);
int ubs_ssim_loss(const float *img, const int64_t *img_strides, const float *gt,
                  const int64_t *gt_strides, float *grad, const int64_t *grad_strides,
                  int32_t n_images, int32_t channels, int32_t height, int32_t width,
                  int32_t valid_padding, double weight_l1, double weight_ssim,
                  double weight_const, float *out, void *workspace, size_t workspace_bytes,
                  void *stream);

/* The L1 term alone (utils/loss_utils.py:18-19, train.py:117): out[0] =
 * mean |x - y| over n contiguous floats, out[1] = weight out[0], and (grad
 * != NULL) grad = weight sign(x - y) / n, in one launch.  Workspace as for
 * ubs_ssim_loss: the first 256 bytes zero before first use, left zero. */
size_t ubs_l1_loss_workspace_bytes(int64_t n);
int ubs_l1_loss(const float *x, const float *y, float *grad, int64_t n, double weight,
                float *out, void *workspace, size_t workspace_bytes, void *stream);

/* --------------------------------------------------- MCMC densification ---
 * BetaModel.relocate_gs / add_new_gs (scene/beta_model.py:553-658) and the
 * position noise of train.py:164-171, on the device with no host
 * synchronisation (sizes never depend on the data, so the calls can be
 * captured in a CUDA graph).
 * A scene is a set of per-primitive FP32 tensors [n, width[k]] (the
 * reference's seven: xyz, mean, rgb, opacity, beta, scale, l_triangle) with
 * their Adam moments (NULL where a tensor has no optimizer state yet). */
#define UBS_MCMC_MAX_TENSORS 8
typedef struct ubs_mcmc_tensors {
    int32_t n_tensors;     /* 1 .. UBS_MCMC_MAX_TENSORS                       */
    int32_t opacity_index; /* the raw (pre-sigmoid) opacity, width 1           */
    int32_t width[UBS_MCMC_MAX_TENSORS];
    float *param[UBS_MCMC_MAX_TENSORS];
    float *exp_avg[UBS_MCMC_MAX_TENSORS];
    float *exp_avg_sq[UBS_MCMC_MAX_TENSORS];
} ubs_mcmc_tensors;

size_t ubs_mcmc_workspace_bytes(int64_t n_prims, int64_t n_draw_max);
/* In place: every dead primitive (dead_mask[i] != 0, or, with a NULL mask,
 * sigmoid(raw opacity) <= dead_threshold) becomes a copy of a live one drawn
 * with probability proportional to its opacity; a primitive drawn c times and
 * its c copies share logit(clamp(1 - (1 - o)^(1/(c+1)), 0.005, 1 - eps));
 * the drawn primitives' Adam moments are zeroed.  Draws come from a counter-
 * based generator keyed by `seed`, or from given_src (n_given live indices,
 * one per dead primitive in index order) to reproduce other draws.  No live
 * primitive: nothing changes.  Bad given indices set a bit in *status
 * (device word, not cleared). */
int ubs_mcmc_relocate(const ubs_mcmc_tensors *scene, int64_t n_prims, const uint8_t *dead_mask,
                      float dead_threshold, uint64_t seed, const int64_t *given_src,
                      int64_t n_given, uint32_t *status, void *workspace,
                      size_t workspace_bytes, void *stream);
/* Writes `grown` (tensors of n_prims + n_add rows, the scene's widths and
 * moment layout): rows < n_prims copy the scene, drawn primitives with their
 * split opacity and zero moments; row n_prims + j copies the j-th draw (from
 * all primitives, proportional to opacity, or given_src[j]) with the split
 * opacity and zero moments. */
int ubs_mcmc_add(const ubs_mcmc_tensors *scene, const ubs_mcmc_tensors *grown, int64_t n_prims,
                 int64_t n_add, uint64_t seed, const int64_t *given_src, uint32_t *status,
                 void *workspace, size_t workspace_bytes, void *stream);
/* xyz += Sigma_xyz (z (1 - sigmoid(raw_opacity))^100 factor) with z standard
 * normal (given_noise [n, 3], or drawn from `seed`), Sigma_xyz = R diag(s^2)
 * R^T, s = softplus(raw_scale[:, :3]) (row stride dim), R = I + A from
 * l_triangle[:, :3] (row stride dim (dim - 1) / 2); factor = noise_lr * lr. */
int ubs_mcmc_perturb_xyz(int64_t n_prims, int32_t dim, float *xyz, const float *raw_opacity,
                         const float *raw_scale, const float *l_triangle, float factor,
                         uint64_t seed, const float *given_noise, void *stream);

/* ----------------------------------------------------------- scene files ---
 * The reference's scene file (scene/beta_model.py:286-404): one PLY "vertex"
 * element of float32 properties x, y, z, red, green, blue, opacity, beta_i,
 * mean_i, scale_i, l_triangle_i, binary little-endian.
 * ubs_ply_read_header parses a header (comments and obj_info lines allowed;
 * other elements only if empty; vertex properties must all be float) and
 * returns the vertex count, the property count, the property names (when
 * `names` is given: UBS_PLY_NAME_BYTES bytes each, NUL-terminated, at most
 * names_capacity of them) and the byte offset of the body; ascii or
 * big-endian files return UBS_ERR_UNSUPPORTED.
 * ubs_ply_read_body reads n_bytes of the body from `offset` into host memory
 * (pinned memory lets the caller overlap the next read with the copy to the
 * device).  ubs_ply_write writes a header with the given names and the
 * records (n_vertices x n_props float32, host memory).
 * ubs_ply_unpack scatters device records [n, record_floats] into the layout's
 * tensors; ubs_ply_pack gathers them back (unmapped properties read 0). */
#define UBS_PLY_MAX_TENSORS 8
#define UBS_PLY_MAX_PROPS 256
#define UBS_PLY_NAME_BYTES 64
typedef struct ubs_ply_layout {
    int32_t record_floats;                  /* properties per vertex           */
    int32_t n_tensors;                      /* 0 .. UBS_PLY_MAX_TENSORS        */
    int32_t width[UBS_PLY_MAX_TENSORS];     /* floats per primitive            */
    float *param[UBS_PLY_MAX_TENSORS];      /* device tensors [n, width]       */
    int16_t tensor_of[UBS_PLY_MAX_PROPS];   /* property -> tensor, -1: skipped */
    int16_t column_of[UBS_PLY_MAX_PROPS];   /* property -> column in its tensor */
} ubs_ply_layout;
int ubs_ply_read_header(const char *path, int64_t *n_vertices, int32_t *n_props, char *names,
                        int32_t names_capacity, int64_t *body_offset);
int ubs_ply_read_body(const char *path, int64_t offset, void *dst, int64_t n_bytes);
int ubs_ply_write(const char *path, int64_t n_vertices, int32_t n_props, const char *names,
                  const void *records);
int ubs_ply_unpack(const ubs_ply_layout *layout, const float *records, int64_t n_vertices,
                   void *stream);
int ubs_ply_pack(const ubs_ply_layout *layout, float *records, int64_t n_vertices,
                 void *stream);

/* ---------------------------------------------------------------- viewer ---
 * Per-frame work of the reference's viewer render (BetaModel.view,
 * scene/beta_model.py:725-831) besides the render itself.
 * ubs_quantile_mask: mask[i] = 1 where every value array a lies within
 * [quantile(lo_a), quantile(hi_a)] of its n values -- quantiles[] = {lo, hi}
 * per array, in [0, 1] -- with torch.quantile's linear interpolation (rank
 * q (n - 1) in float32; a NaN value makes that array's bounds NaN and the
 * mask 0).  arrays[a] (device) has element stride strides[a]; the viewer's
 * arrays are raw_beta[:, 0], raw_beta[:, 1:4].mean(-1) and, 7-D,
 * raw_beta[:, 4] (quantile_mask, scene/beta_model.py:729-757).  The order
 * statistics are exact (radix select on the device).
 * ubs_quantile_mask_bounds copies the 2 n_arrays bounds of the last mask
 * computed in `workspace` to device memory.
 * ubs_depth_colormap (utils/general_utils.py:172-218): out[i] = table[idx]
 * (table: device float [256][3]) with idx = trunc(255 clip((x - min) /
 * (max - min + 1e-10), 0, 1)) over the image's own min and max, NaN -> 0;
 * workspace: 16 bytes of device memory. */
size_t ubs_quantile_mask_workspace_bytes(void);
int ubs_quantile_mask(int64_t n, int32_t n_arrays, const float *const *arrays,
                      const int64_t *strides, const double *quantiles, uint8_t *mask,
                      void *workspace, size_t workspace_bytes, void *stream);
int ubs_quantile_mask_bounds(const void *workspace, int32_t n_arrays, float *bounds_out,
                             void *stream);
int ubs_depth_colormap(const float *image, int64_t n_pixels, const float *table, float *out,
                       void *workspace, void *stream);

/* Forward blend without a workspace (no counterpart in the reference).
 * Same arguments, results and errors as ubs_raster_fwd minus the workspace,
 * for callers that cannot allocate device memory where they render (a host
 * callback or real-time thread that must stay out of the CUDA allocator, or an
 * application whose memory pool is fixed).  It allocates nothing: the packed
 * records go to a fixed scratch array in the library's static device memory,
 * 256 B + 48 B x UBS_RASTER_NOALLOC_MAX_ISECTS (24 MiB), one per device.
 *   - n_isects above UBS_RASTER_NOALLOC_MAX_ISECTS returns UBS_ERR_OVERFLOW.
 *   - The first call on a device looks the scratch address up (set-up work);
 *     make it before capturing a stream.
 *   - Nothing has to start at zero: each call clears the scratch's status
 *     header on `stream` itself.
 *   - One scratch per device: calls on the same device must not overlap in
 *     time (two streams, or unordered host threads, race on the records).
 *   - The scratch address is looked up once per device and kept for the life
 *     of the process: after cudaDeviceReset on a device, do not call the
 *     no-allocation entry points on that device again.
 *   - Device-side status bits (8: a flatten index outside [0, C*N); 1: a
 *     bounded wait ran out) go to the scratch's header; read them with
 *     ubs_raster_noalloc_status (synchronises `stream`; the next call clears
 *     them). */
#define UBS_RASTER_NOALLOC_MAX_ISECTS 524288
int ubs_raster_fwd_noalloc(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                           const float *means2d, const float *conics, const float *colors,
                           const float *opacities, const float *betas, const float *backgrounds,
                           const uint8_t *masks, int32_t width, int32_t height, int32_t tile_size,
                           int32_t tile_width, int32_t tile_height, const int32_t *isect_offsets,
                           const int32_t *flatten_ids, float *render_colors, float *render_alphas,
                           int32_t *last_ids, void *stream);
/* Status word of the last ubs_raster_fwd_noalloc on the current device (no
 * reference counterpart): bits as ubs_raster_status; synchronises `stream`. */
int ubs_raster_noalloc_status(uint32_t *status, void *stream);

/* ------------------------------------------------------- fused multi-view ---
 * One render of a Universal Beta Splatting scene into C views at once (no
 * single reference counterpart: it fuses the reference model's render,
 * scene/beta_model.py:660-722, with rasterization(), rendering.py:17-232).
 * Raw (pre-activation) parameters as the reference model stores them: xyz
 * [N,3], mean [N,dim-3], scale [N,dim] (softplus), l_triangle
 * [N,dim*(dim-1)/2] (first 3 = rotation skew, rest = strictly-lower entries of
 * rows 3..dim-1, row-major), opacity [N] (sigmoid), beta [N,dim-2] (4 exp;
 * beta[:,0] spatial), rgb [N,3]; dim in {6, 7}.
 * Views: viewmats [C,16] world-to-camera row-major, intrinsics [C,4]
 * (fx, fy, cx, cy), centers [C,3] camera centres, timestamps [C] (dim 7; may be
 * NULL for dim 6), view_dims [C,4] (width, height, tile columns, tile rows),
 * tile_base [C+1] (first (view, tile) bucket of each view; tile_base[C] =
 * n_buckets), pix_base [C+1] (first pixel of each view).  Images are one flat
 * buffer: render_colors [P,3], render_alphas [P], last_ids [P], P = pix_base[C].
 * backgrounds [C,3] or NULL.  `capacity` bounds the number of intersections
 * held in the workspace (ubs_scene_workspace_bytes); a frame that needs more
 * sets status bit 4 (read with ubs_scene_stats) and must be re-rendered with a
 * larger capacity.  No host synchronisation: both calls can be captured in a
 * CUDA graph.  The backward uses the workspace of the forward it follows and
 * overwrites the raw-parameter gradients (summed over views). */
size_t ubs_scene_workspace_bytes(int32_t C, int64_t N, int32_t n_buckets, int64_t capacity);
int ubs_scene_forward(int32_t dim, int64_t N, const float *xyz, const float *mean,
                      const float *scale, const float *l_triangle, const float *opacity,
                      const float *beta, const float *rgb, int32_t C, const float *viewmats,
                      const float *intrinsics, const float *centers, const float *timestamps,
                      const int32_t *view_dims, const int32_t *tile_base,
                      const int64_t *pix_base, int32_t n_buckets, int32_t tile_size,
                      float eps2d, float near_plane, float far_plane, float radius_clip,
                      const float *backgrounds, float *render_colors, float *render_alphas,
                      int32_t *last_ids, int64_t capacity, void *workspace,
                      size_t workspace_bytes, void *stream);
/* Byte offsets, inside a forward's workspace, of the per-(view, primitive)
 * radii (int32 [C, N]; 0: not rendered) and depths (float [C, N]) it leaves
 * there -- the reference's meta["radii"] / meta["depths"]. */
int ubs_scene_workspace_offsets(int32_t C, int64_t N, int32_t n_buckets, int64_t capacity,
                                int64_t *radius_offset, int64_t *depth_offset);
/* Byte offsets, inside a forward's workspace, of what the forward leaves
 * there (sections[i] for i < n_sections, in the order of the UBS_SCENE_WS_*
 * indices):
 *   RECORDS  per (view, primitive) 32-B records {x, y, opacity, beta, conic
 *            xx, xy, yy, entry id} -- meta["means2d"] / ["conics"] of the
 *            reference (fully_fused_projection_fwd.cu:20-177), zeros where the
 *            radius is 0;
 *   RADII    int32 [C, N], DEPTHS float [C, N] (as ubs_scene_workspace_offsets);
 *   BUCKET_STARTS  int32 [n_buckets]: first intersection of bucket b =
 *            tile_base[view] + tile (an exclusive scan of the counts; the last
 *            bucket ends at the intersection total, ubs_scene_stats);
 *   KEYS     uint64 [total], sorted within each bucket: float bits of the
 *            depth << 32 | view * N + primitive.
 * Per view, tile << 32 | key >> 32 is the reference's single-camera isect id
 * and the low word minus view * N its flatten id, in the same order
 * (isect_tiles.cu:82-96, 232-280, 287-367). */
#define UBS_SCENE_WS_RECORDS 0
#define UBS_SCENE_WS_RADII 1
#define UBS_SCENE_WS_DEPTHS 2
#define UBS_SCENE_WS_BUCKET_STARTS 3
#define UBS_SCENE_WS_KEYS 4
#define UBS_SCENE_WS_N_SECTIONS 5
int ubs_scene_workspace_layout(int32_t C, int64_t N, int32_t n_buckets, int64_t capacity,
                               int64_t *sections, int32_t n_sections);
/* ubs_scene_forward with two viewer options (scene/beta_model.py:725-831):
 * prim_mask (device uint8 [N], or NULL) leaves out primitives whose entry is
 * 0 -- the same image as rendering the masked subset, as the reference's
 * means[mask] ... does; color_mode 1 renders each primitive's depth in
 * channel 0 (channels 1, 2 zero; one view; forward only), the reference's
 * "Depth" mode when the backgrounds are zero. */
int ubs_scene_forward_masked(int32_t dim, int64_t N, const float *xyz, const float *mean,
                             const float *scale, const float *l_triangle, const float *opacity,
                             const float *beta, const float *rgb, int32_t C,
                             const float *viewmats, const float *intrinsics,
                             const float *centers, const float *timestamps,
                             const int32_t *view_dims, const int32_t *tile_base,
                             const int64_t *pix_base, int32_t n_buckets, int32_t tile_size,
                             float eps2d, float near_plane, float far_plane, float radius_clip,
                             const float *backgrounds, float *render_colors,
                             float *render_alphas, int32_t *last_ids, int64_t capacity,
                             void *workspace, size_t workspace_bytes, const uint8_t *prim_mask,
                             int32_t color_mode, void *stream);
int ubs_scene_backward(int32_t dim, int64_t N, const float *xyz, const float *mean,
                       const float *scale, const float *l_triangle, const float *opacity,
                       const float *beta, const float *rgb, int32_t C, const float *viewmats,
                       const float *intrinsics, const float *centers, const float *timestamps,
                       const int32_t *view_dims, const int32_t *tile_base,
                       const int64_t *pix_base, int32_t n_buckets, int32_t tile_size,
                       float eps2d, float near_plane, float far_plane, float radius_clip,
                       const float *backgrounds, const float *render_alphas,
                       const int32_t *last_ids, const float *v_render_colors,
                       const float *v_render_alphas, float *v_xyz, float *v_mean, float *v_scale,
                       float *v_l_triangle, float *v_opacity, float *v_beta, float *v_rgb,
                       int32_t exact_cond_grad, int64_t capacity, void *workspace,
                       size_t workspace_bytes, void *stream);
/* Intersections counted by the last forward on `workspace` and its device
 * status word; synchronises the stream. */
int ubs_scene_stats(const void *workspace, int64_t *n_isects, uint32_t *status, void *stream);

/* Occupancy variant of the blend kernels (no reference counterpart; the
 * reference's launch shape is fixed, rasterize_to_pixels_fwd.cu:269-292):
 * for 3 channels and tiles of at most 16 x 16 pixels the forward's variants
 * trade records per staged batch against CTAs per SM, the backward's the
 * register bound and the way a batch's per-record sums are accumulated --
 *   forward:  0 (default): 256-record batches, 8 CTAs per SM;
 *             1: 128-record batches, 10 CTAs per SM; 2: 256-record, 6 CTAs per SM
 *   backward: 0 (default): 128-record batches, 8 CTAs per SM, per-warp lists
 *             of reduced sums written with plain stores;
 *             1: the same at 7 CTAs per SM; 2: 128-record batches, 8 CTAs per
 *             SM, one shared accumulator row per record (shared atomics)
 * (for 16 x 16 tiles; an 8 x 8 tile's batches are a quarter of that).
 * Process-wide: it applies to every later launch from any thread (an
 * autotuner sets it between measured steps, outside stream capture).  Images
 * are identical under every variant; backward gradients agree up to the order
 * of their atomic sums. */
int ubs_set_blend_variant(int32_t forward, int32_t backward);
int ubs_get_blend_variant(int32_t *forward, int32_t *backward);

/* Device status word (bits: 1 wait timeout, 2 negative depth, 4 overflow,
 * 8 bad flatten index) and the contributing-pair count of the last packed
 * blend on `workspace` (pair_count may be NULL); synchronises the stream. */
int ubs_raster_status(const void *workspace, uint32_t *status, uint64_t *pair_count,
                      void *stream);
/* After a forward with count_pairs != 0: counts[0] contributing (pixel,
 * record) pairs, counts[1] pairs a per-pixel blend loop evaluates (each
 * pixel's records up to the one that ends it, else its tile's whole range),
 * counts[2] pairs up to each pixel's last contributor (what the backward
 * walks).  Synchronises the stream. */
int ubs_raster_pair_counts(const void *workspace, uint64_t *counts, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* UBS_GB300_H */
