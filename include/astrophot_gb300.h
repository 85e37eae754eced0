/*
 * astrophot_gb300 -- C ABI of the GB300 (sm_103a) render + Levenberg-Marquardt path.
 *
 * Conventions
 *   - Every entry point returns an int status: AP_OK (0) or one of AP_ERR_*.
 *   - Device pointers are plain pointers to caller-owned CUDA memory; nothing in this
 *     library calls cudaMalloc/cudaFree.  Work buffers come from the caller through
 *     ap_batch_bind (size from ap_batch_sizes) and ap_lm_fit (size from
 *     ap_lm_workspace_bytes).
 *   - All device work is enqueued on the stream passed in; calls do not synchronise
 *     unless stated.  One host thread per batch handle; a handle is not thread-safe.
 *   - Images are row-major [ny][nx] float32, packed stamp after stamp at the offsets
 *     returned by ap_batch_offsets.  Parameters are float64.
 *   - The full parameter vector of a stamp is [cx, cy, q, PA, n, Re, Ie, F]
 *     (centre in plane units, PA in radians, Ie and F as log10 of the surface
 *     brightness, F the flat sky).  options.free_mask selects the fitted slots; the
 *     compact vector of fitted slots keeps this order.
 *
 * Reference interfaces replaced (AstroPhot 0.x, file:line in its repository):
 *   ap_render        Component_Model.sample          astrophot/models/model_object.py:258-375
 *                    (+ Group_Model.sample for galaxy + flat sky, models/group_model_object.py:183-231)
 *   ap_jacobian      jacobian(as_representation=...) astrophot/models/_model_methods.py:260-347
 *   ap_psf_shift     _shift_psf (bilinear) + renorm  astrophot/models/_model_methods.py:187-243
 *   ap_damped_solve  LM._h                           astrophot/fit/lm.py:361-371
 *   ap_lm_fit        LM.fit / LM.step                astrophot/fit/lm.py:249-357, 428-493
 *   ap_chi2          LM._chi2                        astrophot/fit/lm.py:374-378
 */
#ifndef ASTROPHOT_GB300_H
#define ASTROPHOT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* ap_stream_t; /* same handle as cudaStream_t */

/* status codes */
#define AP_OK 0
#define AP_ERR_ARG 1          /* bad argument (null pointer, size, shape) */
#define AP_ERR_UNSUPPORTED 2  /* knob outside what the kernels implement */
#define AP_ERR_CUDA 3         /* a CUDA launch or copy failed */
#define AP_ERR_WORKSPACE 4    /* workspace missing or too small */
#define AP_ERR_LIMIT 5        /* a parameter left its limits (InvalidParameter) */
#define AP_ERR_NOT_BOUND 6    /* ap_batch_bind was not called */

/* ap_options.profile */
#define AP_PROFILE_SERSIC 0
#define AP_PROFILE_EXPONENTIAL 1
/* Moffat (Moffat_PSF / Moffat_Galaxy, astrophot/models/moffat_model.py:71-120):
 * I0 / (1 + (R/Rd)^2)^n with n in slot n, Rd in slot Re, log10 I0 in slot Ie; limits of n
 * (0.1, 10).  Render, Jacobian and adjoint only (ap_lm_fit and ap_reference_init return
 * AP_ERR_UNSUPPORTED): a fitted PSF's parameters are fitted by the scene LM. */
#define AP_PROFILE_MOFFAT 2
/* Gaussian (Gaussian_PSF, astrophot/models/gaussian_model.py:255-290): 10^flux / sqrt(2 pi
 * sigma^2) exp(-R^2 / (2 sigma^2)) with sigma in slot Re and flux in slot Ie; no n.  Render,
 * Jacobian and adjoint only, like the Moffat profile. */
#define AP_PROFILE_GAUSSIAN 3
/* ap_options.sampling_mode */
#define AP_SAMPLING_MIDPOINT 0
#define AP_SAMPLING_SIMPSONS 1
#define AP_SAMPLING_QUAD 2
#define AP_SAMPLING_TRAPEZOID 3
/* Midpoint sampling with the pixels whose centres lie within options.center_radius pixels of
 * the model centre (squared distance <= radius^2 + 1e-6) integrated by
 * sampling_quad_level x sampling_quad_level Gauss-Legendre points (the reference's
 * single_quad_integrate, astrophot/utils/operations.py:123-147, on those pixels of its midpoint
 * image, astrophot/models/_model_methods.py:84-87): "midpoint sampling plus 3 x 3 supersampling
 * within 2 px of the centre".  No counterpart mode in the reference.  integrate_mode must be
 * AP_INTEGRATE_NONE. */
#define AP_SAMPLING_MIDPOINT_CENTER 4
/* ap_options.integrate_mode */
#define AP_INTEGRATE_NONE 0
#define AP_INTEGRATE_THRESHOLD 1
/* ap_options.psf_mode */
#define AP_PSF_NONE 0
#define AP_PSF_FULL 1         /* psf_mode="full", psf_subpixel_shift="bilinear" */
#define AP_PSF_FULL_NOSHIFT 2 /* psf_mode="full", psf_subpixel_shift="none" */

/* per-stamp LM status (ap_lm_fit status_out) */
#define AP_LM_RUNNING 0
#define AP_LM_SUCCESS 1          /* "success" */
#define AP_LM_IMMOBILE 2         /* "success by immobility. Convergence not guaranteed" */
#define AP_LM_MAX_ITER 3         /* "fail. Maximum iterations" */
#define AP_LM_NO_STEP 4          /* "fail. Could not find step to improve Chi^2" (OptimizeStop) */
#define AP_LM_LIMIT 5            /* a trial parameter left its limits (InvalidParameter) */

typedef struct ap_options {
  int32_t profile;              /* AP_PROFILE_* */
  int32_t sampling_mode;        /* AP_SAMPLING_* */
  int32_t sampling_quad_level;  /* k of sampling_mode "quad:k" (1..5) */
  int32_t integrate_mode;       /* AP_INTEGRATE_* */
  int32_t psf_mode;             /* AP_PSF_* */
  int32_t integrate_max_depth;  /* 1..3   (reference default 3) */
  int32_t integrate_gridding;   /* 1..5   (reference default 5) */
  int32_t integrate_quad_level; /* 1..5   (reference default 3) */
  double sampling_tolerance;    /* reference default 1e-2 */
  double softening;             /* reference default 1e-3 */
  int32_t free_mask;            /* bit i set: full-vector slot i is fitted */
  int32_t has_sky;              /* 1: a flat sky 10^F * pixel_area is added */
  int32_t fft_min_kernel;       /* stamps whose convolution kernel side (with the shift
                                   padding) is at least this are convolved by FFT
                                   (psf_convolve_mode "fft", models/_model_methods.py:245-257);
                                   0 = direct convolution for every stamp */
  double center_radius;         /* AP_SAMPLING_MIDPOINT_CENTER: radius in pixels (2) */
  int32_t lanczos_order;        /* psf_mode AP_PSF_FULL: 0 = bilinear sub-pixel shift (the
                                   reference default); k = 1..8: psf_subpixel_shift "lanczos:k"
                                   (models/_model_methods.py:209-227): the kernel grows by 2k
                                   instead of 2, and the LM renders its trials in full (no
                                   difference form; ap_render_precise refuses such batches) */
} ap_options;

typedef struct ap_lm_options {
  int32_t max_iter;         /* LM max_iter (100) */
  int32_t max_step_iter;    /* inner damping search (10) */
  double relative_tolerance;/* 1e-5 */
  double curvature_limit;   /* 1.0 */
  double Lup, Ldn, L0;      /* 11, 9, 1 */
  double acceleration;      /* 0 */
  int32_t rounds_per_sync;  /* device rounds between host checks of the active count (>= 1) */
  int32_t use_graph;        /* 1: capture rounds_per_sync rounds in a CUDA graph and replay it */
  int32_t precise_trials;   /* 1 (default): render each damping trial as its difference to the
                               step's base point (sample, kernel and convolution differences formed
                               from the exact parameter differences), so chi^2 changes far below
                               the FP32 rendering error of one model (the reference compares
                               float64 chi^2 values near convergence) decide the damping search,
                               the curvature test and convergence as in float64 (Sersic and
                               exponential stamps, direct or FFT convolution).  0: plain FP32
                               trial renders. */
} ap_lm_options;

typedef struct ap_batch ap_batch; /* opaque host-side plan (host memory only) */

/* Plan a batch of n stamps.  geometry holds 8 doubles per stamp:
 *   P00 P01 P10 P11 (pixel-scale matrix, plane = P (ij - ref_ij) + ref_xy),
 *   ref_i ref_j (reference pixel, x then y), ref_x ref_y (reference plane point).
 * psf_kx/psf_ky may be NULL when options.psf_mode == AP_PSF_NONE; otherwise odd sizes.
 * Host-only; no CUDA call. */
int ap_batch_create(ap_batch** out, int32_t n_stamps, const int32_t* nx, const int32_t* ny,
                    const int32_t* psf_kx, const int32_t* psf_ky, const double* geometry,
                    const ap_options* options);
int ap_batch_destroy(ap_batch* batch);

/* Packed sizes: output pixels (data/weight/mask/model layout), raw PSF pixels, and the
 * workspace bytes ap_batch_bind needs. */
int ap_batch_sizes(const ap_batch* batch, int64_t* out_pixels, int64_t* psf_pixels,
                   int64_t* workspace_bytes);
/* Per-stamp offsets (host arrays of n_stamps) into the packed output and PSF arrays. */
int ap_batch_offsets(const ap_batch* batch, int64_t* out_offsets, int64_t* psf_offsets);

/* Pixel count each stamp's adaptive-integration threshold divides by (default: its working
 * window, as _integrate_reference / sampling_tolerance in the reference, models/sersic_model.py:
 * 87-89).  A Sersic source of a Group_Model is evaluated by the reference on the group's window
 * (models/model_object.py:290-296); rendering it on its own window with the group's working
 * pixel count gives the same pixels inside its window.  numel[n] > 0, host; may follow bind. */
int ap_batch_set_threshold_numel(ap_batch* batch, const double* numel);

/* The window whose samples an exponential (or PSF-profile) stamp's integration threshold sums,
 * in place of its own working window: windows[n][4] = x0, y0, nx, ny in the stamp's working-pixel
 * indices (x0, y0 may be negative; nx = 0 keeps the own window).  The reference evaluates a
 * windowed source of a Group_Model on the group's working window (models/model_object.py:290-296)
 * and its default _integrate_reference sums the samples there (models/_model_methods.py:151-152);
 * with the group's working window here (and ap_batch_set_threshold_numel) the source renders on
 * its own window with the same pixels, the sum taken by a separate sampling pass.  Host; may
 * follow bind. */
int ap_batch_set_threshold_window(ap_batch* batch, const int32_t* windows);

/* Attach caller-owned device workspace and upload the plan's tables into it
 * (synchronous with respect to the host for the table upload). */
int ap_batch_bind(ap_batch* batch, void* workspace, int64_t workspace_bytes, ap_stream_t stream);

/* Model images of every stamp for value-space parameters params[n][8] (device).
 * model[out_pixels] (device) is overwritten.  psf: packed raw PSFs (device) or NULL. */
int ap_render(ap_batch* batch, const double* params, const float* psf, float* model,
              ap_stream_t stream);

/* Model and Jacobian.  jac[n_free][out_pixels] (device), compact fitted-slot order;
 * as_representation != 0 gives d model / d representation (the LM's space). */
int ap_jacobian(ap_batch* batch, const double* params, const float* psf, float* model,
                float* jac, int32_t as_representation, ap_stream_t stream);

/* Derivative of the render along a change of the PSF image (a fitted PSF model's parameter):
 * with N(K) = S(K) / sum S(K) the shifted, renormalised kernel of a raw PSF K (S: the bilinear
 * shift, or the identity under AP_PSF_FULL_NOSHIFT), model[out_pixels] = the stamp's
 * pre-convolution image convolved with dN = (S(dpsf) - N(psf) sum S(dpsf)) / sum S(psf), i.e.
 * d model / d theta for dpsf = d psf / d theta.  psf and dpsf are packed like ap_render's psf.
 * Needs psf_mode != AP_PSF_NONE and no sky (the sky does not depend on the PSF).  Replaces
 * autograd through the live PSF of a model with an auxiliary PSF model: the PSF image sampled
 * each evaluation (astrophot/models/model_object.py:133-149, 306-312) and convolved by
 * _sample_convolve (astrophot/models/_model_methods.py:233-257). */
int ap_render_psf_derivative(ap_batch* batch, const double* params, const float* psf, const float* dpsf,
                             float* model, ap_stream_t stream);

/* Renders for damping trials that must compare chi^2 values closer than one float32 render's
 * rounding (a joint LM near its optimum, where the reference's float64 chi^2 still sees the
 * change).  mode AP_RENDER_BASE: model = ap_render's model, and the evaluation (its constants,
 * shifted kernel, deep image and integration pattern) is recorded in `base`.  mode
 * AP_RENDER_DIFFERENCE: model = the render at params minus the recorded base render, each
 * sample's difference formed from the exact parameter differences (a pixel whose integration
 * pattern changed is differenced from the rounded values), so the change is accurate relative
 * to itself, not to the model.  base: device buffer of ap_render_base_bytes bytes, 16-byte
 * aligned, one per parameter set rendered on the batch (a second BASE overwrites it).  Sersic
 * and exponential batches only (AP_ERR_UNSUPPORTED otherwise).  Replaces, for the joint fit
 * of many sources, the float64 trial renders of LM.step (astrophot/fit/lm.py:270-300), like
 * the batched LM's precise_trials. */
#define AP_RENDER_BASE 1
#define AP_RENDER_DIFFERENCE 2
int ap_render_base_bytes(const ap_batch* batch, int64_t* bytes);
int ap_render_precise(ap_batch* batch, const double* params, const float* psf, float* model, void* base,
                      int64_t base_bytes, int32_t mode, ap_stream_t stream);

/* A PSF model's normalisation (PSF_Model.sample, normalize_psf: the image divided by its sum,
 * astrophot/models/psf_model_object.py:250-252) and its derivative: out = img / S and
 * dout[c] = (dimg[c] - out sum dimg[c]) / S for n_dir <= 8 directions, S = sum img (float64
 * sums).  img[n_pix], dimg[n_dir][n_pix], out, dout: device. */
int ap_psf_normalize(int32_t n_pix, int32_t n_dir, const float* img, const float* dimg, float* out, float* dout,
                     ap_stream_t stream);

/* Adjoint of the render (vector-Jacobian product): grad_params[n][n_free] (device, float64)
 * = sum over each stamp's output pixels of grad_model * d model / d theta, theta the fitted
 * slots in value space or, with AP_VJP_REPRESENTATION, in representation space.
 * grad_model[out_pixels] (device, float32) is the upstream gradient d loss / d model in the
 * output layout (weights and masks are the caller's).  The PSF-convolved derivative tiles are
 * computed and reduced on the fly, never stored.  Replaces autograd's backward through
 * Component_Model.sample (negative_log_likelihood().backward(),
 * astrophot/models/core_model.py:220-256).
 *
 * Center columns under AP_PSF_FULL: the derivative of the render (what ap_jacobian returns, what
 * the reference's forward-mode jacobian() returns, and what finite differences give) flows only
 * through the sub-pixel PSF shift.  The reference's reverse-mode autograd adds the
 * sampling-coordinate path -d profile / d(x, y) on top (the pixel_shift of the working window,
 * astrophot/models/model_object.py:319-323, is not seen by backward); AP_VJP_REFERENCE_CENTER
 * reproduces that value (two extra convolved planes). */
#define AP_VJP_REPRESENTATION 1
#define AP_VJP_REFERENCE_CENTER 2
int ap_render_vjp(ap_batch* batch, const double* params, const float* psf, const float* grad_model,
                  int32_t flags, double* grad_params, ap_stream_t stream);

/* In-project autotuner of the render pass: times the full render pass (forward, or with the
 * Jacobian when jacobian != 0) at params[n][8] for candidate persistent-grid sizes of each
 * kernel group (blocks per SM of sample/select, integration, convolution, PSF shift), one group
 * at a time, keeps the fastest and returns them in chosen[4] (best_ms: the pass time).  Not
 * inside a stream capture; synchronises the stream.  ap_batch_set_grid sets them directly. */
int ap_batch_autotune(ap_batch* batch, const double* params, const float* psf, int32_t jacobian,
                      int32_t* chosen, double* best_ms, ap_stream_t stream);
int ap_batch_set_grid(ap_batch* batch, const int32_t* blocks_per_sm);

/* Value -> representation of the fitted slots (boundaries / cyclic_boundaries,
 * astrophot/utils/conversions/optimization.py:6-54): values[n][8] -> rep[n][popcount(free_mask)],
 * device pointers; the representation vector ap_lm_fit starts from. */
int ap_values_to_rep(const double* values, int32_t n, int32_t free_mask, double* rep,
                     ap_stream_t stream);

/* The reference's own initial values of a Sérsic / exponential galaxy on every stamp of a bound
 * batch: what ``Model.initialize()`` finds for the parameters that have no value
 * (astrophot/models/model_object.py:180-233 centre of light,
 * astrophot/models/galaxy_model_object.py:60-113 PA and isophote q,
 * astrophot/models/_shared_methods.py:71-166 n / Re / Ie by Nelder-Mead on the binned median
 * profile), float64, one CTA per stamp.  data (and mask, optional, 1 = masked) use the batch's
 * output-pixel packing; pixels must be square and unrotated (P = s I).  params[n][8] (value
 * space, device): slots with their bit set in known_mask are inputs, the others are written;
 * status[n] receives AP_INIT_* bits.  workspace (may be NULL when
 * ap_reference_init_workspace_bytes gives 0) holds per-CTA pixel buffers of large stamps. */
#define AP_INIT_CENTRE_EDGE 1  /* the centre-of-light box reached the image edge: window centre kept */
#define AP_INIT_FIT_LIMIT 2    /* Nelder-Mead stopped at its iteration limit: its start kept */
#define AP_INIT_NO_ISOPHOTE 4  /* no isophote had 3 samples (the reference raises): q = 0.9 */
#define AP_INIT_NO_PROFILE 8   /* no positive profile bin (the reference raises) */
int ap_reference_init_workspace_bytes(const ap_batch* batch, int64_t* bytes);
int ap_reference_init(ap_batch* batch, const float* data, const uint8_t* mask, int32_t known_mask,
                      double* params, int32_t* status, void* workspace, int64_t workspace_bytes,
                      ap_stream_t stream);

/* Segmentation maps (astrophot/utils/initialize/segmentation_map.py:33-293), device pointers,
 * seg[ny][nx] int32 ids >= 0, image[ny][nx] float32.
 * ap_segmap_range: min_max[2] = (smallest, largest id).
 * ap_segmap_present: present[id] = 1 for every id in the map (present: max_id + 1 bytes).
 * ap_segmap_stats: per segment k (index[id] = k, -1 for ids left out; n_seg segments): bbox[k] =
 *   (xmin, xmax, ymin, ymax) (windows_from_segmentation_map), centroid[k] = flux-weighted (x, y)
 *   (centroids_from_segmentation_map), pa[k] = angular centre of light + north
 *   (PA_from_segmentation_map), q[k] = axis_ratio_com at pa + north (q_from_segmentation_map);
 *   centroid_in / pa_in (may be NULL): caller's centroids / PAs used instead of computed ones (the
 *   reference functions' centroids= / PAs= arguments); acc: n_seg * 5 doubles of workspace.
 * ap_window_flux: flux[w] = sum of the image over windows[w] = (x0, x1, y0, y1), half-open, clipped
 *   to the image (filter_windows' flux). */
int ap_segmap_range(const int32_t* seg, int64_t npix, int32_t* min_max, ap_stream_t stream);
int ap_segmap_present(const int32_t* seg, int64_t npix, int32_t max_id, uint8_t* present, ap_stream_t stream);
int ap_segmap_stats(const int32_t* seg, const float* image, int32_t nx, int32_t ny, const int32_t* index,
                    int32_t n_seg, double north, const double* centroid_in, const double* pa_in, double* acc,
                    int32_t* bbox, double* centroid, double* pa, double* q, ap_stream_t stream);
int ap_window_flux(const float* image, int32_t nx, int32_t ny, const int32_t* windows, int32_t n, double* flux,
                   ap_stream_t stream);

/* Shifted, renormalised PSF of every stamp for value-space params (device):
 * out[n][(ky+2)*(kx+2)] packed with stride max_kp2 = (max ky + 2) * (max kx + 2)
 * (see ap_batch_psf_stride).  d_out (optional, may be NULL) receives d/d shift_x and
 * d/d shift_y kernels with the same layout, [n][2][stride]. */
int ap_batch_psf_stride(const ap_batch* batch, int64_t* stride);
int ap_psf_shift(ap_batch* batch, const double* params, const float* psf, float* out,
                 float* d_out, ap_stream_t stream);

/* chi2_out[n] = sum over unmasked pixels of weight * (data - model)^2 (float64 sums).
 * mask may be NULL (nonzero = ignored). */
int ap_chi2(ap_batch* batch, const float* data, const float* weight, const uint8_t* mask,
            const float* model, double* chi2_out, ap_stream_t stream);

/* Batched damped solve of LM._h: for m systems of size p,
 * h[i] = solve(H_i o (I + D / (1 + L_i)) + L_i I (1 + diag H_i), g_i)   (float64, device). */
int ap_damped_solve(int32_t m, int32_t p, const double* hess, const double* grad,
                    const double* L, double* h_out, ap_stream_t stream);

/* Full batched LM.  fixed_params[n][8] (device, value space) supplies the locked slots.
 * state[n][n_free] (device, representation space) is read as the initial state and overwritten with BaseOptimizer.res() of each stamp (the lowest-chi2
 * state).  chi2_out[n]: chi2/ndf of that state.  iters_out[n], status_out[n]: AP_LM_*.
 * lm_workspace: caller-owned device memory of ap_lm_workspace_bytes.  ndf per stamp is
 * (#unmasked pixels - n_free), at least 1.  Synchronises the stream between device
 * rounds (one 4-byte read per rounds_per_sync rounds). */
int ap_lm_workspace_bytes(const ap_batch* batch, const ap_lm_options* lm, int64_t* bytes);
int ap_lm_fit(ap_batch* batch, const float* data, const float* weight, const uint8_t* mask,
              const float* psf, const double* fixed_params, double* state,
              const ap_lm_options* lm, void* lm_workspace,
              int64_t lm_workspace_bytes, double* chi2_out, int32_t* iters_out,
              int32_t* status_out, ap_stream_t stream);
/* Histories of the last ap_lm_fit (device pointers into lm_workspace, layout
 * [n][max_iter + 1]; loss = chi2/ndf, lambda = damping L). */
int ap_lm_history(const ap_batch* batch, const double** loss, const double** lambda_,
                  const double** states, int32_t* hist_len);

/* Diagnostics of the last call: [0] integration queue length, [1] selection decisions made
 * in float64 (cumulative), [2] overflow flags, [3] LM rounds, [4] integration-level
 * decisions made in float64 (cumulative). */
int ap_batch_stats(const ap_batch* batch, int64_t* stats_out /* [5] */);

/* Per-kernel CUDA-event timing.  ap_batch_profile(b, 1) clears the totals and records an
 * event pair around every kernel this batch launches from then on (also inside the LM's
 * captured graphs).  ap_batch_kernel_times fills ms_out[8] / launches_out[8] in the order
 * setup, psf_shift, sample, select, integrate, conv, reduce, lm_update (synchronises the
 * device when pairs are pending). */
int ap_batch_profile(ap_batch* batch, int32_t enable);
int ap_batch_kernel_times(ap_batch* batch, double* ms_out, int64_t* launches_out);

/* Algorithmic work counted on the device since bind (or the last reset): out[0] FP32
 * FLOPs of the PSF convolutions (2 per kernel tap, per convolved plane, per output pixel),
 * out[1] profile samples of the adaptive integration, out[2] samples of the sampling pass,
 * out[3] / out[4] the integration samples (of out[1]) of difference / Jacobian evaluations.
 * Synchronises the stream. */
int ap_batch_work_counters(ap_batch* batch, uint64_t* out /* [6] */, int32_t reset,
                           ap_stream_t stream);

/* FP32 FMA throughput probe: blocks x 256 threads, each running 8 independent chains of
 * 16 * iters FMAs (2 FLOP each).  scratch: >= blocks * 256 floats of device memory (never
 * written in practice).  Used to measure the FP32 pipe peak for roofline fractions. */
int ap_fma_probe(float* scratch, int32_t iters, int32_t blocks, ap_stream_t stream);

/* Sample-evaluation probe: blocks x 256 threads, each evaluating 4 * iters Sersic samples with the
 * integration's own device functions, register-resident (kind 0: value, 1: value and its six
 * partials, 2: value and its difference to a base evaluation).  scratch: >= blocks * 256 floats
 * (never written in practice).  The compute roofline of the integration kernels. */
int ap_sample_probe(int32_t kind, float* scratch, int32_t iters, int32_t blocks, ap_stream_t stream);

/* Render of one stamp for callers that cannot allocate device memory (a host that owns
 * the whole device memory pool, a plugin without access to its allocator, a pipeline that
 * must not stall on an allocation).  No counterpart in the reference: it is the
 * ap_render of a single stamp with its scratch in a fixed 8 MiB array inside this library
 * instead of a caller workspace.  geometry / options are host pointers (8 doubles as in
 * ap_batch_create); params[8] (value space), psf[psf_ky * psf_kx] (NULL without a PSF) and
 * model[ny * nx] are device pointers.  Working windows that need more than
 * AP_NOALLOC_SCRATCH_BYTES of scratch (about 80,000 pixels, e.g. 256 x 256 with a 21 x 21
 * PSF) are rejected with AP_ERR_WORKSPACE, and sides beyond 65,536 (PSF sides beyond 4,095) with
 * AP_ERR_ARG.  The plan reaches the device as kernel arguments, so a call only enqueues work.
 * Sersic and exponential profiles, sampling modes midpoint / simpsons / quad / trapezoid; the
 * convolution is always direct (options.fft_min_kernel is not used).  The first call on each
 * device resolves the array's address; make it before any stream capture.  All calls on a
 * device share the array, so calls that overlap on the GPU race.  Calls no cudaMalloc /
 * cudaFree. */
#define AP_NOALLOC_SCRATCH_BYTES ((size_t)8 << 20)
int ap_render_noalloc(int32_t nx, int32_t ny, int32_t psf_kx, int32_t psf_ky,
                      const double* geometry, const ap_options* options, const double* params,
                      const float* psf, float* model, ap_stream_t stream);

/* ---- scenes: many sources on one image, fitted jointly ----------------------------------------
 * Group_Model.sample / jacobian (astrophot/models/group_model_object.py:183-283) over the joint
 * parameter vector of LM (astrophot/fit/lm.py) when the sources share an image.  The sources are
 * rendered by ap_batch stamps (ap_render for the model on the group's window, ap_jacobian on each
 * source's own window, as the reference does); these entry points combine them.  One
 * ap_scene_source per source (device array): */
typedef struct ap_scene_source {
  int64_t fwd_off;    /* element offset of the source's model render in the forward buffer; image
                         pixel (x, y) is at fwd_off + (y - fwd_y0) * fwd_nx + (x - fwd_x0) */
  int64_t jac_off;    /* element offset of its own-window Jacobian (compact slot 0) */
  int64_t jac_stride; /* elements between its compact slots (the batch's output pixels) */
  int32_t x0, y0;     /* own window: first pixel in the image */
  int32_t wx, wy;     /* own window size */
  int32_t n_free;     /* compact (fitted) slots of the source, <= 8 */
  int32_t gidx[8];    /* joint-vector index of each compact slot (linked slots share one) */
  int32_t fwd_x0, fwd_y0, fwd_nx; /* grid of the model render (group window or own window) */
} ap_scene_source;

/* image = sky + sum of the sources' renders inside their own windows.  tile_ptr / tile_src: for
 * every 32 x 32 image tile (row-major, ceil(nx/32) per row) the sources whose windows touch it
 * (CSR; the order fixes the summation order).  sky: a locked flat sky (counts per pixel), used
 * when sky_F is NULL; sky_F: device pointer to a free flat sky's log10 brightness F (float64),
 * the sky then being area * 10^F per pixel (the reference's FlatSky, astrophot/models/flatsky_model.py:55),
 * computed in float64 from the staged F at every launch.  With sky_F0 (device, float64) too,
 * the renders in fwd are differences (AP_RENDER_DIFFERENCE) and the sky term is the sky's own
 * difference area * 10^F0 * (10^(F - F0) - 1), formed without cancellation. */
int ap_scene_forward(const ap_scene_source* sources, const int32_t* tile_ptr, const int32_t* tile_src,
                     const float* fwd, float sky, const double* sky_F, const double* sky_F0, double area,
                     int32_t nx, int32_t ny, float* image, ap_stream_t stream);
/* out[ny][nx] = J h (h[P] float64), own windows, same tile lists. */
int ap_scene_jvp(const ap_scene_source* sources, const int32_t* tile_ptr, const int32_t* tile_src,
                 const float* jac, const double* h, int32_t nx, int32_t ny, float* out, ap_stream_t stream);
/* out[P] = J^T v for an image v[ny][nx]. */
int ap_scene_jt(const ap_scene_source* sources, int32_t n_sources, const float* jac, const float* v,
                int32_t nx, int32_t P, double* out, ap_stream_t stream);
/* H[P][P] = J^T W J; pairs[n_pairs][2] = every (a, b), a <= b, whose windows overlap (a = b
 * included).  weight / mask (1 = ignored) may be NULL. */
int ap_scene_hess(const ap_scene_source* sources, const int32_t* pairs, int32_t n_pairs,
                  const float* jac, const float* weight, const uint8_t* mask, int32_t nx, int32_t P,
                  double* H, ap_stream_t stream);
/* The same two products with a result that does not depend on the order in which blocks run
 * (linked centres make several blocks add into one entry): ap_scene_hess_blocks writes each
 * pair's 8 x 8 block, part[p][a][c] = sum J_a W J_c (n_pairs x 64 doubles), ap_scene_jt_blocks
 * each source's sums, part[s][c] (n_sources x 8 doubles); ap_gather_sum then zeroes out[out_n]
 * and sets out[entry[e]] = sum of part[contrib[k]] for k in [ptr[e], ptr[e + 1]) in that order
 * (e < n_entries; the tables are the caller's, from the pairs and the sources' gidx). */
int ap_scene_hess_blocks(const ap_scene_source* sources, const int32_t* pairs, int32_t n_pairs,
                         const float* jac, const float* weight, const uint8_t* mask, int32_t nx, double* part,
                         ap_stream_t stream);
int ap_scene_jt_blocks(const ap_scene_source* sources, int32_t n_sources, const float* jac, const float* v,
                       int32_t nx, double* part, ap_stream_t stream);
int ap_gather_sum(int64_t n_entries, const int64_t* entry, const int32_t* ptr, const int32_t* contrib,
                  const double* part, double* out, int64_t out_n, ap_stream_t stream);
/* out[0] = sum over unmasked pixels of W (data - model)^2 (float64).  parts: device scratch of
 * n_parts doubles (1024 used at most) for the block partial sums, which are added in a fixed
 * order, so the result has the same bits on every run. */
int ap_scene_chi2(const float* model, const float* data, const float* weight, const uint8_t* mask,
                  int64_t n, double* out, double* parts, int32_t n_parts, ap_stream_t stream);
/* out[0] = sum over unmasked pixels of W dm (dm - 2 (data - base)): the change of chi^2 from
 * the model `base` to base + dm, for a difference image dm (float64 per pixel; the same
 * fixed-order partial sums as ap_scene_chi2, parts likewise). */
int ap_scene_chi2_change(const float* dm, const float* base, const float* data, const float* weight,
                         const uint8_t* mask, int64_t n, double* out, double* parts, int32_t n_parts,
                         ap_stream_t stream);
/* A PSF image finer than the image pixels (psf_upscale u = image pixel / PSF pixel): sources are
 * rendered on u-times finer windows and summed back in u x u blocks (Image.reduce of the cropped
 * working image, astrophot/models/model_object.py:308-350).  out[p][i] for every plane p <
 * n_planes and coarse pixel i < out_total: stamp k's coarse image, cnx[k] pixels wide, starts at
 * out_off[k] (ascending, out_off[0] = 0), its fine image (u cnx[k] wide, row-major) at in_off[k];
 * planes lie in_stride / out_stride floats apart.  All arrays device. */
int ap_reduce_upscaled(int32_t n_stamps, const int64_t* in_off, const int64_t* out_off, const int32_t* cnx,
                       int32_t u, int32_t n_planes, const float* in, int64_t in_stride, float* out,
                       int64_t out_stride, int64_t out_total, ap_stream_t stream);
/* r = W (data - model) on unmasked pixels, 0 on masked ones (LM._r, fit/lm.py:381-385). */
int ap_scene_residual(const float* model, const float* data, const float* weight,
                      const uint8_t* mask, int64_t n, float* r, ap_stream_t stream);
/* out = (2/d)((rh - r)/d - W jh): the image whose J^T is the geodesic-acceleration right-hand
 * side of LM.step (fit/lm.py:286-291). */
int ap_scene_rpp_image(const float* r, const float* rh, const float* jh, const float* weight,
                       const uint8_t* mask, double d, int64_t n, float* out, ap_stream_t stream);
/* The parameter rows of a scene's renders (float64 [rows][8], slots cx cy q PA n Re Ie F) at the
 * joint representation vector x + alpha v, computed on the device so that an LM keeps its
 * vectors there (the parameter setters of Parameter_Node through the maps of
 * utils/conversions/optimization.py:6-54, which LM.step applies at every trial,
 * fit/lm.py:277-293): out[c] = base[c] where gidx[c] < 0 (a locked or absent slot), else the
 * value of slot c % 8 at representation x[g] + alpha v[g], g = gidx[c].  n_cells a multiple of
 * 8; v may be NULL (alpha then unused). */
int ap_scene_stage(int32_t n_cells, const int32_t* gidx, const double* base, const double* x,
                   const double* v, double alpha, double* out, ap_stream_t stream);
/* h = solve(H o (I + D/(1+L)) + L I (1 + diag H), g) for one dense n x n system (LM._h,
 * fit/lm.py:361-371): blocked FP64 Cholesky.  info (device) = 0, or 1 + the row whose pivot
 * was not positive (the system is then not solved). */
size_t ap_dense_solve_workspace_bytes(int32_t n);
int ap_dense_damped_solve(int32_t n, const double* H, const double* g, double L, double* h,
                          void* ws, size_t ws_bytes, int32_t* info, ap_stream_t stream);
/* h = the same damped system solved for another right-hand side g: the two triangular solves
 * on the Cholesky factor the last ap_dense_damped_solve left in ws (it must have reported
 * info = 0).  LM.step solves its damped system twice per trial, for the step and for the
 * geodesic term (fit/lm.py:286-299). */
int ap_dense_factored_solve(int32_t n, const double* g, double* h, void* ws, size_t ws_bytes,
                            ap_stream_t stream);
/* The same damped system (LM._h, fit/lm.py:361-371) solved in mixed precision: float32 blocked
 * Cholesky, then float64 iterative refinement against the float64 damped matrix (off-diagonal
 * H_ij * fl(1/(1+L)), diagonal H_ii + L (1 + H_ii), as the reference forms it) until the residual
 * meets LAPACK dsposv's backward-error test (at most 10 rounds).  H must hold both triangles.
 * info (device) = 0: h solved to float64 accuracy; -1: not solved (the float32 factorisation met
 * a non-positive pivot, or the refinement stalled), h = 0 -- call ap_dense_damped_solve.  n at
 * most 8192 (AP_ERR_UNSUPPORTED beyond).  Everything stays on the stream; no host read. */
int ap_dense_damped_solve_mixed(int32_t n, const double* H, const double* g, double L, double* h,
                                void* ws, size_t ws_bytes, int32_t* info, ap_stream_t stream);
/* Another right-hand side of the system the last ap_dense_damped_solve_mixed factored (same H,
 * same L): refinement on its float32 factor; info as above (-1 also when that factorisation
 * failed). */
int ap_dense_factored_solve_mixed(int32_t n, const double* H, const double* g, double L, double* h,
                                  void* ws, size_t ws_bytes, int32_t* info, ap_stream_t stream);

/* ---- learned initial guess -----------------------------------------------------------------
 * No counterpart in the reference: its initial values come from the heuristics of
 * Galaxy_Model.initialize / parametric_initialize (astrophot/models/galaxy_model_object.py:60-113,
 * astrophot/models/_shared_methods.py:116-166).  A 6-layer CNN (4 stride-2 3x3 convolutions
 * 1->32->64->128->256 channels, fc 4096->192, fc 192->8; 1,176,008 parameters) proposes the
 * 7 Sersic parameters of a 64 x 64 stamp; its forward and backward passes are GEMMs on the
 * tensor cores in bf16 with fp32 accumulation.  Parameters are one flat fp32 vector of
 * ap_cnn_param_count() floats (per layer W[N][K] then b[N], see ap_cnn_layer_offsets) plus its
 * bf16 mirror (ap_cnn_to_bf16).  Batches must be multiples of 16 stamps.  All pointers are
 * device pointers except those of ap_cnn_layer_offsets. */
int64_t ap_cnn_param_count(void);
/* In-project autotuner of the CNN GEMM tiles: with enable != 0 the first GEMM of each
 * (layout, shape) times the 128x128 / 128x64 / 128x32 tiles and keeps the fastest; enable < 0
 * also forgets the choices made so far.  tuned_shapes (may be NULL) = shapes tuned so far. */
int ap_cnn_autotune(int32_t enable, int32_t* tuned_shapes);
size_t ap_cnn_workspace_bytes(int64_t batch);
/* Byte offsets in a workspace of `batch` stamps (host outputs): act_offsets[6] of the bf16
 * activations each layer keeps for the backward pass ([rows][N], rows = batch * hout^2; layer 6
 * keeps none) and out_offset of the fp32 outputs [batch][16]. */
int ap_cnn_workspace_offsets(int64_t batch, int64_t* act_offsets, int64_t* out_offset);
/* w_offsets[6], b_offsets[6], dims[6][6] = {cin, cout, hin, hout, K, N} per layer (host). */
int ap_cnn_layer_offsets(int64_t* w_offsets, int64_t* b_offsets, int32_t* dims);
int ap_cnn_to_bf16(const float* params, void* params_bf16, ap_stream_t stream);
/* x[batch][64][64] (normalised stamps, ap_cnn_prepare) -> out[batch][16] (standardised
 * outputs in columns 0..7).  The workspace keeps the activations for ap_cnn_backward. */
int ap_cnn_forward(const float* params, const void* params_bf16, const float* x, int64_t batch,
                   float* out, void* ws, size_t ws_bytes, ap_stream_t stream);
/* The same outputs as ap_cnn_forward for inference only: on the tcgen05 path the convolutions
 * read the activations directly and no im2col matrix is built, so ap_cnn_backward may not follow. */
int ap_cnn_infer(const float* params, const void* params_bf16, const float* x, int64_t batch,
                 float* out, void* ws, size_t ws_bytes, ap_stream_t stream);
/* grads (flat fp32) of a loss with d loss / d out = dout[batch][16], after ap_cnn_forward on the
 * same workspace. */
int ap_cnn_backward(const void* params_bf16, const float* dout, int64_t batch, float* grads,
                    void* ws, size_t ws_bytes, ap_stream_t stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8, decoupled weight decay) on the mean squared error
 * between out[:, 0..7] and targets[batch][8]; loss_out (device, may be NULL) receives the loss. */
int ap_cnn_train_step(float* params, void* params_bf16, float* grads, float* adam_m, float* adam_v,
                      const float* x, const float* targets, int64_t batch, float lr, int32_t step,
                      float weight_decay, double* loss_out, void* ws, size_t ws_bytes,
                      ap_stream_t stream);
/* data[batch][64][64] -> x = asinh((data - sky) / (4 sigma)) (pixel signal-to-noise,
 * compressed), lscale = log10(sigma); sky[batch], sigma[batch] per stamp. */
int ap_cnn_prepare(const float* data, const float* sky, const float* sigma, int64_t batch, float* x,
                   float* lscale, ap_stream_t stream);
/* out[batch][16] -> params[batch][8] (value space, F = sky_F) through the output statistics
 * mean[8], stdv[8]: outputs are cx - 32, cy - 32, q, cos 2PA, sin 2PA, ln n, ln Re,
 * log10 Ie - log10 sigma. */
int ap_cnn_decode(const float* out, const float* lscale, const float* mean, const float* stdv,
                  const double* sky_F, int64_t batch, double* params, ap_stream_t stream);
/* Moments initial guess of 64 x 64 stamps (the learned proposal's fallback): centre of light,
 * PA and q from second moments of pixels more than sigma above the sky, Re holding half the
 * light, n = 2, Ie at Re. */
int ap_moments_init(const float* data, const float* sky, const float* sigma, const double* sky_F,
                    int64_t batch, double* params, ap_stream_t stream);
/* out = proposal where chi2_proposal <= chi2_fallback, else fallback; which = 0 / 1. */
int ap_select_init(const double* proposal, const double* fallback, const double* chi2_proposal,
                   const double* chi2_fallback, int64_t batch, double* out, int32_t* which,
                   ap_stream_t stream);
/* C[R][S] = sum_t A(r, t) B(s, t) on the tensor cores (bf16 in, fp32 out); A(r, t) = A[r*lda+t]
 * or, with a_trans, A[t*lda+r]; likewise B.  R, S, lda, ldb multiples of 8, T of 16. */
int ap_gemm_bf16(const void* A, int32_t lda, int32_t a_trans, const void* B, int32_t ldb,
                 int32_t b_trans, float* C, int32_t ldc, int32_t R, int32_t S, int32_t T,
                 ap_stream_t stream);

/* Which tensor-core path the CNN forward and training step run: AP_CNN_TCGEN05 (default:
 * tcgen05.mma with the accumulator in tensor memory, operands staged by TMA; the inference
 * forward reads the convolution inputs straight from the NHWC activations, no im2col matrix) or
 * AP_CNN_MMA_SYNC (ldmatrix + mma.sync tiles over explicit im2col matrices).  The backward GEMMs
 * (reduction-strided operands) run on the mma.sync tiles in both modes. */
#define AP_CNN_MMA_SYNC 0
#define AP_CNN_TCGEN05 1
int ap_cnn_set_path(int32_t path);
int ap_cnn_get_path(int32_t* path);
/* C[R][S] = sum_t A[r*lda+t] W[s*ldw+t] (+ bias[s], ReLU, bf16 store into act when act is set;
 * else fp32 into C, row stride ldc) through the tcgen05 kernel.  S and T multiples of 16, lda and
 * ldw of 8, pointers 16-byte aligned. */
int ap_gemm_bf16_tc(const void* A, int32_t lda, const void* W, int32_t ldw, float* C, int32_t ldc,
                    int32_t R, int32_t S, int32_t T, const float* bias, void* act, int32_t relu,
                    ap_stream_t stream);
/* 3x3 stride-2 pad-1 convolution of x[batch][H][H][cin] (NHWC bf16; cin 16, 32 or a multiple of
 * 64) with W[S][9*cin] (k = (ky*3 + kx)*cin + c) through the tcgen05 kernel, each A tile one
 * strided 4-D TMA load: out row (b*H/2 + oy)*H/2 + ox, epilogue as ap_gemm_bf16_tc. */
int ap_conv3x3s2_bf16_tc(const void* x, int64_t batch, int32_t H, int32_t cin, const void* W,
                         int32_t S, float* C, int32_t ldc, const float* bias, void* act,
                         int32_t relu, ap_stream_t stream);
/* First error code a tcgen05 kernel recorded (0 none; 1-5: an mbarrier wait that ran out of its
 * 200 ms limit, after which the kernel stopped, freed its tensor memory and returned, and every
 * later launch returns at once).  clear != 0 resets it.  Synchronises the device. */
int ap_tc_status(int32_t clear, uint32_t* code);

/* Library version string. */
const char* ap_version(void);
/* Text of the last CUDA error behind an AP_ERR_CUDA status on this thread ("" if none). */
const char* ap_last_cuda_error(void);

#ifdef __cplusplus
}
#endif

#endif /* ASTROPHOT_GB300_H */
