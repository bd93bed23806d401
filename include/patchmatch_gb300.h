/*
 * patchmatch_gb300.h -- C ABI of the GB300-native PatchMatch multi-view-stereo engine.
 *
 * This is the drop-in boundary for the hot path of yhsa678/patchMatch_cuda: one depth
 * map (and the sampled view-selection map) for one reference image from N calibrated
 * source views, by row-sweep PatchMatch propagation with homography-warped windowed NCC
 * and HMM view selection. Plain pointers and sizes only; every entry point returns a
 * pm_status and never exits the process. Handles hold no process-global state, so
 * several handles may run concurrently (each owns a CUDA stream). A single handle is not
 * thread-safe.
 *
 * Reference interface each entry point replaces (paths relative to the reference root):
 *   pm_create             PatchMatch::PatchMatch        src/patchMatch.h:71-72, src/patchMatch.cu:132-206
 *   pm_run                PatchMatch::runPatchMatch     src/patchMatch.h:74,    src/patchMatch.cu:263-407
 *   pm_get_depth          Array2D_wrapper::copyData     src/array2d_wrapper.h:37-47 (on _depthMap)
 *   pm_get_view_selection _usedImgsID (never read back by the reference)  src/patchMatch.cu:170, :381-385
 *   pm_save_depth         Array2D_wrapper::saveToFile   src/array2d_wrapper.h:51-70
 *   pm_destroy            PatchMatch::~PatchMatch       src/patchMatch.cu:208-234
 *   pm_run_batch          (no counterpart: several references in one launch per sweep)
 * Lower-level entry points expose single stages for parity checks and for callers that
 * drive their own schedule; each names its reference counterpart below.
 */
#ifndef PATCHMATCH_GB300_H
#define PATCHMATCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pm_status {
    PM_OK = 0,
    PM_ERR_INVALID_ARGUMENT = 1,
    PM_ERR_WINDOW_SIZE = 2,      /* half window outside [1, 22] (patchMatch.cu:265-270,
                                    array2d_refImg.cu:71-97)                            */
    PM_ERR_TOO_FEW_VIEWS = 3,    /* fewer than 2 images (patchMatch.cu:137-142)          */
    PM_ERR_TOO_MANY_VIEWS = 4,   /* more than PM_MAX_SOURCE_VIEWS source views            */
    PM_ERR_IMAGE = 5,            /* missing, empty or oversized image                     */
    PM_ERR_CAMERA = 6,           /* singular or non-finite K / R / t                      */
    PM_ERR_CUDA = 7,             /* a CUDA runtime call failed                            */
    PM_ERR_OUT_OF_MEMORY = 8,
    PM_ERR_IO = 9,
    PM_ERR_NO_DEVICE = 10,
    PM_ERR_STATE = 11,           /* call out of order (e.g. view selection before a run)  */
    PM_ERR_UNSUPPORTED = 12,
    PM_ERR_SCRATCH_LIMIT = 13    /* image too wide for pm_box_moments_noalloc's fixed scratch */
} pm_status;

#define PM_MAX_SOURCE_VIEWS 32
#define PM_MAX_HALF_WINDOW 22

typedef enum pm_prefilter_mode {
    PM_PREFILTER_NONE = 0,      /* what the reference runtime does (GaussianBlurCUDA is never called) */
    PM_PREFILTER_BOX = 1,       /* GaussianBlurCUDA as written: box of width max(5, odd(5 sigma))     */
    PM_PREFILTER_GAUSSIAN = 2   /* the normalised Gaussian weights that class computes first          */
} pm_prefilter_mode;

typedef enum pm_precision {
    PM_PRECISION_FP32 = 0,      /* FP32 texels (u8 texels when unfiltered: the same values)  */
    PM_PRECISION_MIXED = 1      /* FP16 texels, shifted window moments, FP64 window origin    */
} pm_precision;

typedef enum pm_sampler {
    PM_SAMPLER_EXACT = 0,       /* 4-texel gather, exact FP32 bilinear weights (NCC within
                                   1e-4 of an FP64 oracle; slower)                          */
    PM_SAMPLER_HARDWARE = 1     /* default: texture-unit bilinear filtering with 8-bit
                                   fixed-point weights, what the reference's tex2DLayered
                                   fetch does; FP16 texels fall back to the exact sampler   */
} pm_sampler;

typedef enum pm_texel_format {
    PM_TEXELS_AUTO = 0,         /* chosen from precision and prefilter                        */
    PM_TEXELS_U8 = 1,           /* unfiltered images only                                     */
    PM_TEXELS_F16 = 2,
    PM_TEXELS_F32 = 4
} pm_texel_format;

typedef enum pm_init_mode {
    PM_INIT_RANDOM = 0,         /* uniform depth in [near, far) (array2d_wrapper.cu:3-20)      */
    PM_INIT_PROPOSAL = 1        /* the learned proposal (pm_set_proposal); pixels whose
                                   confidence is below proposal_threshold keep the uniform
                                   random depth. No counterpart in the reference.           */
} pm_init_mode;

typedef enum pm_direction {     /* sweep order within one iteration (patchMatch.cu:344-391) */
    PM_DIR_LEFT_TO_RIGHT = 0,
    PM_DIR_TOP_TO_BOTTOM = 1,
    PM_DIR_RIGHT_TO_LEFT = 2,
    PM_DIR_BOTTOM_TO_TOP = 3
} pm_direction;

/* One calibrated grayscale view (Image::updateCamParam, image.cpp:39-61): projection
 * K [R | t], pixel ~ K (R X + t). The engine copies the pixels at pm_create. */
typedef struct pm_view {
    const uint8_t *gray;        /* height rows of width bytes                                */
    int width, height;
    int stride;                 /* bytes between rows (>= width)                             */
    float K[9], R[9], t[3];     /* row-major                                                 */
} pm_view;

/* The PatchMatch constructor's parameters (patchMatch.h:71-72) and main.cpp's INI keys
 * (main.cpp:47-85), plus the engine's own knobs. pm_default_params fills the defaults. */
typedef struct pm_params {
    float depth_near, depth_far;   /* depthRangeNear / depthRangeFar                         */
    int half_window;               /* halfWindowSize, 1..22                                  */
    int num_samples;               /* numOfSamples (views sampled per pixel, >= 1)           */
    float sp_alpha;                /* SPMAlpha                                               */
    float gaussian_sigma;          /* gaussianSigma (prefilter width)                        */
    int prefilter;                 /* pm_prefilter_mode                                      */
    int num_iterations;            /* numOfIterations                                        */
    float orientation_x;           /* orientationX (plane normal x; default 0)               */
    float orientation_z;           /* orientationZ (plane normal z; default 1)               */
    uint64_t seed;                 /* Philox key                                             */
    int precision;                 /* pm_precision                                           */
    int init_mode;                 /* pm_init_mode                                           */
    int threads_per_line;          /* 0 = tuned; else a multiple of 32 up to 192, for both
                                      launches of every sweep                                */
    int quirks;                    /* 1 (default): keep the reference's leading-edge window
                                      misalignment (patchMatch.cu:546); 0: aligned windows   */
    int gpu_id;                    /* gpuId: -1 = current device (main.cpp:56-59)            */
    int block_dim_x, block_dim_y;  /* accepted for signature parity, unused                  */
    int sampler;                   /* pm_sampler                                             */
    int texel_format;              /* pm_texel_format                                        */
    int num_sweeps;                /* 0: all num_iterations x 4 sweeps; else the schedule
                                      stops after this many sweeps                          */
    float proposal_threshold;      /* PM_INIT_PROPOSAL: minimum confidence (default 0.5)     */
    float perturbation;            /* 0 (default): the random hypothesis is uniform in
                                      [near, far] (patchMatch.cu:937). > 0: no counterpart in
                                      the reference; half of the pixels (by a second Philox
                                      word) instead draw within +-perturbation x 2^(-k/4)
                                      (relative) of their current depth in sweep k, a local
                                      search that refines a learned initialisation         */
    int refine_trials;             /* 0 (default): no refinement, as the reference runs
                                      (patchMatch.cu:396). > 0: after the last sweep, that
                                      many hypotheses depth + refine_sigma z (z ~ N(0, 1) by
                                      Irwin-Hall) scored on the last sweep's sampled views;
                                      the reference's never-launched depthRefinement
                                      (patchMatch.cu:717-773) with 10 trials, sigma 0.05      */
    float refine_sigma;            /* depth units (default 0.05)                              */
    int planes;                    /* 0 (default): one plane normal for every pixel, the
                                      reference's orientationX/Z (patchMatch.cu:32,
                                      main.cpp:65-76). 1: no counterpart in the reference; a
                                      slanted plane per pixel, depth plus slopes (a, b) with
                                      normal ~ (a, b, 1) in the reference camera: random
                                      initial slopes, the previous step's plane carried to
                                      each pixel, and a random hypothesis that is a uniform
                                      depth, uniform slopes or a local perturbation of both.
                                      orientation_x/z are then unused                        */
    float plane_depth_step;        /* planes: relative half-width of the depth perturbation
                                      in sweep k, x 2^(-k/4) (default 0.02)                  */
    float plane_slope_step;        /* planes: half-width of the slope perturbation, x 2^(-k/4)
                                      (default 0.25)                                         */
} pm_params;

#define PM_MAX_REFINE_TRIALS 256

typedef struct pm_handle pm_handle;

typedef struct pm_stats {
    unsigned long long cost_evals;       /* NCC evaluations the algorithm performed       */
    unsigned long long cost_evals_done;  /* evaluations actually computed (cache hits are
                                            reused results)                               */
    float ms_prepare;                    /* pm_create device work                         */
    float ms_init;                       /* last run: depth init + initial costs          */
    float ms_sweeps;                     /* last run: all sweeps                          */
    float ms_total;                      /* last run                                      */
    int threads_per_line;                /* chosen by the tuner or the caller             */
    int texel_bytes;                     /* 1 (u8), 2 (fp16) or 4 (fp32)                  */
    int warps_per_line[4];               /* vertical sweeps: interior lines, lines within a
                                            half-window of an edge; horizontal: the same  */
} pm_stats;

void pm_default_params(pm_params *p);
const char *pm_status_string(pm_status s);
/* The sizes of the public structs as this library was built, in the order pm_view, pm_params,
 * pm_stats, pm_fuse_params, pm_depth_view: the first n of them into out. Lets a binding check
 * its mirrors of the structs before it passes one. Returns how many it wrote. */
int pm_struct_sizes(size_t *out, int n);
const char *pm_last_error(const pm_handle *h);

/* Validates, sets up cameras (K^-1, C, H1, H2 in FP64), uploads and prefilters the images,
 * builds source textures and the reference-window moments. ref_id indexes views. */
pm_status pm_create(const pm_view *views, int n_views, int ref_id, const pm_params *p,
                    pm_handle **out);
pm_status pm_destroy(pm_handle *h);

/* Initial depth + every view's cost, then num_iterations x 4 sweeps. Synchronous. */
pm_status pm_run(pm_handle *h);
/* Same work enqueued on the handle's stream (captured once as a CUDA graph). */
pm_status pm_run_async(pm_handle *h);
pm_status pm_synchronize(pm_handle *h);
/* Runs several handles with one launch per sweep for all of them (handles grouped by
 * window size); synchronous. */
pm_status pm_run_batch(pm_handle *const *hs, int n);

/* A reusable batch (no counterpart in the reference): pm_batch_create groups the handles by
 * window side and sampler, times 1 .. 6 warps per line on one sweep of each group and
 * orientation (the autotuner), and captures the whole schedule -- every reference's
 * initialisation and initial costs, then one launch per sweep over the lines of all references
 * of a group -- as one CUDA graph on the first handle's stream. pm_batch_run launches the graph
 * and waits; results and stats are read per handle. The handles must outlive the batch and
 * their parameters stay as they were at creation. pm_batch_info reports the kernel launches
 * per run, the number of groups and the tuned warps per line (vertical, horizontal) per group. */
typedef struct pm_batch pm_batch;
pm_status pm_batch_create(pm_handle *const *hs, int n, pm_batch **out);
pm_status pm_batch_run(pm_batch *b);
pm_status pm_batch_info(const pm_batch *b, int *launches, int *groups, int *wpl, int max_groups);
pm_status pm_batch_destroy(pm_batch *b);

/* Results. dst_pitch in bytes (0 = width * sizeof(float)). */
pm_status pm_get_depth(pm_handle *h, float *dst, size_t dst_pitch);
/* num_samples layers of height*width bytes: layer j, row y, column x holds the view
 * sampled for sample j at (x, y) in the final bottom-to-top sweep (255: none). */
pm_status pm_get_view_selection(pm_handle *h, uint8_t *dst);
/* "<W>&<H>&1&" then raw float32 row-major depth (array2d_wrapper.h:51-70). */
pm_status pm_save_depth(pm_handle *h, const char *path);

pm_status pm_get_stats(const pm_handle *h, pm_stats *out);
/* The handle's cudaStream_t, for callers that time or order work around it. */
pm_status pm_get_stream(const pm_handle *h, void **stream);
pm_status pm_get_size(const pm_handle *h, int *width, int *height, int *n_src);

/* ---- single stages (parity checks, custom schedules) ---------------------------------- */
/* generate_kernel_float (array2d_wrapper.cu:3-20) into the depth map. */
pm_status pm_init_depth(pm_handle *h);
/* computeAllCostGivenDepth (patchMatch.cu:775-816): all costs at the current depth;
 * axis 1 pairs windows like the reference's transposed layout, axis 0 like vertical sweeps. */
pm_status pm_compute_costs(pm_handle *h, int axis);
/* One sweep, topToDown / downToTop (patchMatch.cu:818-1209). sweep_id keys the random
 * draws; record_views writes the view-selection map. */
/* Depth refinement (the step after the last sweep, see refine_trials): `trials` hypotheses
 * around each pixel's depth on the views of rows 0 .. num_samples-1 of the view-selection map
 * (0: all of pm_params.num_samples), window axis 0 (vertical sweeps) or 1 (horizontal),
 * Philox draws keyed by sweep_id. Costs are left as they were. */
pm_status pm_refine(pm_handle *h, int trials, float sigma, uint32_t sweep_id, int num_samples, int axis);
pm_status pm_run_sweep(pm_handle *h, int direction, uint32_t sweep_id, int num_samples,
                       int record_views);
pm_status pm_set_depth(pm_handle *h, const float *src);
/* Costs are pixel-major: (y * width + x) * n_src + view. */
pm_status pm_get_costs(pm_handle *h, float *dst);
pm_status pm_set_costs(pm_handle *h, const float *src);
/* Reference-window box sums (array2d_refImg.cu:11-67) and the reference texels. */
pm_status pm_get_ref_maps(pm_handle *h, float *ref, float *sum_i, float *sum_ii);
/* Source texels as stored for sampling (after prefilter and precision rounding). */
pm_status pm_get_source_texels(pm_handle *h, int view, float *dst);
/* computeNCC (patchMatch.cu:433-611) for n (x, y, view, depth, axis) tuples. */
pm_status pm_eval_costs(pm_handle *h, int n, const int *xs, const int *ys, const int *views,
                        const float *depths, const int *axes, float *out);
/* Slanted-plane mode (pm_params.planes = 1; no counterpart in the reference, whose one plane
 * normal is a constant, patchMatch.cu:32): the per-pixel plane slopes (a, b) as height*width*2
 * floats, row-major, and the unit normals (a, b, 1)/|(a, b, 1)| in the reference camera as
 * height*width*3 floats. PM_ERR_STATE when the handle was created without planes. */
pm_status pm_get_slopes(pm_handle *h, float *dst);
pm_status pm_set_slopes(pm_handle *h, const float *src);
pm_status pm_get_normals(pm_handle *h, float *dst);
/* computeNCC for n (x, y, view, depth, slopes, axis) tuples of a slanted-plane handle:
 * slopes holds (a, b) per query. */
pm_status pm_eval_costs_planes(pm_handle *h, int n, const int *xs, const int *ys, const int *views,
                               const float *depths, const float *slopes, const int *axes, float *out);
/* Bilinear source fetch of patchMatch.cu:543 at source coordinates (xs, ys). */
pm_status pm_sample_source(pm_handle *h, int view, int n, const float *xs, const float *ys,
                           float *out);

/* ---- direction flip ---------------------------------------------------------------------
 * cudaTranspose::transpose2dData (cudaTranspose.h:9-71) over `layers` stacked layers of
 * DEVICE memory: layer l of the input is rows [l*height, (l+1)*height) of a width-wide
 * pitched float image; the output layer is height wide and width tall. The engine's sweeps
 * address both directions in place and never need it; it serves callers that hold maps in
 * the reference's stacked layout. stream may be NULL. */
pm_status pm_transpose_layers(const float *d_in, size_t in_pitch, float *d_out,
                              size_t out_pitch, int width, int height, int layers,
                              void *stream);

/* ---- reference-window moments without any device allocation -----------------------------
 * No counterpart in the reference: an addition for callers that cannot allocate device
 * memory (work recorded inside a stream capture that must not gain allocation nodes, hosts
 * whose framework owns every allocation, plugins that may only use the buffers they are
 * given). For every pixel of a width x height float image in DEVICE memory (row pitch
 * ref_pitch bytes): the window sums S_I = sum I and S_II = sum I^2 over the
 * (2 half_window + 1)^2 window centred on the pixel, pixels outside the image counting as
 * zero, and c1 = S_II - S_I^2 / n with n the number of the window's pixels inside the image,
 * set to 0 where it is below 1e-5. Sums are formed in double and stored as float, row-major
 * with row pitch out_pitch bytes; any output pointer may be NULL. Both pitches must be
 * multiples of 4 bytes and at least width * 4. Intermediate row sums live in a fixed scratch
 * array inside the library (PM_NOALLOC_SCRATCH_DOUBLES doubles, 8 MiB, held on every device
 * that loads the library until the process exits); the image is processed in row strips that
 * fit it, and a width for which two rows plus the window's margin do not fit returns
 * PM_ERR_SCRATCH_LIMIT. The first call on a device resolves the scratch address (make it
 * before any stream capture); after cudaDeviceReset that address is stale, so do not call the
 * entry point on a device that was reset. All calls on a device share the scratch: calls that
 * overlap on the GPU race. Nothing is allocated and the work is enqueued on `stream` (NULL:
 * the default stream). */
#define PM_NOALLOC_SCRATCH_DOUBLES (1u << 20)
pm_status pm_box_moments_noalloc(const float *d_ref, size_t ref_pitch, int width, int height,
                                 int half_window, float *d_sum_i, float *d_sum_ii, float *d_c1,
                                 size_t out_pitch, void *stream);

/* ---- Philox draws (array2d_psng replacement) -------------------------------------------
 * Device-side Philox4x32-10 for n counters; out gets 4 words per counter. */
pm_status pm_philox(uint64_t seed, int n, const uint32_t *counters, uint32_t *out);

/* ---- reciprocal check ---------------------------------------------------------------------
 * No counterpart in the reference (whose fast-math divides are not reproducible on a CPU):
 * the texture-filtering sampler forms 1/z with a Newton-refined hardware reciprocal so that
 * its coordinates equal the correctly rounded ones the CPU oracle forms. Counts, over every
 * significand of the binades [2^e, 2^(e+1)) and their negatives, the values where that
 * reciprocal differs from the correctly rounded one (expected: 0). */
pm_status pm_check_reciprocal(int exp_shift, unsigned long long *mismatches);

/* ---- texture-filtering peak ----------------------------------------------------------------
 * No counterpart in the reference: the measured rate (bilinear samples per second) of layered
 * u8 texture fetches in the NCC's access pattern on the current device, with enough warps to
 * saturate the texture units -- the roofline the sweep kernel's sample rate is reported
 * against. Allocates a small texture, runs about 2 ms. */
pm_status pm_texture_peak(double *samples_per_s);

/* ---- learned proposal on a handle -------------------------------------------------------
 * No counterpart in the reference. pm_set_proposal attaches a network (not owned; NULL
 * detaches) whose batch is 1 and whose size is the handle's proposal size (pm_proposal_input
 * with d_out NULL reports it): ceil16(width / 4) x ceil16(height / 4). With init_mode
 * PM_INIT_PROPOSAL, pm_run then builds the network input from the reference and the two
 * source views nearest to it, runs the network on the handle's stream and initialises the
 * depth map from its output. A network attached to several handles must not be run by them
 * concurrently. pm_proposal_input writes the network input (DEVICE FP32 [height][width][17])
 * for training; d_out may be NULL. */
typedef struct pm_net pm_net;
pm_status pm_set_proposal(pm_handle *h, pm_net *net);
pm_status pm_proposal_input(pm_handle *h, float *d_out, int *height, int *width);

/* ---- learned depth proposal: tensor-core GEMM -----------------------------------------
 * No counterpart in the reference (its initial depth is uniformly random,
 * array2d_wrapper.cu:3-20); the building block of the proposal network's convolutions.
 * C[m, n] (+)= A[m, k] . B[n, k]^T on DEVICE memory, A and B BF16 with k contiguous (leading
 * dimensions lda, ldb in elements), on the fifth-generation tensor cores with an FP32
 * accumulator. mode 0: C is BF16, C = act(A B^T + bias); mode 1: C is FP32, C = A B^T + bias;
 * mode 2: C is FP32, C += A B^T, with k split over `splits` CTAs. act is ReLU when relu != 0.
 * m % 128 == 0, n % 16 == 0, k % 64 == 0, leading dimensions multiples of 8, pointers
 * 16-byte aligned; otherwise PM_ERR_INVALID_ARGUMENT. d_bias (n floats) may be NULL. The work
 * is enqueued on `stream` (NULL: the default stream). A pipeline wait that times out sets an
 * error word, read (and optionally cleared) with pm_gemm_error. */
pm_status pm_gemm_bf16(const void *d_a, int lda, const void *d_b, int ldb, int m, int n, int k,
                       void *d_c, int ldc, int mode, const float *d_bias, int relu, int splits,
                       void *stream);
pm_status pm_gemm_error(unsigned *out, int clear);

/* ---- learned depth proposal: the network --------------------------------------------------
 * No counterpart in the reference. A 5-level BF16 encoder-decoder (widths 32, 64, 96, 128,
 * 128; 3x3 convolutions with ReLU, nearest upsampling with skip concatenation, 1x1 head) on
 * inputs of 17 channels at a quarter of the reference resolution: the reference image and two
 * source images warped onto 8 fronto-parallel depths. Output per pixel: the normalised inverse
 * depth s in [0, 1] (depth = 1 / (1/far + s (1/near - 1/far))) and a confidence in [0, 1].
 * Every convolution runs on pm_gemm_bf16's kernel; training uses the same kernels backward.
 * A pm_net is sized for one batch and level-0 size (height, width multiples of 16); weights
 * move between nets of different sizes with pm_net_get_params / pm_net_set_params (FP32,
 * per layer: weights [cout][ky][kx][cin] then bias [cout]). seed fixes the initial weights. */
pm_status pm_net_create(int batch, int height, int width, uint64_t seed, pm_net **out);
pm_status pm_net_destroy(pm_net *net);
pm_status pm_net_num_params(const pm_net *net, size_t *n);
pm_status pm_net_size(const pm_net *net, int *batch, int *height, int *width);
pm_status pm_net_get_params(pm_net *net, float *dst, size_t n);
pm_status pm_net_set_params(pm_net *net, const float *src, size_t n);
/* d_input: DEVICE FP32 [batch][height][width][17]; d_out (may be NULL): DEVICE FP32
 * [batch][height][width][2] = (s, confidence). */
pm_status pm_net_forward(pm_net *net, const float *d_input, float *d_out, void *stream);
/* Loss and gradients for d_target (DEVICE FP32 [batch][height][width], normalised inverse
 * depth; < 0 masks a pixel): L1 of the relative inverse-depth error |inv - inv_t| / inv_t
 * (inv = inv_far + s inv_range) plus 0.1 x binary cross-entropy of the confidence against
 * "depth within 2 % of the target's". grad_out (HOST, n_grad floats, may be NULL) receives
 * dLoss/dparam with the loss taken as sum over pixels / (batch height width); loss_out (may be
 * NULL) gets 3 floats: mean relative error, mean BCE, valid pixel count. */
pm_status pm_net_gradients(pm_net *net, const float *d_input, const float *d_target, float inv_far,
                           float inv_range, float *grad_out, size_t n_grad, float *loss_out);
/* One Adam step (learning rate lr, betas 0.9 / 0.999) on that loss. */
pm_status pm_net_train_step(pm_net *net, const float *d_input, const float *d_target, float inv_far,
                            float inv_range, float lr, float *loss_out);
/* Layer table: 8 ints per layer (cin, cout, ksize, stride, relu, param offset, input height,
 * input width). */
pm_status pm_net_layout(const pm_net *net, int *n_layers, int *desc, int max_layers);

/* ---- Consistency filtering and fusion over several references (no counterpart in the
 * reference, whose output stops at one depth map per run: patchMatch.cu:263-407,
 * main.cpp:124-128). All references share one world frame.
 *
 * For pixel (x, y) of reference i with depth d and every other reference j: the pixel centre
 * (x + 1/2, y + 1/2) at depth d is projected into j, j's depth at the pixel containing the
 * projection is projected back into i, and j agrees when that round trip lands within
 * max_reproj_px pixels of the start with a depth within max_rel_depth * d of d. Pixels with
 * at least min_consistent agreeing references are kept, with the mean of d and the agreeing
 * round-trip depths as their fused depth and its back-projection as their point. Depths that
 * are not finite and positive count as missing. */
#define PM_MAX_FUSE_REFS 256

typedef struct pm_fuse_params {
    float max_reproj_px;        /* default 1                                                */
    float max_rel_depth;        /* default 0.01                                             */
    int min_consistent;         /* other references that must agree (default 2; 0 keeps
                                   every valid depth)                                       */
} pm_fuse_params;
void pm_default_fuse_params(pm_fuse_params *p);

/* One reference's depth map with its camera, on the host. */
typedef struct pm_depth_view {
    const float *depth;         /* height rows of width floats                               */
    const uint8_t *gray;        /* intensity for the points, same size, or NULL (0)          */
    int width, height;
    float K[9], R[9], t[3];     /* row-major, pixel ~ K (R X + t)                             */
} pm_depth_view;

typedef struct pm_fusion pm_fusion;
/* Copies host depth maps to the device (gpu_id < 0: the current device). */
pm_status pm_fusion_create(const pm_depth_view *views, int n, int gpu_id, pm_fusion **out);
/* Reads the engines' device depth maps in place at every pm_fusion_run (after synchronising
 * their streams), with each engine's reference texels as intensity. The engines must outlive
 * the fusion object and have a depth map (run, initialised or set). */
pm_status pm_fusion_create_from_engines(pm_handle *const *hs, int n, pm_fusion **out);
/* Filters and fuses; synchronous. May run again (e.g. after the engines ran again). */
pm_status pm_fusion_run(pm_fusion *f, const pm_fuse_params *p);
/* Points of the last run, the device time of the consistency kernel and of the whole fusion
 * (CUDA events, ms), and the kernels one run launches (4: consistency, two scan passes,
 * points). */
pm_status pm_fusion_info(const pm_fusion *f, int64_t *num_points, float *ms_check, float *ms_total,
                         int *launches);
/* Up to capacity points as (x, y, z, intensity in [0, 1]), reference by reference in row-major
 * pixel order. */
pm_status pm_fusion_get_points(pm_fusion *f, float *xyzi, int64_t capacity);
/* Reference ref's fused depth (0 where not kept) and per-pixel count of agreeing references
 * (either may be NULL). */
pm_status pm_fusion_get_depth(pm_fusion *f, int ref, float *fused, uint8_t *count);
/* The FP32 matrices the kernels use: pairs[(i n + j) 12 ..] = K_j R_j R_i^T K_i^-1 (row-major)
 * then K_j (t_j - R_j R_i^T t_i); backproject[i 12 ..] = R_i^T K_i^-1 then -R_i^T t_i. */
pm_status pm_fusion_geometry(const pm_fusion *f, float *pairs, float *backproject);
/* Binary little-endian PLY: x y z (float), gray as red = green = blue (uchar). */
pm_status pm_fusion_write_ply(pm_fusion *f, const char *path);
const char *pm_fusion_last_error(const pm_fusion *f);
pm_status pm_fusion_destroy(pm_fusion *f);

#ifdef __cplusplus
}
#endif
#endif
