/*
 * skyfall.h -- C-ABI of the GB300 Gaussian-splat render-and-train library.
 *
 * The library replaces the hot path of Skyfall-Viewer's GaussianRenderer
 * (src/renderers/gaussian-renderer.ts): projection, tile-key emission, the
 * intersection radix sort, tile ranges, the tiled forward rasterizer, the
 * loss, the tiled backward, the geometry backward, Adam, and prune/densify
 * compaction.  Every entry point returns an int status (SKY_OK == 0, negative
 * on error); sky_last_error() returns a thread-local message for the last
 * failing call on the calling thread.
 *
 * Ownership: the library owns all device memory of a context.  Host arrays
 * passed in are copied before the call returns and are never retained.
 * Threading: one context is used by one thread at a time; distinct contexts
 * are independent.  All plain types, no C++ or torch types cross the ABI.
 */
#ifndef SKYFALL_H
#define SKYFALL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define SKY_OK 0
#define SKY_ERR_ARG (-1)      /* invalid argument or size                  */
#define SKY_ERR_OOM (-2)      /* device or host allocation failed          */
#define SKY_ERR_CUDA (-3)     /* CUDA runtime error                        */
#define SKY_ERR_TIMEOUT (-4)  /* a bounded device wait gave up             */
#define SKY_ERR_CAPACITY (-5) /* intersection capacity exceeded (retried)  */
#define SKY_ERR_STATE (-6)    /* call out of order (no points, no cameras) */
#define SKY_ERR_INJECTED (-7) /* host-side fault injection (SKY_FAULT)     */

/* ---- parameter layout --------------------------------------------------
 * Per-Gaussian trainable parameters are 59 f32 planes (structure of arrays),
 * plane p of Gaussian i at params[p * plane_stride + i].  The planes mirror
 * the reference's five f32 training buffers (gaussian-renderer.ts:216-221):
 *   0..2   position x, y, z                  (train_position)
 *   3..5   log sigma x, y, z                 (train_scale)
 *   6..9   quaternion x, y, z, w             (train_rotation)
 *   10     opacity logit                     (train_opacity)
 *   11..58 SH coefficient k, channel c at 11 + 3k + c (train_sh)
 */
#define SKY_PLANE_POS 0
#define SKY_PLANE_LOGSCALE 3
#define SKY_PLANE_ROT 6
#define SKY_PLANE_OPACITY 10
#define SKY_PLANE_SH 11
#define SKY_NUM_PLANES 59

/* ---- backward modes ------------------------------------------------------ */
/* Exact adjoint of the forward (default): every composited splat, the
 * colour clamp and the view-direction term of the SH colour are
 * differentiated; per-(tile, intersection) partial sums are reduced in a
 * fixed order, so gradients are bit-stable from run to run.               */
#define SKY_BWD_EXACT 0
/* Reference semantics of backward-tiles-local.wgsl:185-382: splats with
 * alpha > 0.98 are skipped, each per-pixel value is truncated to i32 fixed
 * point (x65536) and summed per (tile, intersection) for all 54 values,
 * then summed per Gaussian exactly in i64.  Used for bit-exact parity.    */
#define SKY_BWD_REFERENCE 1

/* ---- camera ---------------------------------------------------------------
 * Mirrors TrainingCameraData / CameraUniforms (src/camera/training-camera.ts:4-15,
 * src/shaders/common.wgsl:21-28): column-major view (world->camera) and
 * projection matrices, focal lengths in pixels, and the training image size.
 */
typedef struct SkyCamera {
  float view[16];
  float proj[16];
  float focal[2];
  uint32_t width;
  uint32_t height;
} SkyCamera;

/* ---- configuration ---------------------------------------------------------
 * Defaults (sky_config_default) follow the reference: projection params
 * (gaussian-renderer.ts:474-488), background (:490-504), learning rates and
 * schedules (:82-98), Adam constants (:2422-2424), SH schedule (:3625-3636). */
typedef struct SkyConfig {
  uint32_t struct_size;        /* sizeof(SkyConfig)                          */
  uint32_t tile_size;          /* 8, 16 or 32 (reference: 16)                */
  uint32_t sh_degree;          /* SH degree of the scene, 0..3               */
  uint32_t sh_degree_interval; /* active degree = min(sh_degree, it/interval) */
  float near_plane;            /* 0.2                                        */
  float far_plane;             /* 1e4                                        */
  float radius_clip;           /* 512                                        */
  float eps2d;                 /* 0.3                                        */
  float background[3];         /* 0, 0, 0                                    */
  float w_l2, w_l1, w_ssim;    /* loss weights                               */
  float lr_means;              /* 1.6e-4, log-lerp to lr_means_final         */
  float lr_means_final;        /* 1.6e-6                                     */
  float lr_means_delay_mult;   /* 0.01                                       */
  uint32_t lr_means_max_steps; /* 30000                                      */
  float lr_sh, lr_opacity, lr_scale, lr_rotation;
  float beta1, beta2, adam_eps;
  uint32_t sh_update_interval; /* SH planes updated when it % interval == 0  */
  uint32_t round_params_f16;   /* 1: projection reads f16-rounded params, as
                                  the reference's packed storage does       */
  uint32_t backward_mode;      /* SKY_BWD_EXACT or SKY_BWD_REFERENCE         */
  uint32_t use_graph;          /* capture sky_step as one CUDA graph         */
  uint32_t max_views_per_step; /* batch size bound (buffers sized for it)    */
  uint64_t seed;               /* camera choice and densify randomness       */
  uint32_t fwd_batch;          /* splat-batch depth of the forward: 64, 128,
                                  256 (0 = 256)                              */
  uint32_t bwd_batch;          /* of the 16x16-tile exact backward: 32, 64,
                                  128 (0 = 64); neither changes a result,
                                  both may change with sky_set_config        */
  uint32_t tile_cull;          /* 1: the intersection lists of backward and
                                  training steps in the exact backward mode
                                  hold only the tiles of each Gaussian's
                                  rectangle that its alpha >= 1/255 ellipse
                                  reaches.  Images, loss, gradients,
                                  statistics and parameters are
                                  bit-identical to 0 (the reference's lists:
                                  every tile of the rectangle); the per-item
                                  counts, keys and tile ranges of those steps
                                  are the shorter lists.  Renders, forward
                                  passes and the reference backward mode
                                  always list every tile.  Default 0.        */
  uint32_t batch_scaling;      /* Adam hyperparameters of a step of B views.
                                  0: those of one view, whatever B (the
                                  reference trains one view per step).
                                  1: the learning rates times sqrt(B), beta1
                                  and beta2 raised to the power B, bias
                                  correction counted in views (the batch
                                  rule of Zhao et al. 2024, "On Scaling Up
                                  3D Gaussian Splatting Training"); steps of
                                  one view are unchanged.  Default 0.        */
} SkyConfig;

typedef struct SkyStepStats {
  uint64_t iteration;         /* training iteration after this step         */
  uint64_t num_intersections; /* sum over the step's views                  */
  double loss;                /* sum over pixels/channels of
                                 0.5 w_l2 r^2 + w_l1 |r| (no SSIM term)      */
  uint32_t num_gaussians;
  uint32_t num_views;
  uint32_t sh_degree;         /* active SH degree used by this step         */
  uint32_t sh_updated;        /* 1 if the SH planes took an Adam step       */
} SkyStepStats;

typedef struct SkyStatus {
  uint64_t iteration;
  uint64_t adam_steps;
  uint64_t last_intersections;
  uint64_t device_bytes;      /* device memory held by the context          */
  uint32_t num_gaussians;
  uint32_t capacity;
  uint32_t num_cameras;
  uint32_t error_flags;       /* sticky device error word (0 = none)        */
  uint64_t kernel_launches;   /* kernels launched by the context so far     */
  uint64_t graph_replays;     /* training steps run as a graph replay       */
  uint64_t graph_captures;    /* graph (re-)captures                        */
  float scene_extent;         /* max bounding-box extent of the loaded points */
  uint32_t scored_views;      /* views behind the current multi-view scores */
  uint32_t densify_runs;      /* sky_densify calls that changed the scene   */
  uint32_t prune_runs;        /* prunes that removed Gaussians              */
  uint64_t step_h2d_bytes;    /* host->device bytes the passes copied (step
                                 parameters), cumulative                    */
  uint64_t step_d2h_bytes;    /* device->host bytes the passes copied (step
                                 status: loss, counts), cumulative; images
                                 and gradients returned by sky_render /
                                 sky_backward are not included              */
} SkyStatus;

/* Stages timed by sky_set_profiling / sky_get_stage_times, in order.  The
 * reference's TrainingProfiler (src/utils/training-profiler.ts:27-192) times
 * the same passes with wall clock around queue fences; here each stage is
 * bracketed by CUDA events on the context's stream.                       */
#define SKY_STAGE_PREPROCESS 0
#define SKY_STAGE_SCAN 1
#define SKY_STAGE_EMIT 2
#define SKY_STAGE_SORT 3
#define SKY_STAGE_RANGES 4
#define SKY_STAGE_FORWARD 5
#define SKY_STAGE_BACKWARD 6
#define SKY_STAGE_GEOM_ADAM 7
#define SKY_NUM_STAGES 8

/* Prune rule of applyMultiViewPrune (gaussian-renderer.ts:2840-2886) with
 * the random budget replaced by a seeded one: prunable if
 * sigmoid(logit) < min_opacity or max(exp(log sigma)) > max_scale.  The
 * removal set is capped at max_remove_ratio * N when that is > 0.        */
typedef struct SkyPruneParams {
  float min_opacity;       /* 0.005                      */
  float max_scale;         /* scene_extent * 0.1         */
  float max_remove_ratio;  /* 0 = no cap                 */
  uint32_t reserved;
} SkyPruneParams;

/* Densify rule of performDensification (gaussian-renderer.ts:3248-3318):
 * a Gaussian seen in >= min_visibility steps whose multi-view importance
 * (error-pixel count / scored views) exceeds importance_threshold is cloned
 * when max sigma <= size_threshold and its mean |dL/dmean2d| >=
 * grad_threshold * pixel_width / 2, split when larger and its mean
 * |dL/dconic| >= grad_abs_threshold * pixel_width / 2.  At most
 * max(1, floor(max_new_ratio * N)) candidates, by descending normalised
 * gradient, are applied.  sky_densify_default fills the reference values. */
typedef struct SkyDensifyParams {
  float grad_threshold;      /* 0.003 (scaled by width / 2)           */
  float grad_abs_threshold;  /* 0.015 (scaled by width / 2)           */
  float size_threshold;      /* 0.001 * scene extent                  */
  float min_visibility;      /* 25                                    */
  float importance_threshold;/* 5 (MULTI_VIEW_IMPORTANCE_THRESHOLD)   */
  float max_new_ratio;       /* 0.1                                   */
  float pixel_width;         /* 0: width of camera 0                  */
  uint32_t reserved;
} SkyDensifyParams;

/* Multi-view weighted prune of applyMultiViewPrune (gaussian-renderer.ts:
 * 2800-2915).  Prunable: sigmoid(logit) < min_opacity, max sigma >
 * max_scale, or (use_screen_size) decayed max screen radius >
 * max_screen_radius.  Each prunable Gaussian gets the weight
 * 1 / (1e-6 + 1 - clamp(normalised pruning score + bonuses, 0, 0.999)) and
 * min(prunable, max(1, floor(prune_ratio * prunable)),
 *     max(1, floor(max_ratio * scored count))) of them are drawn without
 * replacement with probability proportional to weight (seeded).          */
typedef struct SkyScoredPruneParams {
  float min_opacity;       /* 0.005                                     */
  float max_scale;         /* 1.0 (maxScaleAbsolute)                    */
  float max_screen_radius; /* 20 pixels                                 */
  uint32_t use_screen_size;/* 1 after the first opacity reset           */
  float prune_ratio;       /* 0.5  (MULTI_VIEW_PRUNE_RATIO)             */
  float max_ratio;         /* 0.02 (MULTI_VIEW_PRUNE_MAX_RATIO)         */
  float opacity_bonus;     /* 0.35                                      */
  float scale_bonus;       /* 0.25                                      */
  float screen_bonus;      /* 0.25                                      */
  uint32_t use_last_scores;/* 1: use the last scores even if a densify
                              has run since (runDensifyAndPruneCombined
                              :3468-3490); 0: rescore if stale          */
} SkyScoredPruneParams;

/* Training schedule of TrainingController (src/utils/training-controller.ts:
 * 23-160), run by sky_train after each step when enabled: densify (with
 * the combined prune) every densify_interval steps in [densify_from,
 * densify_until], otherwise prune every prune_interval steps in
 * [prune_from, prune_until], and clamp opacities to opacity_reset_value
 * every opacity_reset_interval steps inside the densify window.          */
typedef struct SkySchedule {
  uint32_t enabled;
  uint32_t densify_from, densify_until, densify_interval;   /* 500, 15000, 100 */
  uint32_t prune_from, prune_until, prune_interval;         /* 500, 25000, 100 */
  uint32_t opacity_reset_interval;                          /* 3000            */
  float opacity_reset_value;                                /* 0.01            */
  float min_opacity;                                        /* 0.005           */
  float max_screen_size;                                    /* 20              */
  float max_scale_ratio;                                    /* 0               */
  float max_scale_absolute;                                 /* 1.0             */
  float scene_extent;                                       /* 0: from points  */
  SkyDensifyParams densify;
} SkySchedule;

/* ---- buffers readable with sky_read_buffer (introspection) -------------- */
#define SKY_BUF_RECORDS 1      /* per (view, Gaussian) raster record, 12 f32:
                                  mean x, y, conic a, b, c, opacity, colour r,
                                  g, b, alpha-skip bound on s, box half-widths */
#define SKY_BUF_COUNTS 2       /* per (view, Gaussian) tile count, u32            */
#define SKY_BUF_CUMSUM 3       /* inclusive scan of the counts taken in emission
                                  order (SKY_BUF_ITEM_ORDER), u32                 */
#define SKY_BUF_KEYS_EMIT 4    /* keys in emission order, u32                     */
#define SKY_BUF_ITEM_ORDER 20  /* (view, Gaussian) item at each emission position:
                                  items by (view, depth16, Gaussian), u32        */
#define SKY_BUF_KEYS_SORTED 5  /* keys after the sort, u32                        */
#define SKY_BUF_VALS_SORTED 6  /* emission index after the sort, u32              */
#define SKY_BUF_FLATTEN 7      /* record index per sorted intersection, u32       */
#define SKY_BUF_TILE_OFFSETS 8 /* tile range starts, total tiles + 1, u32         */
#define SKY_BUF_COLOR 9        /* rendered rgba f32 per pixel                     */
#define SKY_BUF_ALPHA 10       /* accumulated alpha f32 per pixel                 */
#define SKY_BUF_LAST_IDS 11    /* last visited intersection per pixel, u32        */
#define SKY_BUF_RESIDUAL 12    /* dL/dcolor rgba f32 per pixel                    */
#define SKY_BUF_PARTIALS 13    /* per intersection (emission order) 12 f32        */
#define SKY_BUF_TILE_GRADS 14  /* reference mode: 54 i32 per sorted intersection  */
#define SKY_BUF_GRADS 15       /* 59 gradient planes of the last backward         */
#define SKY_BUF_GROUPS 16      /* per sort group: begin, end intersection, u32    */
#define SKY_BUF_DEPTH_RADIUS 18 /* per (view, Gaussian) camera depth, radius, f32 */
#define SKY_BUF_PAIR_COUNTS 21  /* 8 u64 of the last pass, counted only at profiling
                                   level 2 (16x16 tiles, default batch depths):
                                   forward (pixel, splat) pairs evaluated, pairs
                                   composited, warp list entries (32 pixels
                                   each); backward pixel pairs evaluated, pairs
                                   contributing, warp list entries (64 pixels
                                   each), entries at which no pixel of the warp
                                   contributed; 0                                */
#define SKY_BUF_STEP_SCALARS 17 /* f32: lr pos, scale, rot, opacity, sh, beta1,
                                   beta2, eps, bias-correction 1/bc1, 1/sqrt(bc2),
                                   SH degree, SH-update flag                     */

/* ---- lifecycle ------------------------------------------------------------ */
void sky_config_default(SkyConfig* cfg);
int sky_create(const SkyConfig* cfg, void** ctx_out);
int sky_destroy(void* ctx);
int sky_set_config(void* ctx, const SkyConfig* cfg); /* mutable fields only   */
int sky_get_config(void* ctx, SkyConfig* out);       /* the context's config  */
const char* sky_last_error(void);
int sky_version(void);

/* Builds a training camera exactly as get_pinhole_projection_matrix
 * (src/camera/training-camera.ts:29-52) does: f64 arithmetic, f32 storage. */
int sky_camera_pinhole(const float view[16], double fx, double fy, double cx,
                       double cy, uint32_t width, uint32_t height, SkyCamera* out);

/* ---- scene ------------------------------------------------------------------
 * sky_load_points replaces reloadPointCloud + training_init_params
 * (gaussian-renderer.ts:2092-2126, training-params.wgsl:35-79);
 * sky_load_packed takes the reference's packed f16 buffers (Gaussian = 6 u32
 * words, SH = 24 u32 words, common.wgsl:39-43).                              */
int sky_load_points(void* ctx, const float* params, uint32_t n, uint64_t plane_stride);
int sky_load_packed(void* ctx, const uint32_t* gaussians, const uint32_t* sh, uint32_t n);
/* sky_load_ply replaces loadPlyFile / load() (src/utils/dataset-loader.ts:19,
 * src/utils/load.ts:14-172, src/utils/plyreader.ts): binary little-endian
 * PLY, 3DGS layout (f_dc_*, f_rest_*, opacity, scale_*, rot_0 = w) or xyz
 * (+ rgb) point clouds with the reference's defaults; values are stored
 * through f16 as the reference's packed buffers hold them.  n_out and
 * sh_degree_out (may be NULL) receive the count and the file's SH degree;
 * the scene extent becomes the max bounding-box extent of the positions.
 * sky_save_ply writes the 3DGS layout (f32; rot_0 = w) for coefficients up
 * to sh_degree -- it has no counterpart in the reference.
 * sky_save_checkpoint / sky_load_checkpoint store and restore the whole
 * training state (parameters, Adam moments, densification statistics,
 * iteration and Adam counters, the camera-choice generator): training
 * resumed from a checkpoint continues bit for bit as if uninterrupted.
 * They have no counterpart in the reference.                               */
int sky_load_ply(void* ctx, const char* path, uint32_t* n_out, uint32_t* sh_degree_out);
/* The same import into host memory, without a context or a GPU: call with
 * planes == NULL for the count, then with room for 59 * n floats (plane p of
 * Gaussian i at planes[p * n + i]).  extent_out (may be NULL) receives the
 * scene extent.                                                             */
int sky_ply_read_host(const char* path, uint32_t* n_out, uint32_t* sh_degree_out, float* planes,
                      uint64_t capacity_floats, double* extent_out);
int sky_save_ply(void* ctx, const char* path, uint32_t sh_degree);
int sky_save_checkpoint(void* ctx, const char* path);
int sky_load_checkpoint(void* ctx, const char* path);
/* sky_knn_init replaces initializeKnnAndSync (gaussian-renderer.ts:2131-2171,
 * knn-init.wgsl:40-90): per Gaussian the mean distance to its three nearest
 * other Gaussians (positions through f16), sigma = min(clamp(max(mean / 3,
 * 0.0015 E), 0.0007 E, 0.007 E), 0.1) with E = scene_extent (0: the
 * context's), and every parameter re-read through f16 with log sigma in
 * the three scale planes.  density_out (n floats, may be NULL) receives the
 * mean distances.  Exact nearest neighbours from a uniform grid instead of
 * the reference's all-pairs scan; results are identical.                  */
int sky_knn_init(void* ctx, float scene_extent, float* density_out);
int sky_set_cameras(void* ctx, const SkyCamera* cams, uint32_t n);  /* setTrainingCameras :4084 */
int sky_set_target(void* ctx, uint32_t camera, const float* rgb, uint32_t width,
                   uint32_t height);                                /* setTrainingImages :4098 */

/* ---- hot path --------------------------------------------------------------
 * sky_render: forward only for n cameras; rgba (4 f32) and alpha (1 f32) per
 * pixel, images concatenated in camera order (either pointer may be NULL).
 * sky_forward + sky_backward: the forward/backward op pair; sky_forward also
 * evaluates the loss against the cameras' targets, sky_backward returns the
 * 59 gradient planes (summed over the forward's views) without an Adam step.
 * sky_step: one training step over n cameras (trainStep :3638-3660, batched);
 * sky_train: the reference train(n) loop (:3744-3854) with a seeded camera
 * choice, one camera per step.                                               */
int sky_render(void* ctx, const uint32_t* cameras, uint32_t n, float* rgba, float* alpha);
int sky_forward(void* ctx, const uint32_t* cameras, uint32_t n, double* loss);
int sky_backward(void* ctx, float* grads, uint64_t plane_stride);
int sky_step(void* ctx, const uint32_t* cameras, uint32_t n, SkyStepStats* stats);
int sky_train(void* ctx, uint32_t iterations, uint32_t views_per_step, SkyStepStats* last);

/* ---- prune / densify / opacity reset ------------------------------------
 * sky_prune: rule or mask prune without the random budget (prune-decide
 * path), compaction as applyPruneMask (:2917-3000).
 * sky_densify_stats: per Gaussian the densify accumulator (|dmean2d| sum, 0,
 * |dconic| sum, count; densify-accum.wgsl) and the importance statistics
 * (decayed tile count, visibility, max screen radius, 0;
 * importance-accum.wgsl), 4 f32 each, gathered by every training step.
 * sky_score_views: multi-view error scores (generateMultiViewScores
 * :2758-2788) over the given cameras, or when cameras is NULL over
 * min(10, cameras) drawn by the context's seeded generator; per Gaussian a
 * u32 importance (error-pixel hits) and an f32 pruning score (hits x mean
 * L1 of the view).  Scores are kept for sky_densify / sky_prune_scored in
 * the same iteration (getMultiViewScores :2790-2798).
 * sky_densify: clone/split on the device; new Gaussians are appended after
 * the survivors with zero Adam moments; resets both statistics.
 * sky_prune_scored: the weighted prune; resets both statistics.          */
int sky_prune(void* ctx, const SkyPruneParams* p, const uint8_t* mask, uint32_t* removed);
int sky_densify_stats(void* ctx, float* grad_accum, float* importance);
int sky_score_views(void* ctx, const uint32_t* cameras, uint32_t n, uint32_t* importance,
                    float* pruning);
void sky_densify_default(SkyDensifyParams* p);
int sky_densify(void* ctx, const SkyDensifyParams* p, uint32_t* cloned, uint32_t* split);
void sky_scored_prune_default(SkyScoredPruneParams* p);
int sky_prune_scored(void* ctx, const SkyScoredPruneParams* p, uint32_t* removed);
int sky_reset_opacity(void* ctx, float max_opacity);                   /* resetOpacity :3867 */
void sky_schedule_default(SkySchedule* s);
int sky_set_schedule(void* ctx, const SkySchedule* s);

/* ---- headless viewer frame --------------------------------------------------
 * The viewer path of frame(encoder, view) (gaussian-renderer.ts:4111-4123):
 * preprocess.wgsl:116-215 per Gaussian, a global back-to-front depth sort,
 * and one quad of half-width ceil(3 sqrt(lambda_max)) per splat blended
 * "over" (src-alpha, one-minus-src-alpha; gaussian.wgsl:15-67) into a target
 * cleared to transparent black.  The swapchain texture becomes an f32 RGBA
 * buffer (W x H x 4, row-major, y down); rgba8, if given, receives it
 * converted as round(clamp(v, 0, 1) * 255).  Either pointer may be NULL (the
 * image stays readable as SKY_BUF_VIEW_RGBA).  Camera: view, proj, focal and
 * the viewport size (width, height) as in SkyCamera.                       */
typedef struct SkyViewSettings {
  float gaussian_scaling;     /* RenderSettings.gaussian_scaling, 1.0      */
  uint32_t sh_degree;         /* RenderSettings.sh_deg, 0..3               */
  uint32_t round_params_f16;  /* 1: parameters read through f16 storage   */
  uint32_t reserved;
} SkyViewSettings;
#define SKY_BUF_VIEW_RGBA 19  /* last viewer frame, 4 f32 per pixel */
void sky_view_settings_default(SkyViewSettings* s);
int sky_view_render(void* ctx, const SkyCamera* camera, const SkyViewSettings* s, float* rgba,
                    uint8_t* rgba8);

/* ---- readback ------------------------------------------------------------- */
int sky_get_params(void* ctx, float* params, uint64_t plane_stride);
int sky_get_moments(void* ctx, float* m1, float* m2, uint64_t plane_stride);
int sky_get_count(void* ctx, uint32_t* n);
int sky_get_status(void* ctx, SkyStatus* st);
int sky_read_buffer(void* ctx, int which, void* dst, uint64_t bytes, uint64_t* size_out);
int sky_sync(void* ctx);

/* ---- streams and profiling ------------------------------------------------
 * sky_get_stream: the cudaStream_t all of the context's work runs on, so a
 * caller can order its own work (or CUDA events) against it.
 * sky_set_profiling(1) resets and starts per-stage timing (profiledTrainStep,
 * gaussian-renderer.ts:3662-3742); sky_get_stage_times returns the summed
 * milliseconds of SKY_NUM_STAGES stages and the number of timed steps.
 * sky_set_profiling(2) also runs the rasterizers' counting variants, which
 * fill SKY_BUF_PAIR_COUNTS (same results, somewhat slower); 0 stops.      */
int sky_get_stream(void* ctx, void** stream);
int sky_set_profiling(void* ctx, int enabled);
int sky_get_stage_times(void* ctx, double* ms, uint32_t n, uint64_t* steps);

/* ---- device-pointer operators --------------------------------------------
 * Stable LSD radix sort of (u32 key, u32 value) pairs on the low key_bits
 * bits, replacing get_sorter(...).sort (src/sort/sort.ts:260-370,
 * radix_sort.wgsl:55-519).  All pointers are device pointers; stream is a
 * cudaStream_t (NULL = legacy default stream).  Input and output arrays must
 * not overlap.  Scratch is allocated and cached by the library per device.  */
int sky_sort_pairs(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                   uint32_t* vals_out, uint32_t n, uint32_t key_bits, void* stream);

/* The same sort for callers that cannot let the library allocate device
 * memory (a host that owns the whole GPU through its own pool or caching
 * allocator, or code that must not call cudaMalloc mid-work).  It has no
 * counterpart in the reference.  It allocates nothing: its scratch is one
 * fixed device array (about 9 MiB, held by every GPU that loads the library
 * until the process exits), so n is limited to SKY_SORT_NOALLOC_MAX_KEYS
 * (larger n returns SKY_ERR_ARG).  The first call on a device looks up that
 * array's address with the device current; make it before any stream
 * capture begins.  The address is kept for the life of the process, so a
 * cudaDeviceReset after that first call is not supported (the same holds for
 * the scratch sky_sort_pairs caches).  All calls share the array: calls whose
 * GPU work overlaps race with each other and must be serialised.  Like
 * sky_sort_pairs, the call returns once the sort has finished: it reads the
 * sort's error word back and waits for `stream`.                          */
#define SKY_SORT_NOALLOC_MAX_KEYS (1u << 20)
int sky_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                           uint32_t* vals_out, uint32_t n, uint32_t key_bits, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SKYFALL_H */
