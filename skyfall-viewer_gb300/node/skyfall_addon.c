/*
 * skyfall_addon.c -- Node N-API binding of libskyfall (include/skyfall.h) for
 * the TypeScript host of Skyfall-Viewer.
 *
 * It replaces, for the render-and-train hot path, the WebGPU work behind the
 * GaussianRenderer object of src/renderers/gaussian-renderer.ts (interface
 * :30-58, returned object :4110-4153).  skyfall-renderer.ts wraps these
 * functions in a class with the reference's method names.  Every function
 * takes the context handle (an external created by create()) first, copies
 * typed arrays in or out synchronously, and throws a JS Error carrying
 * sky_last_error() when the library returns a negative status.  step() and
 * train() run on a libuv worker and return Promises, as the reference's
 * train() does; a context must not be used by two calls at once (the façade
 * serialises them).
 *
 * Build: node-gyp with binding.gyp in this folder (links libskyfall.so from
 * ../skyfall and adds ../../include to the include path).
 */
#include <node_api.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "skyfall.h"

/* ---- helpers -------------------------------------------------------------- */

#define NAPI_OK(env, call)                                                     \
  do {                                                                         \
    if ((call) != napi_ok) {                                                   \
      napi_throw_error((env), "SKY_NAPI", "N-API call failed: " #call);        \
      return NULL;                                                             \
    }                                                                          \
  } while (0)

#define SKY_OK_OR_THROW(env, rc)                                               \
  do {                                                                         \
    int rc_ = (rc);                                                            \
    if (rc_ != SKY_OK) {                                                       \
      throw_sky((env), rc_);                                                   \
      return NULL;                                                             \
    }                                                                          \
  } while (0)

static const char* status_name(int rc) {
  switch (rc) {
    case SKY_ERR_ARG: return "SKY_ERR_ARG";
    case SKY_ERR_OOM: return "SKY_ERR_OOM";
    case SKY_ERR_CUDA: return "SKY_ERR_CUDA";
    case SKY_ERR_TIMEOUT: return "SKY_ERR_TIMEOUT";
    case SKY_ERR_CAPACITY: return "SKY_ERR_CAPACITY";
    case SKY_ERR_STATE: return "SKY_ERR_STATE";
    case SKY_ERR_INJECTED: return "SKY_ERR_INJECTED";
    default: return "SKY_ERR";
  }
}

static void throw_sky(napi_env env, int rc) { napi_throw_error(env, status_name(rc), sky_last_error()); }

/* The n arguments of the call; missing ones are `undefined`. */
static int get_args(napi_env env, napi_callback_info info, size_t n, napi_value* argv) {
  size_t argc = n;
  if (napi_get_cb_info(env, info, &argc, argv, NULL, NULL) != napi_ok) return 0;
  for (size_t k = argc; k < n; ++k) napi_get_undefined(env, &argv[k]);
  return 1;
}

/* The external behind a context handle: destroy() releases the context at
 * once and clears it; the finalizer releases what is left at collection. */
typedef struct {
  void* ctx;
} Handle;

static void* get_ctx(napi_env env, napi_value v) {
  Handle* h = NULL;
  if (napi_get_value_external(env, v, (void**)&h) != napi_ok || h == NULL) {
    napi_throw_type_error(env, "SKY_NAPI", "expected a skyfall context");
    return NULL;
  }
  if (h->ctx == NULL) {
    napi_throw_error(env, "SKY_ERR_STATE", "the skyfall context was destroyed");
    return NULL;
  }
  return h->ctx;
}

static int is_nullish(napi_env env, napi_value v) {
  napi_valuetype t;
  if (napi_typeof(env, v, &t) != napi_ok) return 1;
  return t == napi_undefined || t == napi_null;
}

/* Data pointer and element count of a typed array of the expected type. */
static void* typed(napi_env env, napi_value v, napi_typedarray_type want, size_t* len) {
  napi_typedarray_type t;
  size_t n = 0, off = 0;
  void* data = NULL;
  napi_value ab;
  if (napi_get_typedarray_info(env, v, &t, &n, &data, &ab, &off) != napi_ok || t != want) {
    napi_throw_type_error(env, "SKY_NAPI", "typed array of the wrong type");
    return NULL;
  }
  *len = n;
  return data;
}

static int get_u32(napi_env env, napi_value v, uint32_t* out) {
  if (napi_get_value_uint32(env, v, out) != napi_ok) {
    napi_throw_type_error(env, "SKY_NAPI", "expected an unsigned integer");
    return 0;
  }
  return 1;
}

static int get_f64(napi_env env, napi_value v, double* out) {
  if (napi_get_value_double(env, v, out) != napi_ok) {
    napi_throw_type_error(env, "SKY_NAPI", "expected a number");
    return 0;
  }
  return 1;
}

/* Optional named number property of an object (absent: left unchanged). */
static int opt_f64(napi_env env, napi_value obj, const char* name, double* out) {
  bool has = false;
  if (is_nullish(env, obj)) return 1;
  if (napi_has_named_property(env, obj, name, &has) != napi_ok) return 0;
  if (!has) return 1;
  napi_value v;
  if (napi_get_named_property(env, obj, name, &v) != napi_ok) return 0;
  return get_f64(env, v, out);
}

static int opt_float(napi_env env, napi_value obj, const char* name, float* out) {
  double d = *out;
  if (!opt_f64(env, obj, name, &d)) return 0;
  *out = (float)d;
  return 1;
}

static int opt_uint(napi_env env, napi_value obj, const char* name, uint32_t* out) {
  double d = *out;
  if (!opt_f64(env, obj, name, &d)) return 0;
  *out = (uint32_t)d;
  return 1;
}

static int set_num(napi_env env, napi_value obj, const char* name, double v) {
  napi_value x;
  return napi_create_double(env, v, &x) == napi_ok && napi_set_named_property(env, obj, name, x) == napi_ok;
}

static napi_value undefined(napi_env env) {
  napi_value u;
  napi_get_undefined(env, &u);
  return u;
}

/* A new typed array of `count` elements of `bytes_each`; *data receives its storage. */
static napi_value new_typed(napi_env env, napi_typedarray_type t, size_t count, size_t bytes_each,
                            void** data) {
  napi_value ab, out;
  if (napi_create_arraybuffer(env, count * bytes_each, data, &ab) != napi_ok) return NULL;
  if (napi_create_typedarray(env, t, count, ab, 0, &out) != napi_ok) return NULL;
  return out;
}

/* One camera of a JS array: {view, proj: Float32Array(16), focal:
 * Float32Array(2), width, height}. */
static int read_camera(napi_env env, napi_value o, SkyCamera* cam) {
  const char* mats[2] = {"view", "proj"};
  float* dst[2] = {cam->view, cam->proj};
  memset(cam, 0, sizeof(*cam));
  for (int m = 0; m < 2; ++m) {
    napi_value a;
    size_t len = 0;
    if (napi_get_named_property(env, o, mats[m], &a) != napi_ok) return 0;
    const float* src = (const float*)typed(env, a, napi_float32_array, &len);
    if (!src || len != 16) {
      napi_throw_type_error(env, "SKY_NAPI", "camera view/proj must be Float32Array(16)");
      return 0;
    }
    memcpy(dst[m], src, 16 * sizeof(float));
  }
  napi_value f;
  size_t flen = 0;
  if (napi_get_named_property(env, o, "focal", &f) != napi_ok) return 0;
  const float* fp = (const float*)typed(env, f, napi_float32_array, &flen);
  if (!fp || flen < 2) return 0;
  cam->focal[0] = fp[0];
  cam->focal[1] = fp[1];
  napi_value w, h;
  if (napi_get_named_property(env, o, "width", &w) != napi_ok ||
      napi_get_named_property(env, o, "height", &h) != napi_ok)
    return 0;
  return get_u32(env, w, &cam->width) && get_u32(env, h, &cam->height);
}

/* ---- lifecycle and configuration ---------------------------------------- */

static void finalize_ctx(napi_env env, void* data, void* hint) {
  (void)env;
  (void)hint;
  Handle* h = (Handle*)data;
  if (h->ctx) sky_destroy(h->ctx);
  free(h);
}

/* Applies the mutable SkyConfig fields present in a JS object (the names of
 * TrainingParams / LossWeights of gaussian-renderer.ts:99-113, plus the
 * library's own switches). */
static int apply_config(napi_env env, napi_value o, SkyConfig* c) {
  return opt_float(env, o, "lr_means", &c->lr_means) && opt_float(env, o, "lr_sh", &c->lr_sh) &&
         opt_float(env, o, "lr_opacity", &c->lr_opacity) && opt_float(env, o, "lr_scale", &c->lr_scale) &&
         opt_float(env, o, "lr_rotation", &c->lr_rotation) &&
         opt_uint(env, o, "sh_update_interval", &c->sh_update_interval) &&
         opt_float(env, o, "w_l2", &c->w_l2) && opt_float(env, o, "w_l1", &c->w_l1) &&
         opt_float(env, o, "w_ssim", &c->w_ssim) && opt_uint(env, o, "fwdBatch", &c->fwd_batch) &&
         opt_uint(env, o, "bwdBatch", &c->bwd_batch) && opt_uint(env, o, "tileCull", &c->tile_cull) &&
         opt_uint(env, o, "batchScaling", &c->batch_scaling);
}

/* create({tileSize, shDegree, useGraph, maxViewsPerStep, seed, ...config}?) */
static napi_value Create(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  if (!get_args(env, info, 1, argv)) return NULL;
  SkyConfig cfg;
  sky_config_default(&cfg);
  double seed = (double)cfg.seed;
  if (!opt_uint(env, argv[0], "tileSize", &cfg.tile_size) ||
      !opt_uint(env, argv[0], "shDegree", &cfg.sh_degree) ||
      !opt_uint(env, argv[0], "shDegreeInterval", &cfg.sh_degree_interval) ||
      !opt_uint(env, argv[0], "useGraph", &cfg.use_graph) ||
      !opt_uint(env, argv[0], "maxViewsPerStep", &cfg.max_views_per_step) ||
      !opt_uint(env, argv[0], "backwardMode", &cfg.backward_mode) ||
      !opt_f64(env, argv[0], "seed", &seed) || !apply_config(env, argv[0], &cfg))
    return NULL;
  cfg.seed = (uint64_t)seed;
  Handle* h = (Handle*)calloc(1, sizeof(Handle));
  if (!h) {
    napi_throw_error(env, "SKY_ERR_OOM", "out of host memory");
    return NULL;
  }
  int rc = sky_create(&cfg, &h->ctx);
  if (rc != SKY_OK) {
    free(h);
    throw_sky(env, rc);
    return NULL;
  }
  napi_value out;
  if (napi_create_external(env, h, finalize_ctx, NULL, &out) != napi_ok) {
    sky_destroy(h->ctx);
    free(h);
    napi_throw_error(env, "SKY_NAPI", "napi_create_external failed");
    return NULL;
  }
  return out;
}

/* getConfig(ctx) -> the mutable fields; setConfig(ctx, partial) */
static napi_value GetConfig(napi_env env, napi_callback_info info) {
  napi_value argv[1], o;
  if (!get_args(env, info, 1, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyConfig c;
  c.struct_size = sizeof c;
  SKY_OK_OR_THROW(env, sky_get_config(ctx, &c));
  NAPI_OK(env, napi_create_object(env, &o));
  set_num(env, o, "lr_means", c.lr_means);
  set_num(env, o, "lr_sh", c.lr_sh);
  set_num(env, o, "lr_opacity", c.lr_opacity);
  set_num(env, o, "lr_scale", c.lr_scale);
  set_num(env, o, "lr_rotation", c.lr_rotation);
  set_num(env, o, "sh_update_interval", c.sh_update_interval);
  set_num(env, o, "w_l2", c.w_l2);
  set_num(env, o, "w_l1", c.w_l1);
  set_num(env, o, "w_ssim", c.w_ssim);
  set_num(env, o, "fwdBatch", c.fwd_batch);
  set_num(env, o, "bwdBatch", c.bwd_batch);
  set_num(env, o, "tileCull", c.tile_cull);
  set_num(env, o, "batchScaling", c.batch_scaling);
  set_num(env, o, "tileSize", c.tile_size);
  set_num(env, o, "shDegree", c.sh_degree);
  return o;
}

static napi_value SetConfig(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyConfig c;
  c.struct_size = sizeof c;
  SKY_OK_OR_THROW(env, sky_get_config(ctx, &c));
  if (!apply_config(env, argv[1], &c)) return NULL;
  SKY_OK_OR_THROW(env, sky_set_config(ctx, &c));
  return undefined(env);
}

/* destroy(ctx): releases the context and its device memory now instead of at
 * garbage collection; later calls with the handle throw SKY_ERR_STATE. */
static napi_value Destroy(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  Handle* h = NULL;
  if (!get_args(env, info, 1, argv)) return NULL;
  if (napi_get_value_external(env, argv[0], (void**)&h) != napi_ok || h == NULL) {
    napi_throw_type_error(env, "SKY_NAPI", "expected a skyfall context");
    return NULL;
  }
  if (h->ctx) {
    void* ctx = h->ctx;
    h->ctx = NULL;
    SKY_OK_OR_THROW(env, sky_destroy(ctx));
  }
  return undefined(env);
}

/* ---- scene ---------------------------------------------------------------- */

/* loadPoints(ctx, Float32Array(59 * n) plane-major, n) */
static napi_value LoadPoints(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  uint32_t n = 0;
  size_t len = 0;
  if (!get_args(env, info, 3, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  const float* p = (const float*)typed(env, argv[1], napi_float32_array, &len);
  if (!p || !get_u32(env, argv[2], &n)) return NULL;
  if (len < (size_t)SKY_NUM_PLANES * n) {
    napi_throw_range_error(env, "SKY_ERR_ARG", "params must hold 59 * n floats");
    return NULL;
  }
  SKY_OK_OR_THROW(env, sky_load_points(ctx, p, n, n));
  return undefined(env);
}

/* loadPacked(ctx, Uint32Array(6 n) gaussians, Uint32Array(24 n) | null sh, n):
 * the reference's packed f16 buffers (common.wgsl:39-43) as they are. */
static napi_value LoadPacked(napi_env env, napi_callback_info info) {
  napi_value argv[4];
  uint32_t n = 0;
  size_t lg = 0, ls = 0;
  if (!get_args(env, info, 4, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  const uint32_t* g = (const uint32_t*)typed(env, argv[1], napi_uint32_array, &lg);
  if (!g || !get_u32(env, argv[3], &n)) return NULL;
  const uint32_t* sh = NULL;
  if (!is_nullish(env, argv[2])) {
    sh = (const uint32_t*)typed(env, argv[2], napi_uint32_array, &ls);
    if (!sh) return NULL;
    if (ls < (size_t)24 * n) {
      napi_throw_range_error(env, "SKY_ERR_ARG", "sh must hold 24 * n words");
      return NULL;
    }
  }
  if (lg < (size_t)6 * n) {
    napi_throw_range_error(env, "SKY_ERR_ARG", "gaussians must hold 6 * n words");
    return NULL;
  }
  SKY_OK_OR_THROW(env, sky_load_packed(ctx, g, sh, n));
  return undefined(env);
}

static int get_path(napi_env env, napi_value v, char* buf, size_t cap) {
  size_t got = 0;
  if (napi_get_value_string_utf8(env, v, buf, cap, &got) != napi_ok || got + 1 >= cap) {
    napi_throw_type_error(env, "SKY_NAPI", "expected a path string");
    return 0;
  }
  return 1;
}

/* loadPly(ctx, path) -> {count, shDegree}  (loadPlyFile + reloadPointCloud) */
static napi_value LoadPly(napi_env env, napi_callback_info info) {
  napi_value argv[2], o;
  char path[4096];
  uint32_t n = 0, deg = 0;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_path(env, argv[1], path, sizeof path)) return NULL;
  SKY_OK_OR_THROW(env, sky_load_ply(ctx, path, &n, &deg));
  NAPI_OK(env, napi_create_object(env, &o));
  set_num(env, o, "count", n);
  set_num(env, o, "shDegree", deg);
  return o;
}

/* savePly(ctx, path, shDegree) */
static napi_value SavePly(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  char path[4096];
  uint32_t deg = 3;
  if (!get_args(env, info, 3, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_path(env, argv[1], path, sizeof path)) return NULL;
  if (!is_nullish(env, argv[2]) && !get_u32(env, argv[2], &deg)) return NULL;
  SKY_OK_OR_THROW(env, sky_save_ply(ctx, path, deg));
  return undefined(env);
}

/* saveCheckpoint(ctx, path) / loadCheckpoint(ctx, path) */
static napi_value SaveCheckpoint(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  char path[4096];
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_path(env, argv[1], path, sizeof path)) return NULL;
  SKY_OK_OR_THROW(env, sky_save_checkpoint(ctx, path));
  return undefined(env);
}

static napi_value LoadCheckpoint(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  char path[4096];
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_path(env, argv[1], path, sizeof path)) return NULL;
  SKY_OK_OR_THROW(env, sky_load_checkpoint(ctx, path));
  return undefined(env);
}

/* knnInit(ctx, sceneExtent = 0) -> Float32Array of mean neighbour distances
 * (initializeKnnAndSync, gaussian-renderer.ts:2131-2171) */
static napi_value KnnInit(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  double ext = 0.0;
  uint32_t n = 0;
  void* data = NULL;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  if (!is_nullish(env, argv[1]) && !get_f64(env, argv[1], &ext)) return NULL;
  SKY_OK_OR_THROW(env, sky_get_count(ctx, &n));
  napi_value out = new_typed(env, napi_float32_array, n, 4, &data);
  if (!out) return NULL;
  SKY_OK_OR_THROW(env, sky_knn_init(ctx, (float)ext, (float*)data));
  return out;
}

/* setCameras(ctx, [{view, proj, focal, width, height}])  (setTrainingCameras :4084) */
static napi_value SetCameras(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  uint32_t n = 0;
  bool is_array = false;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  if (napi_is_array(env, argv[1], &is_array) != napi_ok || !is_array) {
    napi_throw_type_error(env, "SKY_NAPI", "cameras must be an array");
    return NULL;
  }
  NAPI_OK(env, napi_get_array_length(env, argv[1], &n));
  SkyCamera* cams = (SkyCamera*)calloc(n ? n : 1, sizeof(SkyCamera));
  if (!cams) {
    napi_throw_error(env, "SKY_ERR_OOM", "out of host memory");
    return NULL;
  }
  for (uint32_t k = 0; k < n; ++k) {
    napi_value e;
    if (napi_get_element(env, argv[1], k, &e) != napi_ok || !read_camera(env, e, &cams[k])) {
      free(cams);
      return NULL;
    }
  }
  int rc = sky_set_cameras(ctx, cams, n);
  free(cams);
  SKY_OK_OR_THROW(env, rc);
  return undefined(env);
}

/* setTarget(ctx, camera, Float32Array(w * h * 3) rgb, width, height)
 * (setTrainingImages :4098, one image per camera) */
static napi_value SetTarget(napi_env env, napi_callback_info info) {
  napi_value argv[5];
  uint32_t cam = 0, w = 0, h = 0;
  size_t len = 0;
  if (!get_args(env, info, 5, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_u32(env, argv[1], &cam)) return NULL;
  const float* rgb = (const float*)typed(env, argv[2], napi_float32_array, &len);
  if (!rgb || !get_u32(env, argv[3], &w) || !get_u32(env, argv[4], &h)) return NULL;
  if (len < (size_t)w * h * 3) {
    napi_throw_range_error(env, "SKY_ERR_ARG", "target must hold width * height * 3 floats");
    return NULL;
  }
  SKY_OK_OR_THROW(env, sky_set_target(ctx, cam, rgb, w, h));
  return undefined(env);
}

/* ---- hot path -------------------------------------------------------------- */

static napi_value stats_object(napi_env env, const SkyStepStats* st) {
  napi_value o;
  if (napi_create_object(env, &o) != napi_ok) return NULL;
  set_num(env, o, "iteration", (double)st->iteration);
  set_num(env, o, "loss", st->loss);
  set_num(env, o, "intersections", (double)st->num_intersections);
  set_num(env, o, "gaussians", st->num_gaussians);
  set_num(env, o, "views", st->num_views);
  set_num(env, o, "shDegree", st->sh_degree);
  set_num(env, o, "shUpdated", st->sh_updated);
  return o;
}

/* Training work on a libuv worker: sky_step over given cameras, or sky_train. */
typedef struct {
  napi_async_work work;
  napi_deferred deferred;
  void* ctx;
  uint32_t cams[64];
  uint32_t ncams;
  uint32_t iterations, views_per_step;  /* train() */
  int is_train;
  int rc;
  char err[512];
  SkyStepStats st;
} TrainJob;

static void train_exec(napi_env env, void* data) {
  (void)env;
  TrainJob* j = (TrainJob*)data;
  if (j->is_train)
    j->rc = sky_train(j->ctx, j->iterations, j->views_per_step, &j->st);
  else
    j->rc = sky_step(j->ctx, j->cams, j->ncams, &j->st);
  if (j->rc != SKY_OK) {
    /* sky_last_error is per thread: copy it on the worker that failed */
    strncpy(j->err, sky_last_error(), sizeof j->err - 1);
    j->err[sizeof j->err - 1] = 0;
  }
}

static void train_done(napi_env env, napi_status status, void* data) {
  TrainJob* j = (TrainJob*)data;
  napi_value v = NULL;
  if (status != napi_ok || j->rc != SKY_OK) {
    napi_value msg, code;
    napi_create_string_utf8(env, j->rc != SKY_OK ? j->err : "async work failed", NAPI_AUTO_LENGTH, &msg);
    napi_create_string_utf8(env, status_name(j->rc), NAPI_AUTO_LENGTH, &code);
    napi_create_error(env, code, msg, &v);
    napi_reject_deferred(env, j->deferred, v);
  } else {
    v = stats_object(env, &j->st);
    napi_resolve_deferred(env, j->deferred, v);
  }
  napi_delete_async_work(env, j->work);
  free(j);
}

static napi_value queue_job(napi_env env, TrainJob* j, const char* name) {
  napi_value promise, nm;
  if (napi_create_promise(env, &j->deferred, &promise) != napi_ok ||
      napi_create_string_utf8(env, name, NAPI_AUTO_LENGTH, &nm) != napi_ok ||
      napi_create_async_work(env, NULL, nm, train_exec, train_done, j, &j->work) != napi_ok ||
      napi_queue_async_work(env, j->work) != napi_ok) {
    free(j);
    napi_throw_error(env, "SKY_NAPI", "could not queue the training work");
    return NULL;
  }
  return promise;
}

/* step(ctx, Uint32Array cameras) -> Promise<stats>  (trainStep :3638-3660, batched) */
static napi_value Step(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  size_t len = 0;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  const uint32_t* cams = (const uint32_t*)typed(env, argv[1], napi_uint32_array, &len);
  if (!cams) return NULL;
  if (len == 0 || len > 64) {
    napi_throw_range_error(env, "SKY_ERR_ARG", "a step takes 1 to 64 cameras");
    return NULL;
  }
  TrainJob* j = (TrainJob*)calloc(1, sizeof(TrainJob));
  if (!j) {
    napi_throw_error(env, "SKY_ERR_OOM", "out of host memory");
    return NULL;
  }
  j->ctx = ctx;
  j->ncams = (uint32_t)len;
  memcpy(j->cams, cams, len * sizeof(uint32_t));
  return queue_job(env, j, "sky_step");
}

/* train(ctx, iterations, viewsPerStep = 1) -> Promise<stats of the last step>
 * (train(n) :3744-3854: seeded camera choice, the schedule if set) */
static napi_value Train(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  uint32_t it = 0, vps = 1;
  if (!get_args(env, info, 3, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_u32(env, argv[1], &it)) return NULL;
  if (!is_nullish(env, argv[2]) && !get_u32(env, argv[2], &vps)) return NULL;
  TrainJob* j = (TrainJob*)calloc(1, sizeof(TrainJob));
  if (!j) {
    napi_throw_error(env, "SKY_ERR_OOM", "out of host memory");
    return NULL;
  }
  j->ctx = ctx;
  j->is_train = 1;
  j->iterations = it;
  j->views_per_step = vps;
  return queue_job(env, j, "sky_train");
}

static int camera_list(napi_env env, napi_value v, const uint32_t** cams, uint32_t* n) {
  size_t len = 0;
  *cams = (const uint32_t*)typed(env, v, napi_uint32_array, &len);
  if (!*cams) return 0;
  *n = (uint32_t)len;
  return 1;
}

/* render(ctx, Uint32Array cameras) -> {rgba: Float32Array(4 px), alpha:
 * Float32Array(px)}, the cameras' images concatenated in the given order */
static napi_value Render(napi_env env, napi_callback_info info) {
  napi_value argv[2], o;
  const uint32_t* cams = NULL;
  uint32_t n = 0;
  uint64_t bytes = 0;
  void *rgba = NULL, *alpha = NULL;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !camera_list(env, argv[1], &cams, &n)) return NULL;
  /* render on the device, then size the host arrays from the image buffer */
  SKY_OK_OR_THROW(env, sky_render(ctx, cams, n, NULL, NULL));
  SKY_OK_OR_THROW(env, sky_read_buffer(ctx, SKY_BUF_COLOR, NULL, 0, &bytes));
  const size_t px = (size_t)(bytes / 16);
  napi_value a = new_typed(env, napi_float32_array, px * 4, 4, &rgba);
  napi_value b = new_typed(env, napi_float32_array, px, 4, &alpha);
  if (!a || !b) return NULL;
  SKY_OK_OR_THROW(env, sky_read_buffer(ctx, SKY_BUF_COLOR, rgba, (uint64_t)px * 16, &bytes));
  SKY_OK_OR_THROW(env, sky_read_buffer(ctx, SKY_BUF_ALPHA, alpha, (uint64_t)px * 4, &bytes));
  NAPI_OK(env, napi_create_object(env, &o));
  NAPI_OK(env, napi_set_named_property(env, o, "rgba", a));
  NAPI_OK(env, napi_set_named_property(env, o, "alpha", b));
  return o;
}

/* forward(ctx, Uint32Array cameras) -> loss: the op pair's forward (images
 * and the loss against the cameras' targets stay on the device) */
static napi_value Forward(napi_env env, napi_callback_info info) {
  napi_value argv[2], out;
  const uint32_t* cams = NULL;
  uint32_t n = 0;
  double loss = 0.0;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !camera_list(env, argv[1], &cams, &n)) return NULL;
  SKY_OK_OR_THROW(env, sky_forward(ctx, cams, n, &loss));
  NAPI_OK(env, napi_create_double(env, loss, &out));
  return out;
}

/* backward(ctx) -> Float32Array(59 * n): the op pair's backward, gradients of
 * the last forward's loss for every parameter plane (no Adam step) */
static napi_value Backward(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  uint32_t n = 0;
  void* data = NULL;
  if (!get_args(env, info, 1, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SKY_OK_OR_THROW(env, sky_get_count(ctx, &n));
  napi_value out = new_typed(env, napi_float32_array, (size_t)SKY_NUM_PLANES * n, 4, &data);
  if (!out) return NULL;
  SKY_OK_OR_THROW(env, sky_backward(ctx, (float*)data, n));
  return out;
}

/* ---- prune / densify / opacity reset ------------------------------------- */

/* prune(ctx, {minOpacity, maxScale, maxRemoveRatio}?, Uint8Array mask?) -> removed */
static napi_value Prune(napi_env env, napi_callback_info info) {
  napi_value argv[3], out;
  size_t len = 0;
  uint32_t n = 0, removed = 0;
  if (!get_args(env, info, 3, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyPruneParams p = {0.005f, 3.4e38f, 0.0f, 0u};
  if (!opt_float(env, argv[1], "minOpacity", &p.min_opacity) ||
      !opt_float(env, argv[1], "maxScale", &p.max_scale) ||
      !opt_float(env, argv[1], "maxRemoveRatio", &p.max_remove_ratio))
    return NULL;
  const uint8_t* mask = NULL;
  if (!is_nullish(env, argv[2])) {
    mask = (const uint8_t*)typed(env, argv[2], napi_uint8_array, &len);
    if (!mask) return NULL;
    SKY_OK_OR_THROW(env, sky_get_count(ctx, &n));
    if (len < n) {
      napi_throw_range_error(env, "SKY_ERR_ARG", "mask must hold one byte per Gaussian");
      return NULL;
    }
  }
  SKY_OK_OR_THROW(env, sky_prune(ctx, &p, mask, &removed));
  NAPI_OK(env, napi_create_uint32(env, removed, &out));
  return out;
}

/* resetOpacity(ctx, maxOpacity = 0.1)  (resetOpacity :3867) */
static napi_value ResetOpacity(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  double m = 0.1;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  if (!is_nullish(env, argv[1]) && !get_f64(env, argv[1], &m)) return NULL;
  SKY_OK_OR_THROW(env, sky_reset_opacity(ctx, (float)m));
  return undefined(env);
}

/* scoreViews(ctx, Uint32Array cameras | null) -> {importance, pruning}
 * (generateMultiViewScores :2758-2788) */
static napi_value ScoreViews(napi_env env, napi_callback_info info) {
  napi_value argv[2], o;
  const uint32_t* cams = NULL;
  uint32_t nc = 0, n = 0;
  void *imp = NULL, *pr = NULL;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  if (!is_nullish(env, argv[1]) && !camera_list(env, argv[1], &cams, &nc)) return NULL;
  SKY_OK_OR_THROW(env, sky_get_count(ctx, &n));
  napi_value a = new_typed(env, napi_uint32_array, n, 4, &imp);
  napi_value b = new_typed(env, napi_float32_array, n, 4, &pr);
  if (!a || !b) return NULL;
  SKY_OK_OR_THROW(env, sky_score_views(ctx, cams, nc, (uint32_t*)imp, (float*)pr));
  NAPI_OK(env, napi_create_object(env, &o));
  NAPI_OK(env, napi_set_named_property(env, o, "importance", a));
  NAPI_OK(env, napi_set_named_property(env, o, "pruning", b));
  return o;
}

static int read_densify(napi_env env, napi_value o, SkyDensifyParams* p) {
  return opt_float(env, o, "gradThreshold", &p->grad_threshold) &&
         opt_float(env, o, "gradAbsThreshold", &p->grad_abs_threshold) &&
         opt_float(env, o, "sizeThreshold", &p->size_threshold) &&
         opt_float(env, o, "minVisibility", &p->min_visibility) &&
         opt_float(env, o, "importanceThreshold", &p->importance_threshold) &&
         opt_float(env, o, "maxNewRatio", &p->max_new_ratio) &&
         opt_float(env, o, "pixelWidth", &p->pixel_width);
}

/* densify(ctx, overrides?) -> {cloned, split}  (performDensification :3211-3466) */
static napi_value Densify(napi_env env, napi_callback_info info) {
  napi_value argv[2], o;
  uint32_t cl = 0, sp = 0;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyDensifyParams p;
  sky_densify_default(&p);
  if (!read_densify(env, argv[1], &p)) return NULL;
  SKY_OK_OR_THROW(env, sky_densify(ctx, &p, &cl, &sp));
  NAPI_OK(env, napi_create_object(env, &o));
  set_num(env, o, "cloned", cl);
  set_num(env, o, "split", sp);
  return o;
}

/* pruneScored(ctx, overrides?) -> removed  (applyMultiViewPrune :2800-2915) */
static napi_value PruneScored(napi_env env, napi_callback_info info) {
  napi_value argv[2], out;
  uint32_t removed = 0;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyScoredPruneParams p;
  sky_scored_prune_default(&p);
  if (!opt_float(env, argv[1], "minOpacity", &p.min_opacity) ||
      !opt_float(env, argv[1], "maxScale", &p.max_scale) ||
      !opt_float(env, argv[1], "maxScreenRadius", &p.max_screen_radius) ||
      !opt_uint(env, argv[1], "useScreenSizePruning", &p.use_screen_size) ||
      !opt_float(env, argv[1], "pruneRatio", &p.prune_ratio) ||
      !opt_float(env, argv[1], "maxRatio", &p.max_ratio) ||
      !opt_uint(env, argv[1], "useLastScores", &p.use_last_scores))
    return NULL;
  SKY_OK_OR_THROW(env, sky_prune_scored(ctx, &p, &removed));
  NAPI_OK(env, napi_create_uint32(env, removed, &out));
  return out;
}

/* setSchedule(ctx, overrides? | false): the TrainingController schedule
 * (training-controller.ts:23-160) that train() runs; false disables it */
static napi_value SetSchedule(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  napi_valuetype t;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkySchedule s;
  sky_schedule_default(&s);
  s.enabled = 1;
  NAPI_OK(env, napi_typeof(env, argv[1], &t));
  if (t == napi_boolean) {
    bool on = true;
    NAPI_OK(env, napi_get_value_bool(env, argv[1], &on));
    s.enabled = on ? 1u : 0u;
  } else if (!opt_uint(env, argv[1], "densifyFrom", &s.densify_from) ||
             !opt_uint(env, argv[1], "densifyUntil", &s.densify_until) ||
             !opt_uint(env, argv[1], "densifyInterval", &s.densify_interval) ||
             !opt_uint(env, argv[1], "pruneFrom", &s.prune_from) ||
             !opt_uint(env, argv[1], "pruneUntil", &s.prune_until) ||
             !opt_uint(env, argv[1], "pruneInterval", &s.prune_interval) ||
             !opt_uint(env, argv[1], "opacityResetInterval", &s.opacity_reset_interval) ||
             !opt_float(env, argv[1], "opacityResetValue", &s.opacity_reset_value) ||
             !opt_float(env, argv[1], "minOpacity", &s.min_opacity) ||
             !opt_float(env, argv[1], "maxScreenSize", &s.max_screen_size) ||
             !opt_float(env, argv[1], "maxScaleRatio", &s.max_scale_ratio) ||
             !opt_float(env, argv[1], "maxScaleAbsolute", &s.max_scale_absolute) ||
             !opt_float(env, argv[1], "sceneExtent", &s.scene_extent) ||
             !read_densify(env, argv[1], &s.densify)) {
    return NULL;
  }
  SKY_OK_OR_THROW(env, sky_set_schedule(ctx, &s));
  return undefined(env);
}

/* ---- status, readback, profiling, viewer --------------------------------- */

/* getStatus(ctx) -> {iteration, adamSteps, numGaussians, ...} */
static napi_value GetStatus(napi_env env, napi_callback_info info) {
  napi_value argv[1], o;
  if (!get_args(env, info, 1, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyStatus st;
  SKY_OK_OR_THROW(env, sky_get_status(ctx, &st));
  NAPI_OK(env, napi_create_object(env, &o));
  set_num(env, o, "iteration", (double)st.iteration);
  set_num(env, o, "adamSteps", (double)st.adam_steps);
  set_num(env, o, "lastIntersections", (double)st.last_intersections);
  set_num(env, o, "deviceBytes", (double)st.device_bytes);
  set_num(env, o, "numGaussians", st.num_gaussians);
  set_num(env, o, "numCameras", st.num_cameras);
  set_num(env, o, "errorFlags", st.error_flags);
  set_num(env, o, "kernelLaunches", (double)st.kernel_launches);
  set_num(env, o, "graphReplays", (double)st.graph_replays);
  set_num(env, o, "sceneExtent", st.scene_extent);
  set_num(env, o, "densifyRuns", st.densify_runs);
  set_num(env, o, "pruneRuns", st.prune_runs);
  return o;
}

/* getParams(ctx) -> Float32Array(59 * n), plane-major */
static napi_value GetParams(napi_env env, napi_callback_info info) {
  napi_value argv[1];
  uint32_t n = 0;
  void* data = NULL;
  if (!get_args(env, info, 1, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SKY_OK_OR_THROW(env, sky_get_count(ctx, &n));
  napi_value out = new_typed(env, napi_float32_array, (size_t)SKY_NUM_PLANES * n, 4, &data);
  if (!out) return NULL;
  SKY_OK_OR_THROW(env, sky_get_params(ctx, (float*)data, n));
  return out;
}

/* setProfiling(ctx, level): 0 off, 1 stage times, 2 also pair counts */
static napi_value SetProfiling(napi_env env, napi_callback_info info) {
  napi_value argv[2];
  uint32_t level = 0;
  if (!get_args(env, info, 2, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx || !get_u32(env, argv[1], &level)) return NULL;
  SKY_OK_OR_THROW(env, sky_set_profiling(ctx, (int)level));
  return undefined(env);
}

/* getStageTimes(ctx) -> {steps, ms: Float64Array(SKY_NUM_STAGES)} summed */
static napi_value GetStageTimes(napi_env env, napi_callback_info info) {
  napi_value argv[1], o;
  uint64_t steps = 0;
  void* data = NULL;
  if (!get_args(env, info, 1, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  napi_value ms = new_typed(env, napi_float64_array, SKY_NUM_STAGES, 8, &data);
  if (!ms) return NULL;
  SKY_OK_OR_THROW(env, sky_get_stage_times(ctx, (double*)data, SKY_NUM_STAGES, &steps));
  NAPI_OK(env, napi_create_object(env, &o));
  set_num(env, o, "steps", (double)steps);
  NAPI_OK(env, napi_set_named_property(env, o, "ms", ms));
  return o;
}

/* frame(ctx, camera{view, proj, focal, width, height}, {gaussianScaling,
 * shDegree}?) -> Uint8Array RGBA8 of the viewer frame (frame :4111-4123) */
static napi_value Frame(napi_env env, napi_callback_info info) {
  napi_value argv[3];
  void* px = NULL;
  if (!get_args(env, info, 3, argv)) return NULL;
  void* ctx = get_ctx(env, argv[0]);
  if (!ctx) return NULL;
  SkyCamera cam;
  if (!read_camera(env, argv[1], &cam)) return NULL;
  SkyViewSettings vs;
  sky_view_settings_default(&vs);
  if (!opt_float(env, argv[2], "gaussianScaling", &vs.gaussian_scaling) ||
      !opt_uint(env, argv[2], "shDegree", &vs.sh_degree))
    return NULL;
  napi_value out = new_typed(env, napi_uint8_array, (size_t)cam.width * cam.height * 4, 1, &px);
  if (!out) return NULL;
  SKY_OK_OR_THROW(env, sky_view_render(ctx, &cam, &vs, NULL, (uint8_t*)px));
  return out;
}

#define FN(name, fn) {name, NULL, fn, NULL, NULL, NULL, napi_default, NULL}

static napi_value Init(napi_env env, napi_value exports) {
  napi_property_descriptor d[] = {
      FN("create", Create),           FN("destroy", Destroy),
      FN("getConfig", GetConfig),     FN("setConfig", SetConfig),
      FN("loadPoints", LoadPoints),   FN("loadPacked", LoadPacked),
      FN("loadPly", LoadPly),         FN("savePly", SavePly),
      FN("saveCheckpoint", SaveCheckpoint), FN("loadCheckpoint", LoadCheckpoint),
      FN("knnInit", KnnInit),         FN("setCameras", SetCameras),
      FN("setTarget", SetTarget),     FN("step", Step),
      FN("train", Train),             FN("render", Render),
      FN("forward", Forward),         FN("backward", Backward),
      FN("prune", Prune),             FN("resetOpacity", ResetOpacity),
      FN("scoreViews", ScoreViews),   FN("densify", Densify),
      FN("pruneScored", PruneScored), FN("setSchedule", SetSchedule),
      FN("getStatus", GetStatus),     FN("getParams", GetParams),
      FN("setProfiling", SetProfiling), FN("getStageTimes", GetStageTimes),
      FN("frame", Frame),
  };
  if (napi_define_properties(env, exports, sizeof d / sizeof d[0], d) != napi_ok) return NULL;
  return exports;
}

NAPI_MODULE(NODE_GYP_MODULE_NAME, Init)
