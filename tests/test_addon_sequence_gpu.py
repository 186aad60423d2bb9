"""The N-API addon's sequence of C-ABI calls, made from C on the GPU.

skyfall-viewer_gb300/node/skyfall_addon.c is not compiled here (no Node),
so this test compiles a C program that makes, in order, the library calls
the addon's functions make for the TypeScript façade's training loop:
create -> load_points -> set_cameras -> set_target (per camera) -> step
(batched, then single views) -> forward -> backward -> render -> get_status
-> score_views -> densify -> prune_scored -> prune -> reset_opacity ->
set_schedule -> train -> save_ply -> load_ply -> knn_init -> destroy.  The
scene and targets come from a file the test writes; the losses, gradients
and parameters the C program reports must equal, bit for bit, those of the
same calls through the Python binding.
"""
import shutil
import subprocess

import numpy as np
import pytest

from conftest import REPO
from skyfall import scenes

pytestmark = pytest.mark.gpu

C_SEQUENCE = r"""
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "skyfall.h"

#define CK(x) do { int rc_ = (x); if (rc_ != SKY_OK) { \
  fprintf(stderr, "%s -> %d: %s\n", #x, rc_, sky_last_error()); return 10; } } while (0)

static int read_all(const char* path, void* dst, size_t bytes) {
  FILE* f = fopen(path, "rb");
  if (!f) return 0;
  size_t got = fread(dst, 1, bytes, f);
  fclose(f);
  return got == bytes;
}
static int write_all(const char* path, const void* src, size_t bytes) {
  FILE* f = fopen(path, "wb");
  if (!f) return 0;
  size_t put = fwrite(src, 1, bytes, f);
  fclose(f);
  return put == bytes;
}

int main(int argc, char** argv) {
  if (argc < 3) return 1;
  const char* dir = argv[1];
  const unsigned n = (unsigned)atoi(argv[2]);
  char path[1024];
  /* inputs: params (59 x n f32), 2 cameras, 2 targets of 160 x 120 x 3 f32 */
  float* params = malloc((size_t)59 * n * 4);
  SkyCamera cams[2];
  const unsigned W = 160, H = 120;
  float* tgt = malloc((size_t)2 * W * H * 3 * 4);
  snprintf(path, sizeof path, "%s/params.bin", dir);
  if (!read_all(path, params, (size_t)59 * n * 4)) return 2;
  snprintf(path, sizeof path, "%s/cams.bin", dir);
  if (!read_all(path, cams, sizeof cams)) return 3;
  snprintf(path, sizeof path, "%s/targets.bin", dir);
  if (!read_all(path, tgt, (size_t)2 * W * H * 3 * 4)) return 4;

  SkyConfig cfg;                                  /* create({shDegree: 3, ...}) */
  sky_config_default(&cfg);
  cfg.sh_degree = 3; cfg.sh_degree_interval = 0; cfg.w_l2 = 1.0f; cfg.w_l1 = 0.2f; cfg.w_ssim = 0.0f;
  cfg.use_graph = 1; cfg.max_views_per_step = 2;
  void* ctx = NULL;
  CK(sky_create(&cfg, &ctx));
  CK(sky_load_points(ctx, params, n, n));         /* loadPoints */
  CK(sky_set_cameras(ctx, cams, 2));              /* setCameras */
  for (unsigned k = 0; k < 2; ++k)                /* setTarget per camera */
    CK(sky_set_target(ctx, k, tgt + (size_t)k * W * H * 3, W, H));
  SkyStepStats st[4];
  const unsigned both[2] = {0, 1}, one[1] = {1};
  CK(sky_step(ctx, both, 2, &st[0]));             /* step (batched) */
  CK(sky_step(ctx, both, 2, &st[1]));             /* step (graph replay) */
  CK(sky_step(ctx, one, 1, &st[2]));              /* step (one view) */
  double loss = 0.0;
  CK(sky_forward(ctx, both, 2, &loss));           /* forward */
  float* grads = malloc((size_t)59 * n * 4);
  CK(sky_backward(ctx, grads, n));                /* backward */
  uint64_t bytes = 0;
  CK(sky_render(ctx, both, 2, NULL, NULL));       /* render */
  CK(sky_read_buffer(ctx, SKY_BUF_COLOR, NULL, 0, &bytes));
  float* rgba = malloc(bytes);
  CK(sky_read_buffer(ctx, SKY_BUF_COLOR, rgba, bytes, &bytes));
  SkyStatus s0;
  CK(sky_get_status(ctx, &s0));                   /* getStatus */
  float* after = malloc((size_t)59 * n * 4);
  CK(sky_get_params(ctx, after, n));              /* getParams */
  unsigned* imp = malloc((size_t)n * 4);
  float* pr = malloc((size_t)n * 4);
  CK(sky_score_views(ctx, both, 2, imp, pr));     /* scoreViews */
  SkyDensifyParams dp; sky_densify_default(&dp);
  dp.min_visibility = 1.0f; dp.importance_threshold = 0.0f;
  unsigned cl = 0, sp = 0, removed = 0, removed2 = 0;
  CK(sky_densify(ctx, &dp, &cl, &sp));            /* densify */
  SkyScoredPruneParams pp; sky_scored_prune_default(&pp);
  CK(sky_prune_scored(ctx, &pp, &removed));       /* pruneScored */
  SkyPruneParams rp = {0.05f, 3.4e38f, 0.0f, 0u};
  CK(sky_prune(ctx, &rp, NULL, &removed2));       /* prune */
  CK(sky_reset_opacity(ctx, 0.1f));               /* resetOpacity */
  SkySchedule sch; sky_schedule_default(&sch);
  sch.enabled = 1; sch.densify_from = 1; sch.densify_interval = 2; sch.prune_from = 1;
  sch.prune_interval = 3;
  CK(sky_set_schedule(ctx, &sch));                /* setSchedule */
  CK(sky_train(ctx, 4, 1, &st[3]));               /* train */
  snprintf(path, sizeof path, "%s/scene.ply", dir);
  CK(sky_save_ply(ctx, path, 3));                 /* savePly */
  unsigned n2 = 0, d2 = 0, n3 = 0;
  CK(sky_load_ply(ctx, path, &n2, &d2));          /* loadPly */
  CK(sky_get_count(ctx, &n3));
  float* dens = malloc((size_t)n3 * 4);
  CK(sky_knn_init(ctx, 0.0f, dens));              /* knnInit */
  CK(sky_destroy(ctx));                           /* destroy */
  snprintf(path, sizeof path, "%s/grads.bin", dir);
  if (!write_all(path, grads, (size_t)59 * n * 4)) return 5;
  snprintf(path, sizeof path, "%s/after.bin", dir);
  if (!write_all(path, after, (size_t)59 * n * 4)) return 6;
  snprintf(path, sizeof path, "%s/rgba.bin", dir);
  if (!write_all(path, rgba, bytes)) return 7;
  printf("{\"loss\": [%.17g, %.17g, %.17g], \"fwd_loss\": %.17g, \"it3\": %llu, \"replays\": %llu, "
         "\"cloned\": %u, \"split\": %u, \"removed\": %u, \"removed2\": %u, \"ply_n\": %u, \"ply_deg\": %u, "
         "\"train_it\": %llu, \"rgba_bytes\": %llu, \"dens0\": %.9g}\n",
         st[0].loss, st[1].loss, st[2].loss, loss, (unsigned long long)st[2].iteration,
         (unsigned long long)s0.graph_replays, cl, sp, removed, removed2, n2, d2,
         (unsigned long long)st[3].iteration, (unsigned long long)bytes, n3 ? dens[0] : 0.0f);
  return 0;
}
"""


def test_addon_call_sequence_from_c_matches_python(sky, tmp_path):
    import json
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    n = 6000
    P = scenes.scene_clusters(n, seed=1401, clusters=8, center_range=1.0, cluster_sigma=0.25,
                              logscale_mean=-3.6)
    cams = scenes.cameras_orbit(2, 3.5, 160, 120)
    tgts = [scenes.target_uniform(160, 120, seed=2400 + k) for k in range(2)]
    P.astype(np.float32).tofile(tmp_path / "params.bin")
    camarr = (sky._lib.SkyCamera * 2)(*[sky.renderer.to_sky_camera(c) for c in cams])
    (tmp_path / "cams.bin").write_bytes(bytes(camarr))
    np.concatenate([t.reshape(-1) for t in tgts]).astype(np.float32).tofile(tmp_path / "targets.bin")
    src = tmp_path / "seq.c"
    src.write_text(C_SEQUENCE)
    libdir = sky._lib.LIB_PATH.parent
    exe = tmp_path / "seq"
    subprocess.run([cc, "-std=c99", "-O1", "-Wall", "-Werror", f"-I{REPO / 'include'}", str(src),
                    f"-L{libdir}", "-lskyfall", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path), str(n)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    res = json.loads(out.stdout.strip().splitlines()[-1])

    # the same calls through the Python binding
    r = sky.GaussianRenderer(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0,
                             use_graph=1, max_views_per_step=2)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(tgts)
    losses = [r.trainStep([0, 1]).loss, r.trainStep([0, 1]).loss, r.trainStep([1]).loss]
    fwd = r.forward([0, 1])
    g = r.backward()
    rgba, _ = r.render([0, 1])
    after = r.params()
    r.close()
    assert res["loss"] == losses and res["fwd_loss"] == fwd
    assert res["it3"] == 3 and res["replays"] >= 1
    assert np.array_equal(np.fromfile(tmp_path / "grads.bin", np.float32).reshape(59, n).view(np.uint32),
                          g.view(np.uint32))
    assert np.array_equal(np.fromfile(tmp_path / "after.bin", np.float32).reshape(59, n).view(np.uint32),
                          after.view(np.uint32))
    assert np.array_equal(np.fromfile(tmp_path / "rgba.bin", np.float32).reshape(-1, 4), rgba)
    assert res["rgba_bytes"] == 2 * 160 * 120 * 16
    # the rest of the sequence ran and left a consistent scene
    assert res["ply_deg"] == 3 and res["ply_n"] > 0 and res["train_it"] >= 4
    assert res["dens0"] > 0.0
