"""The C-ABI library on a host without a GPU: it loads, exports every entry
point include/skyfall.h declares, keeps the struct layouts the header
describes, and reports errors through status codes (no compute calls)."""
import ctypes as C
import re

import numpy as np
import pytest

from conftest import REPO


def header_functions():
    text = (REPO / "include" / "skyfall.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sky_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(sky):
    L = sky.lib()
    names = header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares a prototype for each of them
    assert set(names) <= set(sky._lib.PROTOTYPES)


def test_config_defaults_are_the_reference_defaults(sky):
    c = sky.default_config()
    assert c.struct_size == C.sizeof(sky._lib.SkyConfig)
    assert (c.tile_size, c.sh_degree_interval, c.sh_update_interval) == (16, 1000, 16)
    assert (c.near_plane, c.far_plane, c.radius_clip) == (np.float32(0.2), 10000.0, 512.0)
    assert c.eps2d == np.float32(0.3)
    assert (c.w_l2, c.w_l1, c.w_ssim) == (0.0, np.float32(0.8), np.float32(0.2))
    assert c.lr_means == np.float32(0.00016) and c.lr_sh == np.float32(0.0025)
    assert c.lr_opacity == np.float32(0.025) and c.lr_scale == np.float32(0.005)
    assert c.lr_rotation == np.float32(0.001)
    assert (c.beta1, c.beta2, c.adam_eps) == (np.float32(0.9), np.float32(0.999), np.float32(1e-8))


def test_config_size_is_checked_before_touching_the_device(sky):
    L = sky.lib()
    c = sky.default_config()
    c.struct_size = 12
    h = C.c_void_p()
    assert L.sky_create(C.byref(c), C.byref(h)) == sky._lib.SKY_ERR_ARG
    assert b"SkyConfig size" in L.sky_last_error()
    c = sky.default_config(tile_size=12)
    assert L.sky_create(C.byref(c), C.byref(h)) == sky._lib.SKY_ERR_ARG
    # splat-batch depths outside the compiled variants are refused up front
    for kw in (dict(fwd_batch=100), dict(fwd_batch=512), dict(bwd_batch=256), dict(bwd_batch=16)):
        c = sky.default_config(**kw)
        assert L.sky_create(C.byref(c), C.byref(h)) == sky._lib.SKY_ERR_ARG
        assert b"batch" in L.sky_last_error()
    assert sky.default_config().fwd_batch == 0 and sky.default_config().bwd_batch == 0
    # culled lists are a switch, off by default (the reference's lists)
    assert sky.default_config().tile_cull == 0
    c = sky.default_config(tile_cull=2)
    assert L.sky_create(C.byref(c), C.byref(h)) == sky._lib.SKY_ERR_ARG
    assert b"tile_cull" in L.sky_last_error()
    # batch-scaled Adam hyperparameters: a switch, off by default
    assert sky.default_config().batch_scaling == 0
    c = sky.default_config(batch_scaling=2)
    assert L.sky_create(C.byref(c), C.byref(h)) == sky._lib.SKY_ERR_ARG
    assert b"batch_scaling" in L.sky_last_error()


def test_pinhole_camera_matches_reference_projection(sky):
    from skyfall import scenes
    view = scenes.look_at((1.0, 2.0, -3.0))
    out = sky._lib.SkyCamera()
    vp = view.ctypes.data_as(C.c_void_p)
    assert sky.lib().sky_camera_pinhole(vp, 900.5, 880.25, 955.0, 530.0, 1920, 1080, C.byref(out)) == 0
    ref = scenes.pinhole(view, 900.5, 880.25, 955.0, 530.0, 1920, 1080)
    assert np.array_equal(np.ctypeslib.as_array(out.proj), ref["proj"])
    assert np.array_equal(np.ctypeslib.as_array(out.view), ref["view"])
    # row 3 of the projection is (0, 0, 1, 0): clip.w = camera-space z
    P = ref["proj"].reshape(4, 4).T
    assert np.array_equal(P[3], [0, 0, 1, 0])


def test_null_context_and_argument_errors(sky):
    L = sky.lib()
    E = sky._lib
    assert L.sky_get_count(None, None) == E.SKY_ERR_ARG
    assert L.sky_render(None, None, 0, None, None) == E.SKY_ERR_ARG
    assert L.sky_destroy(None) == 0
    assert L.sky_sort_pairs(None, None, None, None, 4, 8, None) == E.SKY_ERR_ARG
    c = sky.default_config()
    assert L.sky_get_config(None, C.byref(c)) == E.SKY_ERR_ARG
    assert L.sky_version() == 1


C_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "skyfall.h"

int main(void) {
  SkyConfig cfg;
  sky_config_default(&cfg);
  if (cfg.struct_size != sizeof(SkyConfig) || cfg.tile_size != 16) return 1;
  void* ctx = NULL;
  cfg.tile_size = 12;                       /* refused before any device call */
  if (sky_create(&cfg, &ctx) != SKY_ERR_ARG || ctx != NULL) return 2;
  if (strstr(sky_last_error(), "tile_size") == NULL) return 3;
  if (sky_get_count(NULL, NULL) != SKY_ERR_ARG) return 4;
  SkyCamera cam;
  float view[16] = {1,0,0,0, 0,1,0,0, 0,0,1,0, 0,0,3,1};
  if (sky_camera_pinhole(view, 100.0, 100.0, 32.0, 24.0, 64, 48, &cam) != SKY_OK) return 5;
  printf("%d %u %u %.3f\n", sky_version(), cam.width, cam.height, cam.proj[0]);
  return 0;
}
"""


def test_header_is_c99_and_links_from_c(sky, tmp_path):
    """include/skyfall.h compiles as C99 and a C program links and calls the
    library -- what a cgo / N-API / FFI binding does (no device calls)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    src.write_text(C_PROGRAM)
    libdir = sky._lib.LIB_PATH.parent
    exe = tmp_path / "abi"
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-pedantic", f"-I{REPO / 'include'}", str(src),
                    f"-L{libdir}", "-lskyfall", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stderr)
    ver, w, h, sx = out.stdout.split()
    assert (int(ver), int(w), int(h)) == (1, 64, 48) and float(sx) == pytest.approx(2 * 100 / 64, rel=1e-6)


NODE_DIR = REPO / "skyfall-viewer_gb300" / "node"


def test_napi_addon_type_checks_against_the_napi_declarations():
    """skyfall_addon.c compiles (syntax and types, -Wall -Wextra -Werror)
    against a declarations-only stand-in of <node_api.h> and include/skyfall.h:
    every N-API and sky_* call has the right signature.  (No Node here, so it
    is not linked or run; tests/test_addon_sequence_gpu.py makes its
    sequence of library calls on the GPU.)"""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    subprocess.run([cc, "-std=c11", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
                    f"-I{REPO / 'tests' / 'napi_decls'}", f"-I{REPO / 'include'}",
                    str(NODE_DIR / "skyfall_addon.c")], check=True)


def test_facade_calls_only_functions_the_addon_defines():
    """Every addon.<name>( the TypeScript façade makes is exported by the
    addon's Init table and declared in its .d.ts, and every sky_* entry point
    the addon calls is declared in include/skyfall.h."""
    c_src = (NODE_DIR / "skyfall_addon.c").read_text()
    exported = set(re.findall(r'FN\("([A-Za-z]+)"', c_src))
    ts = (NODE_DIR / "skyfall-renderer.ts").read_text()
    called = set(re.findall(r"\baddon\.([A-Za-z]+)\(", ts))
    dts = (NODE_DIR / "skyfall_addon.d.ts").read_text()
    declared = set(re.findall(r"^\s+([A-Za-z]+)\(ctx", dts, flags=re.M)) | {"create"}
    assert called, "the façade calls the addon"
    assert called <= exported, sorted(called - exported)
    assert exported <= declared, sorted(exported - declared)
    # the reference's GaussianRenderer training methods are all there
    for name in ("train", "stopTraining", "prune", "resetOpacity", "setTrainingCameras",
                 "setTrainingImages", "buildTrainingTiles", "initializeKnnAndSync",
                 "getTrainingParams", "setTrainingParams", "getTrainingStatus", "getGaussianCount",
                 "getLossWeights", "setLossWeights", "enableProfiling", "printProfilingReport",
                 "profiledTrainStep", "getSceneExtent", "dumpTrainingDiagnostics",
                 "setGaussianScale", "resizeViewport", "forward", "backward"):
        assert re.search(rf"^\s+(async\s+)?{name}\(", ts, flags=re.M), name
    sky_calls = set(re.findall(r"\b(sky_[a-z0-9_]+)\(", c_src))
    assert sky_calls <= set(header_functions()), sorted(sky_calls - set(header_functions()))
