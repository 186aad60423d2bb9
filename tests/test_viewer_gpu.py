"""GPU parity of the headless viewer frame (sky_view_render) against the
oracle's per-quad restatement: the CUDA path blends the same splats in the
same order per pixel, so images must be identical (held to 1e-5 max abs and
checked bit for bit)."""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5


def renderer(sky, P, sh_degree=3):
    r = sky.GaussianRenderer(sh_degree=sh_degree)
    r.load_points(P)
    return r


@pytest.mark.parametrize("sh_deg,scaling,r16", [(0, 1.0, 1), (3, 1.0, 1), (3, 0.5, 0), (1, 2.0, 1)])
def test_viewer_frame_matches_oracle(sky, orc, sh_deg, scaling, r16):
    P = scenes.scene_clusters(20000, seed=1203)
    cam = scenes.cameras_orbit(3, 4.0, 320, 200)[1]
    r = renderer(sky, P)
    img = r.frame(cam, gaussian_scaling=scaling, sh_degree=sh_deg, round_params_f16=bool(r16))
    ref = orc.view_render(P, cam, scaling, sh_deg, r16)
    want = ref["rgba"].reshape(img.shape)
    assert np.max(np.abs(img - want)) <= IMG_TOL
    assert np.array_equal(img, want)
    assert (img[..., 3] > 0).mean() > 0.2          # the scene fills part of the view


def test_viewer_frame_u8_and_readback(sky, orc):
    P = scenes.scene_uniform(8192, seed=1204)
    cam = scenes.cameras_single(160, 120, 3.0)[0]
    r = renderer(sky, P, sh_degree=0)
    f32 = r.frame(cam, sh_degree=0)
    u8 = r.frame(cam, sh_degree=0, as_u8=True)
    # round(clamp(v, 0, 1) * 255), halves away from zero, product in f32
    scaled = np.clip(f32, 0.0, 1.0) * np.float32(255.0)
    want = np.floor(scaled.astype(np.float64) + 0.5).astype(np.uint8)
    assert np.array_equal(u8, want)
    back = r.read_buffer("view_rgba").reshape(f32.shape)
    assert np.array_equal(back, f32)


def test_viewer_frame_empty_and_edges(sky, orc):
    P = scenes.scene_uniform(4096, seed=1205)
    r = renderer(sky, P, sh_degree=0)
    # looking away from the scene: nothing in front of the camera
    away = scenes.camera_fov((0.0, 0.0, -3.0), 64, 48, target=(0.0, 0.0, -10.0))
    img = r.frame(away, sh_degree=0)
    ref = orc.view_render(P, away, 1.0, 0, 1)
    assert np.array_equal(img, ref["rgba"].reshape(img.shape))
    # a view whose size is not a multiple of the 16-pixel tile
    odd = scenes.camera_fov((0.2, 0.1, -2.5), 97, 61)
    img = r.frame(odd, sh_degree=0)
    ref = orc.view_render(P, odd, 1.0, 0, 1)
    assert np.array_equal(img, ref["rgba"].reshape(img.shape))
