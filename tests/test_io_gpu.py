"""Scene files and training checkpoints through a live context: a PLY
written by sky_save_ply loads back as the f16-rounded parameters, and
training resumed from a checkpoint continues bit for bit."""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu


def f16(a):
    return a.astype(np.float32).astype(np.float16).astype(np.float32)


def test_ply_round_trip(sky, tmp_path):
    P = scenes.scene_clusters(5000, seed=1301)
    r = sky.GaussianRenderer(sh_degree=3)
    r.load_points(P)
    path = tmp_path / "scene.ply"
    r.savePly(path, 3)
    q = sky.GaussianRenderer(sh_degree=3)
    n, deg = q.loadPly(path)
    assert (n, deg) == (P.shape[1], 3)
    assert np.array_equal(q.params(), f16(P))
    host, hdeg, ext = sky._lib.read_ply(path)
    assert np.array_equal(host, q.params())
    assert q.getStatus().scene_extent == pytest.approx(
        float(max(P[k].max() - P[k].min() for k in range(3))), rel=1e-6)
    # a degree-1 export keeps the first four coefficients
    r.savePly(tmp_path / "d1.ply", 1)
    host1, d1, _ = sky._lib.read_ply(tmp_path / "d1.ply")
    assert d1 == 1
    assert np.array_equal(host1[:11 + 12], f16(P[:11 + 12]))
    assert not host1[11 + 12:].any()


def setup(sky, P, cams, tgts):
    r = sky.GaussianRenderer(sh_degree=1, w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(tgts)
    return r


def test_checkpoint_resume_is_bit_exact(sky, tmp_path):
    P = scenes.scene_uniform(4096, seed=1302)
    cams = scenes.cameras_orbit(4, 3.0, 96, 80)
    tgts = [scenes.target_uniform(96, 80, seed=2300 + k) for k in range(4)]
    a = setup(sky, P, cams, tgts)
    a.train(5)
    ck = tmp_path / "a.ckpt"
    a.saveCheckpoint(ck)
    a.train(5)
    b = setup(sky, P, cams, tgts)
    b.loadCheckpoint(ck)
    assert b.getStatus().iteration == 5
    b.train(5)
    sa, sb = a.getStatus(), b.getStatus()
    assert (sa.iteration, sa.adam_steps) == (sb.iteration, sb.adam_steps) == (10, 10)
    assert np.array_equal(a.params(), b.params())
    ma, mb = a.moments(), b.moments()
    assert np.array_equal(ma[0], mb[0]) and np.array_equal(ma[1], mb[1])
    ga, ia = a.densifyStats()
    gb, ib = b.densifyStats()
    assert np.array_equal(ga, gb) and np.array_equal(ia, ib)


def test_checkpoint_rejects_other_files(sky, tmp_path):
    bad = tmp_path / "bad.ckpt"
    bad.write_bytes(b"not a checkpoint at all")
    r = sky.GaussianRenderer()
    with pytest.raises(sky.SkyError):
        r.loadCheckpoint(bad)
