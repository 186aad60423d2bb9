"""Batch-scaled Adam hyperparameters (SkyConfig.batch_scaling) on the GPU.

With the switch on, a training step over B views takes its Adam step with
the learning rates times sqrt(B), beta1 and beta2 raised to the power B and
the bias correction counted in views (Zhao et al. 2024, "On Scaling Up 3D
Gaussian Splatting Training"); steps of one view must not change at all.
The Adam update itself is checked bit for bit against the oracle's, given
the step's gradients and its scalars."""
import math

import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu


def js(x):
    """The double a JavaScript literal of the f32 value would give."""
    return float(str(np.float32(x)))


def case():
    P = scenes.scene_clusters(6000, seed=1007, clusters=8, center_range=1.0, cluster_sigma=0.25,
                              logscale_mean=-3.8)
    cams = scenes.cameras_orbit(3, 3.5, 128, 96)
    tgt = [scenes.target_uniform(128, 96, seed=2300 + k) for k in range(3)]
    cfg = dict(sh_degree=3, sh_degree_interval=0, sh_update_interval=1, w_l2=1.0, w_l1=0.2,
               w_ssim=0.0, tile_size=16, max_views_per_step=3)
    return P, cams, tgt, cfg


def make(sky, P, cams, tgt, **cfg):
    r = sky.GaussianRenderer(**cfg)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(tgt)
    return r


def test_one_view_steps_unchanged_by_batch_scaling(sky):
    P, cams, tgt, cfg = case()
    out = []
    for on in (0, 1):
        with make(sky, P, cams, tgt, batch_scaling=on, **cfg) as r:
            for k in range(4):
                r.trainStep([k % 3])
            out.append((r.params(), *r.moments()))
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_multi_view_step_scales_lr_and_betas(sky, orc):
    P, cams, tgt, cfg = case()
    views = [0, 1, 2]
    B = len(views)
    with make(sky, P, cams, tgt, **cfg) as r0:
        r0.trainStep(views)
        plain = r0.read_buffer("step_scalars")
    with make(sky, P, cams, tgt, batch_scaling=1, **cfg) as r:
        for step in range(2):
            r.forward(views)
            g = r.backward()
            p0 = r.params()
            m1_0, m2_0 = r.moments()
            st = r.trainStep(views)
            assert st.sh_updated == 1
            sc = r.read_buffer("step_scalars")
            lr = sc[0:5]
            b1, b2, eps, bc1, bc2 = sc[5:10]
            c = r.config
            sq = math.sqrt(B)
            # position: the schedule's rate (identical for both configurations
            # at this iteration) times sqrt(B)
            if step == 0:
                assert abs(lr[0] / plain[0] - sq) <= 1e-6 * sq
            for k, name in enumerate(("lr_scale", "lr_rotation", "lr_opacity", "lr_sh"), start=1):
                assert lr[k] == np.float32(js(getattr(c, name)) * sq)
            assert b1 == np.float32(js(c.beta1) ** B) and b2 == np.float32(js(c.beta2) ** B)
            t = B * max(1, step)  # t = max(B, views of the earlier Adam steps)
            assert bc1 == np.float32(1.0 / (1.0 - js(c.beta1) ** t))
            assert bc2 == np.float32(1.0 / math.sqrt(1.0 - js(c.beta2) ** t))
            p1 = r.params()
            m1, m2 = r.moments()
            exp_p, exp_m1, exp_m2 = p0.copy(), m1_0.copy(), m2_0.copy()
            groups = [(0, 3, lr[0]), (3, 6, lr[1]), (6, 10, lr[2]), (10, 11, lr[3]),
                      (11, p0.shape[0], lr[4])]
            for lo, hi, l in groups:
                pp = np.ascontiguousarray(exp_p[lo:hi])
                a, b = np.ascontiguousarray(exp_m1[lo:hi]), np.ascontiguousarray(exp_m2[lo:hi])
                orc.adam(pp, a, b, np.ascontiguousarray(g[lo:hi]), l, b1, b2, eps, bc1, bc2)
                exp_p[lo:hi], exp_m1[lo:hi], exp_m2[lo:hi] = pp, a, b
            assert np.array_equal(p1, exp_p)
            assert np.array_equal(m1, exp_m1) and np.array_equal(m2, exp_m2)


def test_batch_scaling_survives_a_checkpoint(sky, tmp_path):
    P, cams, tgt, cfg = case()
    path = str(tmp_path / "bs.ckpt")
    with make(sky, P, cams, tgt, batch_scaling=1, **cfg) as r:
        r.trainStep([0, 1, 2])
        r.saveCheckpoint(path)
        r.trainStep([0, 1, 2])
        want = r.read_buffer("step_scalars")
    with make(sky, P, cams, tgt, batch_scaling=1, **cfg) as r:
        r.loadCheckpoint(path)
        r.trainStep([0, 1, 2])
        assert np.array_equal(r.read_buffer("step_scalars"), want)
