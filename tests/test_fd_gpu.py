"""GPU gradients (exact adjoint, through sky_forward/sky_backward) against
FP64 central finite differences (h = 1e-4) of the oracle's f64 loss, on 256
random parameters per scene.  Tolerance: 1e-3 relative (plus a 1e-6 floor
for near-zero derivatives).  Perturbations that flip a discrete decision of
the forward (cull, tile rectangle, depth order, alpha threshold, early
termination, the sign of an L1 residual) are rejected, as a finite
difference across a jump says nothing about the derivative."""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu

REL = 1e-3
ABS = 1e-6
H = 1e-4


def fd_check(sky, orc, P, cam, tgt, deg, planes, count=256, seed=0):
    cfg = dict(sh_degree=deg, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0,
               round_params_f16=0)
    r = sky.GaussianRenderer(**cfg)
    r.load_points(P)
    r.setTrainingCameras([cam])
    r.setTrainingImages([tgt])
    r.forward([0])
    g = r.backward()
    r.close()
    s = orc.settings(w_l2=1.0, w_l1=0.2, w_ssim=0.0, round_f16=0, nthreads=8)
    P64 = P.astype(np.float64)
    rng = np.random.default_rng(seed)
    cand = [(p, i) for p in planes for i in range(P.shape[1]) if abs(g[p, i]) > 1e-4]
    picks = [cand[k] for k in rng.choice(len(cand), size=min(count, len(cand)), replace=False)]
    _, s0 = orc.loss_f64(P64, cam, s, deg, tgt)
    checked, bad = 0, []
    for p, i in picks:
        Pp, Pm = P64.copy(), P64.copy()
        Pp[p, i] += H
        Pm[p, i] -= H
        lp, sp = orc.loss_f64(Pp, cam, s, deg, tgt)
        lm, sm = orc.loss_f64(Pm, cam, s, deg, tgt)
        if not (sp == sm == s0):
            continue
        fd = (lp - lm) / (2 * H)
        checked += 1
        if abs(g[p, i] - fd) > REL * abs(fd) + ABS:
            bad.append((p, i, float(g[p, i]), fd))
    return checked, bad


def test_fd_sh0_uniform_scene(sky, orc):
    P = scenes.scene_uniform(600, seed=11)
    P[3:6] += 1.2
    cam = scenes.cameras_single(96, 96, 3.0)[0]
    tgt = scenes.target_uniform(96, 96, seed=5)
    checked, bad = fd_check(sky, orc, P, cam, tgt, 0, list(range(14)))
    assert checked >= 200, checked
    assert not bad, bad[:5]


def test_fd_sh3_clustered_scene(sky, orc):
    P = scenes.scene_clusters(800, seed=21, clusters=4, center_range=0.5, logscale_mean=-3.2,
                              sh_degree=3, sh_rest_sigma=0.3)
    cam = scenes.cameras_single(96, 96, 3.0)[0]
    tgt = scenes.target_uniform(96, 96, seed=6)
    checked, bad = fd_check(sky, orc, P, cam, tgt, 3, list(range(59)), seed=1)
    assert checked >= 200, checked
    assert not bad, bad[:5]
