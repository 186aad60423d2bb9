"""Densify and prune cycles after a long run, against oracle/densify.py.

A reduced training run (4,096 Gaussians, 4 cameras of 128x96, SH degree 0)
takes 200 steps; then one densify cycle, 100 more steps, and one scored
prune.  Each cycle is checked against the oracle from the GPU's own state at
that point (parameters, Adam moments, accumulated statistics, multi-view
scores, iteration): the candidate set (clone / split), the survivor order,
the copied planes and moments, and the prune's removal set must be identical;
sampled positions and scales of the new Gaussians (f64 libm on either side)
within 1e-6.  After 200 steps the statistics have accumulated over many
views, so the decisions are made on a trained scene rather than a fresh one.
"""
import numpy as np
import pytest

from oracle import densify as D
from skyfall import scenes

pytestmark = pytest.mark.gpu

W, H = 128, 96


def js(x):
    """The double the library uses for an f32 hyperparameter (7 digits)."""
    return float(f"{float(np.float32(x)):.7g}")


def test_densify_and_prune_cycles_after_200_steps(sky, orc):
    P = scenes.scene_uniform(4096, seed=1121)
    cams = scenes.cameras_orbit(4, 3.0, W, H)
    tgts = [scenes.target_uniform(W, H, seed=2150 + k) for k in range(4)]
    r = sky.GaussianRenderer(sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=16)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(tgts)
    losses = [r.trainStep([k % 4]).loss for k in range(200)]
    assert np.mean(losses[-8:]) < np.mean(losses[:8])       # it trains

    # ---- densify cycle ------------------------------------------------------
    g, _ = r.densifyStats()
    assert g[:, 3].max() >= 40                              # statistics of many views
    P0 = r.params()
    m1, m2 = r.moments()
    imp, _ = r.scoreViews([0, 1, 2, 3])
    it = r.getStatus().iteration
    assert it == 200
    vis = g[:, 3] >= 10
    ms = np.exp(P0[3:6].astype(np.float64)).max(axis=0)
    size = float(np.median(ms[vis]))
    # thresholds from the statistics themselves: the gradient median of the
    # small visible Gaussians (clone side) and of the large ones (split side),
    # so that the decision has both kinds
    small, large = vis & (ms <= size), vis & (ms > size)
    avg = g[small, 0] / g[small, 3]
    avg_abs = g[large, 2] / g[large, 3]
    prm = dict(grad_threshold=float(np.median(avg)) / (W / 2),
               grad_abs_threshold=float(np.median(avg_abs)) / (W / 2),
               size_threshold=size, min_visibility=10.0,
               importance_threshold=0.0, max_new_ratio=0.3, pixel_width=float(W))
    p32 = {k: float(np.float32(v)) for k, v in prm.items()}
    action = D.densify_decide(P0, g, imp, 4, js(p32["grad_threshold"]) * (W / 2),
                              js(p32["grad_abs_threshold"]) * (W / 2), p32["size_threshold"],
                              js(p32["min_visibility"]), js(p32["importance_threshold"]),
                              js(p32["max_new_ratio"]))
    assert (action == 1).sum() >= 10 and (action == 2).sum() >= 10
    NP, NM1, NM2 = D.densify_build(P0, m1, m2, action, 0x5EED, it)
    cl, sp = r.densify(**prm)
    assert (cl, sp) == (int((action == 1).sum()), int((action == 2).sum()))
    P1 = r.params()
    M1, M2 = r.moments()
    assert P1.shape == NP.shape
    surv = int((action != 2).sum())
    assert np.array_equal(P1[:, :surv], NP[:, :surv])
    assert np.array_equal(M1, NM1) and np.array_equal(M2, NM2)
    assert np.array_equal(P1[6:, surv:], NP[6:, surv:])
    np.testing.assert_allclose(P1[:6, surv:], NP[:6, surv:], rtol=1e-6, atol=1e-6)

    # ---- 100 more steps, then a scored prune ----------------------------------
    for k in range(100):
        r.trainStep([k % 4])
    _, stats = r.densifyStats()
    P2 = r.params()
    n = P2.shape[1]
    _, pr = r.scoreViews([0, 1, 2, 3])
    it = r.getStatus().iteration
    assert it == 300
    radius = float(np.median(stats[stats[:, 2] > 0, 2]))
    pprm = dict(min_opacity=0.4, max_scale=0.2, max_screen_radius=radius, use_screen_size=1,
                prune_ratio=0.5, max_ratio=0.2)
    prunable, _, keys = D.prune_keys(P2, pr, n, stats, js(0.4), js(0.2), js(radius), True,
                                     0x5EED, it)
    budget = D.prune_budget(int(prunable.sum()), n, js(0.5), js(0.2))
    order = np.argsort(keys, kind="stable")
    assert 0 < budget < prunable.sum()
    kb, ka = keys[order[budget - 1]], keys[order[budget]]
    assert ka - kb > 1e-9 * abs(ka)                          # the boundary is not a near tie
    removed = r.pruneScored(**pprm)
    assert removed == budget
    keep = np.ones(n, bool)
    keep[order[:budget]] = False
    assert np.array_equal(r.params(), P2[:, keep])
    st = r.getStatus()
    assert (st.densify_runs, st.prune_runs) == (1, 1)
    r.close()
