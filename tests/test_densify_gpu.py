"""GPU parity of the densification path through the C-ABI against the
oracle (oracle/densify.py): per-step statistics, multi-view scores, the
clone/split decision and construction, the weighted prune, and the training
schedule (deterministic, graph replay identical to direct launches).

Integer results (importance statistics, error-pixel hits, candidate and
survivor sets, counts) must be identical.  Floating-point results carry the
tolerance written beside each check."""
import math

import numpy as np
import pytest

from oracle import densify as D
from skyfall import scenes

pytestmark = pytest.mark.gpu

W, H = 128, 96
CFG = dict(sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=16)


def js(x):
    """The double the library uses for an f32 hyperparameter (7 digits)."""
    return float(f"{float(np.float32(x)):.7g}")


def case(n=4096, ncam=3):
    P = scenes.scene_uniform(n, seed=1101)
    cams = scenes.cameras_orbit(ncam, 3.0, W, H)
    tgts = [scenes.target_uniform(W, H, seed=2100 + k) for k in range(ncam)]
    return P, cams, tgts


def make(sky, P, cams, tgts, **extra):
    r = sky.GaussianRenderer(**{**CFG, **extra})
    r.load_points(P)
    r.setTrainingCameras(cams)
    if tgts is not None:
        r.setTrainingImages(tgts)
    return r


def settings(orc):
    return orc.settings(tile_size=16, w_l2=CFG["w_l2"], w_l1=CFG["w_l1"], w_ssim=0.0, round_f16=1)


def oracle_scores(orc, P, cams, tgts, views):
    s = settings(orc)
    out = []
    for v in views:
        ref = orc.view_pipeline(P, cams[v], None, s, 0)
        out.append(D.metric_view(ref["fw"]["rgba"], tgts[v], ref["fw"]["last"], ref["tl"]["offsets"],
                                 ref["tl"]["gidx_sorted"], ref["pr"]["rec"], W, H, 16, P.shape[1]))
    return D.combine_scores(out)


def test_step_statistics(sky, orc):
    P, cams, tgts = case()
    n = P.shape[1]
    r = make(sky, P, cams, tgts)
    r.trainStep([0])
    g, imp = r.densifyStats()
    ref = orc.view_pipeline(P, cams[0], tgts[0], settings(orc), 0, mode=0)
    want_imp = D.importance_update(np.zeros((n, 4), np.float32), ref["pr"]["counts"],
                                   ref["pr"]["rec"][:, 10])
    assert np.array_equal(imp, want_imp)
    want_acc = D.densify_accum_update(np.zeros((n, 4)), ref["bw"]["gsum9"])
    assert np.array_equal(g[:, 3], want_acc[:, 3])
    assert not g[:, 1].any()
    # per-Gaussian f32 sums of partials vs the oracle's f64 sums
    np.testing.assert_allclose(g[:, [0, 2]], want_acc[:, [0, 2]], rtol=1e-4, atol=1e-7)
    # a batched step applies the per-view updates in view order
    r.trainStep([1, 2])
    _, imp2 = r.densifyStats()
    counts = r.read_buffer("counts")
    radius = r.read_buffer("depth_radius").reshape(-1, 2)[:, 1]
    want = imp
    for v in range(2):
        want = D.importance_update(want, counts[v * n:(v + 1) * n], radius[v * n:(v + 1) * n])
    assert np.array_equal(imp2, want)


def test_multiview_scores(sky, orc):
    P, cams, tgts = case()
    r = make(sky, P, cams, tgts)
    imp, pr = r.scoreViews([0, 1, 2])
    want_imp, want_pr = oracle_scores(orc, P, cams, tgts, [0, 1, 2])
    assert imp.sum() > 0
    assert np.array_equal(imp, want_imp)
    # the mean L1 is an f64 sum in another order: 1e-6 relative
    np.testing.assert_allclose(pr, want_pr, rtol=1e-6, atol=1e-12)
    # no camera list: all cameras in order when there are at most 10
    imp_all, _ = r.scoreViews(None)
    assert np.array_equal(imp_all, want_imp)
    assert r.getStatus().scored_views == 3


def test_scores_need_targets(sky):
    P, cams, _ = case()
    r = make(sky, P, cams, None)
    with pytest.raises(sky.SkyError):
        r.scoreViews([0])
    # densify without any scored view: nothing changes
    assert r.densify(min_visibility=1.0, importance_threshold=0.0) == (0, 0)
    assert r.getGaussianCount() == P.shape[1]


def trained(sky, P, cams, tgts, steps=3):
    r = make(sky, P, cams, tgts)
    for k in range(steps):
        r.trainStep([k % len(cams)])
    return r


def test_densify_matches_oracle(sky, orc):
    P, cams, tgts = case()
    r = trained(sky, P, cams, tgts)
    g, _ = r.densifyStats()
    P0 = r.params()
    m1, m2 = r.moments()
    imp, _ = r.scoreViews([0, 1, 2])
    it = r.getStatus().iteration
    vis = g[:, 3] > 0
    avg = g[vis, 0] / g[vis, 3]
    avg_abs = g[vis, 2] / g[vis, 3]
    ms = np.exp(P0[3:6].astype(np.float64)).max(axis=0)
    prm = dict(grad_threshold=float(np.quantile(avg, 0.6)) / (W / 2),
               grad_abs_threshold=float(np.quantile(avg_abs, 0.6)) / (W / 2),
               size_threshold=float(np.median(ms)), min_visibility=1.0,
               importance_threshold=0.5, max_new_ratio=0.05, pixel_width=float(W))
    p32 = {k: float(np.float32(v)) for k, v in prm.items()}
    action = D.densify_decide(P0, g, imp, 3, js(p32["grad_threshold"]) * (W / 2),
                              js(p32["grad_abs_threshold"]) * (W / 2), p32["size_threshold"],
                              js(p32["min_visibility"]), js(p32["importance_threshold"]),
                              js(p32["max_new_ratio"]))
    assert (action == 1).any() and (action == 2).any()
    NP, NM1, NM2 = D.densify_build(P0, m1, m2, action, 0x5EED, it)
    cl, sp = r.densify(**prm)
    assert (cl, sp) == (int((action == 1).sum()), int((action == 2).sum()))
    n1 = r.getGaussianCount()
    assert n1 == NP.shape[1]
    P1 = r.params()
    M1, M2 = r.moments()
    surv = int((action != 2).sum())
    assert np.array_equal(P1[:, :surv], NP[:, :surv])
    assert np.array_equal(M1, NM1) and np.array_equal(M2, NM2)
    # new Gaussians: copied planes identical; sampled position / scale from
    # f64 libm on either side, 1e-6
    assert np.array_equal(P1[6:, surv:], NP[6:, surv:])
    np.testing.assert_allclose(P1[:6, surv:], NP[:6, surv:], rtol=1e-6, atol=1e-6)
    g1, i1 = r.densifyStats()
    assert not g1.any() and not i1.any()
    assert r.getStatus().densify_runs == 1
    # the scene keeps training
    st = r.trainStep([0])
    assert st.num_gaussians == n1 and np.isfinite(st.loss)


def test_prune_scored_matches_oracle(sky, orc):
    P, cams, tgts = case()
    r = trained(sky, P, cams, tgts)
    _, stats = r.densifyStats()
    P0 = r.params()
    n = P0.shape[1]
    _, pr = r.scoreViews([0, 1, 2])
    it = r.getStatus().iteration
    radius = float(np.median(stats[stats[:, 2] > 0, 2]))
    prm = dict(min_opacity=0.5, max_scale=0.2, max_screen_radius=radius, use_screen_size=1,
               prune_ratio=0.5, max_ratio=0.2)
    prunable, _, keys = D.prune_keys(P0, pr, n, stats, js(0.5), js(0.2), js(radius), True,
                                     0x5EED, it)
    budget = D.prune_budget(int(prunable.sum()), n, js(0.5), js(0.2))
    order = np.argsort(keys, kind="stable")
    assert 0 < budget < prunable.sum()
    # the boundary is not a near tie
    kb, ka = keys[order[budget - 1]], keys[order[budget]]
    assert ka - kb > 1e-9 * abs(ka)
    removed = r.pruneScored(**prm)
    assert removed == budget
    keep = np.ones(n, bool)
    keep[order[:budget]] = False
    assert np.array_equal(r.params(), P0[:, keep])
    assert r.getStatus().prune_runs == 1


def schedule_run(sky, P, cams, tgts, use_graph):
    r = make(sky, P, cams, tgts, use_graph=use_graph)
    r.setSchedule(densify_from=2, densify_until=100, densify_interval=3, prune_from=2,
                  prune_until=100, prune_interval=2, opacity_reset_interval=5, min_opacity=0.4,
                  densify=dict(min_visibility=1.0, importance_threshold=0.0,
                               grad_threshold=1e-6, grad_abs_threshold=1e-6))
    r.train(11)
    return r


def test_schedule_graph_matches_direct(sky):
    P, cams, tgts = case(n=2048)
    a = schedule_run(sky, P, cams, tgts, 0)
    b = schedule_run(sky, P, cams, tgts, 1)
    sa, sb = a.getStatus(), b.getStatus()
    assert sa.densify_runs >= 2 and sa.prune_runs >= 1
    assert sa.num_gaussians != P.shape[1]
    assert sb.graph_replays > 0
    assert (sa.num_gaussians, sa.densify_runs, sa.prune_runs) == \
        (sb.num_gaussians, sb.densify_runs, sb.prune_runs)
    assert np.array_equal(a.params(), b.params())
    # opacity reset at iteration 5 and 10: logits clamped to logit(0.01)
    c = schedule_run(sky, P, cams, tgts, 0)
    assert np.array_equal(c.params(), a.params())
