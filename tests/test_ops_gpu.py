"""GPU checks of the remaining entry points: the SSIM loss term, prune
compaction (order-preserving survivors of parameters and Adam moments),
opacity reset, loading the reference's packed f16 buffers, the train loop,
tile sizes 8 and 32, and error reporting."""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu


def make(sky, P, cams, targets, **cfg):
    r = sky.GaussianRenderer(**cfg)
    r.load_points(P)
    r.setTrainingCameras(cams)
    if targets is not None:
        r.setTrainingImages(targets)
    return r


def test_ssim_loss_term_matches_oracle(sky, orc):
    P = scenes.scene_uniform(8192, seed=31)
    cams = scenes.cameras_single(128, 96, 3.0)
    tgt = [scenes.target_uniform(128, 96, seed=32)]
    cfg = dict(sh_degree=0, w_l2=0.0, w_l1=0.8, w_ssim=0.2)
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([0])
    s = orc.settings(w_l2=0.0, w_l1=0.8, w_ssim=0.2)
    ref = orc.view_pipeline(P, cams[0], tgt[0], s, 0, mode=0)
    res = r.read_buffer("residual").reshape(-1, 4)
    assert np.array_equal(res, ref["ls"]["residual"])


@pytest.mark.parametrize("ts", [8, 32])
def test_tile_sizes_render_bit_exact(sky, orc, ts):
    P = scenes.scene_uniform(8192, seed=33)
    cams = scenes.cameras_single(200, 150, 3.0)
    tgt = [scenes.target_uniform(200, 150, seed=34)]
    r = make(sky, P, cams, tgt, sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=ts)
    r.forward([0])
    g = r.backward()
    s = orc.settings(tile_size=ts, w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    ref = orc.view_pipeline(P, cams[0], tgt[0], s, 0, mode=0)
    assert np.array_equal(r.read_buffer("tile_offsets"), ref["tl"]["offsets"])
    assert np.array_equal(r.read_buffer("color").reshape(-1, 4), ref["fw"]["rgba"])
    g_ref = orc.geom(P, cams[0], s, 0, ref["bw"]["gsum9"].astype(np.float32))
    scale = np.abs(g_ref[:14]).max()
    assert np.all(np.abs(g[:14] - g_ref[:14]) <= 1e-3 * np.abs(g_ref[:14]) + 1e-4 * scale)


def test_prune_with_mask_keeps_survivors_in_order(sky):
    P = scenes.scene_uniform(10000, seed=35)
    cams = scenes.cameras_single(64, 64, 3.0)
    tgt = [scenes.target_uniform(64, 64, seed=36)]
    r = make(sky, P, cams, tgt, sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    for _ in range(3):
        r.trainStep([0])
    p0 = r.params()
    m10, m20 = r.moments()
    mask = np.random.default_rng(0).random(10000) < 0.3
    n = r.prune(mask=mask.astype(np.uint8))
    assert n == int((~mask).sum())
    assert np.array_equal(r.params(), p0[:, ~mask])
    m1, m2 = r.moments()
    assert np.array_equal(m1, m10[:, ~mask]) and np.array_equal(m2, m20[:, ~mask])
    st = r.trainStep([0])          # training continues on the compacted set
    assert st.num_gaussians == n


def test_prune_rule_opacity_and_scale(sky):
    P = scenes.scene_uniform(20000, seed=37)
    P[10] = scenes.f16(np.random.default_rng(1).normal(-4.0, 2.0, 20000))
    P[3] = scenes.f16(np.random.default_rng(2).normal(-4.0, 1.5, 20000))
    r = make(sky, P, scenes.cameras_single(), None, sh_degree=0)
    op = 1.0 / (1.0 + np.exp(-P[10].astype(np.float64)))
    ms = np.exp(P[3:6].astype(np.float64)).max(axis=0)
    prunable = (op < 0.005) | (ms > 0.05)
    assert 0 < prunable.sum() < 20000
    n = r.prune(minOpacity=0.005, maxScale=0.05)
    assert n == int((~prunable).sum())
    assert np.array_equal(r.params(), P[:, ~prunable])


def test_prune_never_removes_everything(sky):
    P = scenes.scene_uniform(1000, seed=38)
    r = make(sky, P, scenes.cameras_single(), None, sh_degree=0)
    assert r.prune(mask=np.ones(1000, np.uint8)) == 1000
    assert r.prune(mask=np.zeros(1000, np.uint8)) == 1000


def test_reset_opacity_caps_logits(sky):
    P = scenes.scene_uniform(5000, seed=39)
    r = make(sky, P, scenes.cameras_single(), None, sh_degree=0)
    r.resetOpacity(0.1)
    cap = np.float32(np.log(0.1 / 0.9))
    expect = P.copy()
    expect[10] = np.where(P[10] > cap, cap, P[10])
    assert np.array_equal(r.params(), expect)


def test_load_packed_reference_layout(sky):
    P = scenes.scene_clusters(3000, seed=40)
    n = P.shape[1]
    h = np.zeros((n, 12), np.float16)
    h[:, 0:3] = P[0:3].T
    h[:, 3] = P[10]
    h[:, 4] = P[9]               # rot0 = w
    h[:, 5:8] = P[6:9].T         # rot1..rot3 = x, y, z
    h[:, 8:11] = P[3:6].T
    sh = np.ascontiguousarray(P[11:59].T.astype(np.float16))
    r = sky.GaussianRenderer(sh_degree=3)
    r.load_packed(np.ascontiguousarray(h).view(np.uint32), sh.view(np.uint32))
    assert np.array_equal(r.params(), P)


def test_train_loop_is_seeded_and_reduces_loss(sky):
    P = scenes.scene_uniform(16384, seed=41)
    cams = scenes.cameras_orbit(4, 3.5, 128, 128)
    tgt = [scenes.target_uniform(128, 128, seed=42 + k) * 0.2 for k in range(4)]
    losses = []
    for _ in range(2):
        r = make(sky, P, cams, tgt, sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, seed=99)
        first = r.forward([0, 1, 2, 3])
        r.train(60)
        losses.append((first, r.forward([0, 1, 2, 3]), r.params()))
        assert r.getTrainingStatus().currentIteration == 60
        r.close()
    assert losses[0][1] < losses[0][0]
    assert losses[0][1] == losses[1][1]
    assert np.array_equal(losses[0][2], losses[1][2])


def test_errors_are_reported(sky):
    r = sky.GaussianRenderer()
    with pytest.raises(sky.SkyError) as e:
        r.trainStep([0])
    assert e.value.code == sky._lib.SKY_ERR_STATE
    r.load_points(scenes.scene_uniform(100))
    with pytest.raises(sky.SkyError) as e:
        r.trainStep([0])
    assert e.value.code == sky._lib.SKY_ERR_ARG
    r.setTrainingCameras(scenes.cameras_single(32, 32))
    with pytest.raises(sky.SkyError) as e:
        r.forward([0])                # no target image
    assert e.value.code == sky._lib.SKY_ERR_STATE
    with pytest.raises(sky.SkyError):
        r.setTrainingImage(0, np.zeros((16, 16, 3), np.float32))


def test_tile_size_autotuner(sky):
    from skyfall import scenes
    from skyfall.autotune import pick_tile_size
    P = scenes.scene_uniform(4096, seed=1501)
    cams = scenes.cameras_orbit(4, 3.0, 160, 120)
    tgts = [scenes.target_uniform(160, 120, seed=2500 + k) for k in range(4)]

    def make(ts):
        r = sky.GaussianRenderer(sh_degree=0, tile_size=ts, use_graph=1, w_ssim=0.0)
        r.load_points(P)
        r.setTrainingCameras(cams)
        r.setTrainingImages(tgts)
        return r

    best, times = pick_tile_size(make, [[0, 1, 2, 3]] * 3)
    assert best in (8, 16, 32) and set(times) == {8, 16, 32}
    assert all(t > 0 for t in times.values()) and times[best] == min(times.values())
    from skyfall.autotune import autotune
    ts, fb, bb, tt = autotune(make, [[0, 1, 2, 3]] * 3)
    assert ts in (8, 16, 32) and fb in (64, 128, 256)
    assert set(tt["fwd_batch"]) == {64, 128, 256} and tt["fwd_batch"][fb] == min(tt["fwd_batch"].values())
    if ts == 16:
        assert bb in (32, 64, 128) and tt["bwd_batch"][bb] == min(tt["bwd_batch"].values())
    else:
        assert bb == 0 and tt["bwd_batch"] == {}


def test_views_with_nothing_in_front(sky, orc):
    """A view that sees no Gaussian: its items have no tiles, its sort-group
    segment or its share of one is empty.  Batched with a normal view it
    renders the background and adds nothing to the gradients; a step of empty
    views only gives zero gradients; the graph path runs such steps too."""
    P = scenes.scene_uniform(8192, seed=37)
    normal = scenes.cameras_single(64, 64, 3.0)[0]
    away = scenes.camera_fov((0.0, 0.0, -3.0), 64, 64, target=(0.0, 0.0, -10.0))
    cams = [away, normal]
    tgt = [scenes.target_uniform(64, 64, seed=38), scenes.target_uniform(64, 64, seed=39)]
    cfg = dict(sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([1])
    g_normal = r.backward()
    loss = r.forward([0, 1])
    g_both = r.backward()
    assert np.array_equal(g_both, g_normal)
    rgba = r.read_buffer("color").reshape(-1, 4)
    assert not rgba[:64 * 64, :3].any() and not r.read_buffer("alpha")[:64 * 64].any()
    s = orc.settings(w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    ref = orc.view_pipeline(P, normal, tgt[1], s, 0, mode=0)
    assert np.array_equal(rgba[64 * 64:], ref["fw"]["rgba"])
    r.forward([0, 0])
    assert not r.backward().any()
    assert r.read_buffer("counts").sum() == 0
    r.close()
    r = make(sky, P, cams, tgt, use_graph=1, **cfg)
    for views in ([0, 1], [0, 1], [0, 0], [1, 0]):
        st = r.trainStep(views)
        assert np.isfinite(st.loss)
    assert np.all(np.isfinite(r.params()))


def test_splat_batch_depths_change_no_result(sky):
    """Every forward depth gives the same images, alphas, last indices and
    loss, every backward depth the same gradients, bit for bit (the batch
    only sets how many splats are staged at once)."""
    from skyfall import scenes
    P = scenes.scene_clusters(20000, seed=1601, clusters=16, center_range=1.0, cluster_sigma=0.25,
                              logscale_mean=-3.8)
    cams = scenes.cameras_orbit(2, 3.5, 240, 176)
    tgts = [scenes.target_uniform(240, 176, seed=2600 + k) for k in range(2)]
    r = make(sky, P, cams, tgts, sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2,
             w_ssim=0.0, tile_size=16)
    ref = None
    for fb, bb in [(0, 0), (64, 32), (128, 64), (256, 128), (64, 128)]:
        r.setBatchDepth(fb, bb)
        got = r.getConfig()
        assert (got.fwd_batch, got.bwd_batch, got.tile_size) == (fb, bb, 16)
        loss = r.forward([0, 1])
        out = (loss, r.read_buffer("color"), r.read_buffer("alpha"), r.read_buffer("last_ids"),
               r.backward())
        if ref is None:
            ref = out
            continue
        assert out[0] == ref[0]
        for a, b in zip(out[1:], ref[1:]):
            assert np.array_equal(a, b)
    # and on the graph-captured training path, a changed depth re-captures
    r.close()
    r = make(sky, P, cams, tgts, sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2,
             w_ssim=0.0, tile_size=16, use_graph=1)
    for fb, bb in [(0, 0), (0, 0), (64, 32), (64, 32)]:
        r.setBatchDepth(fb, bb)
        r.trainStep([0, 1])
    st = r.getStatus()
    # step 1 runs directly, step 2 captures, step 3 re-captures, step 4 replays
    assert st.graph_captures == 2 and st.graph_replays == 3
