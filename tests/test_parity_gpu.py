"""GPU parity of the full hot path, through the C-ABI, against the oracle.

Small single-view workload (16,384 Gaussians, 256x256, SH degree 0, the
plain-step configuration) and a clustered SH-3 scene with two views.
Integer and index outputs must be identical; images are held to the 1e-5
max-abs bound (and are in fact bit-identical: both sides evaluate the same
f32 operations in the same order); gradients to the oracle within the
stated relative tolerances."""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-5      # rendered images, max abs per channel


def make(sky, P, cams, targets, **cfg):
    r = sky.GaussianRenderer(**cfg)
    r.load_points(P)
    r.setTrainingCameras(cams)
    if targets is not None:
        r.setTrainingImages(targets)
    return r


def small_case():
    P = scenes.scene_uniform(16384, seed=1001)
    cams = scenes.cameras_single(256, 256, 3.0)
    tgt = [scenes.target_uniform(256, 256, seed=2001)]
    cfg = dict(sh_degree=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=16)
    return P, cams, tgt, cfg


def oracle_settings(orc, cfg):
    return orc.settings(tile_size=cfg.get("tile_size", 16), w_l2=cfg["w_l2"], w_l1=cfg["w_l1"],
                        w_ssim=cfg["w_ssim"], round_f16=cfg.get("round_params_f16", 1))


def check_view(r, ref, n, view_index, tile_base, item_base, isect_base):
    """Compares the GPU buffers of one view of the last step with the oracle."""
    rec = r.read_buffer("records").reshape(-1, 12)[item_base:item_base + n]
    counts = r.read_buffer("counts")[item_base:item_base + n]
    pr = ref["pr"]
    assert np.array_equal(counts, pr["counts"])
    dr = r.read_buffer("depth_radius").reshape(-1, 2)[item_base:item_base + n]
    vis = pr["rec"][:, 10] > 0
    assert np.array_equal(rec[:, :9][vis], pr["rec"][:, :9][vis])
    assert np.array_equal(dr[vis], pr["rec"][:, 9:11][vis])
    assert np.all(dr[~vis] == 0)
    tl = ref["tl"]
    I = tl["keys_sorted"].shape[0]
    ks = r.read_buffer("keys_sorted")[isect_base:isect_base + I]
    assert np.array_equal((ks >> 16) - (tile_base - ref["group_tile_base"]), tl["keys_sorted"] >> 16)
    assert np.array_equal(ks & 0xFFFF, tl["keys_sorted"] & 0xFFFF)
    flat = r.read_buffer("flatten")[isect_base:isect_base + I]
    assert np.array_equal(flat - item_base, tl["gidx_sorted"])
    T = tl["offsets"].shape[0] - 1
    off = r.read_buffer("tile_offsets")[tile_base:tile_base + T + 1]
    assert np.array_equal(off - isect_base, tl["offsets"])


def test_small_view_forward_bit_exact(sky, orc):
    P, cams, tgt, cfg = small_case()
    r = make(sky, P, cams, tgt, **cfg)
    loss = r.forward([0])
    s = oracle_settings(orc, cfg)
    ref = orc.view_pipeline(P, cams[0], tgt[0], s, 0, mode=0)
    ref["group_tile_base"] = 0
    check_view(r, ref, P.shape[1], 0, 0, 0, 0)
    rgba = r.read_buffer("color").reshape(-1, 4)
    assert np.max(np.abs(rgba - ref["fw"]["rgba"])) <= IMG_TOL
    assert np.array_equal(rgba, ref["fw"]["rgba"])
    alpha = r.read_buffer("alpha")
    assert np.array_equal(alpha, ref["fw"]["alpha"])
    assert np.array_equal(r.read_buffer("last_ids"), ref["fw"]["last"])
    res = r.read_buffer("residual").reshape(-1, 4)
    assert np.array_equal(res, ref["ls"]["residual"])
    assert loss == pytest.approx(ref["ls"]["loss"], rel=1e-12)
    # the public render entry point returns the same image
    img, a2 = r.render([0])
    assert np.array_equal(img, ref["fw"]["rgba"]) and np.array_equal(a2, ref["fw"]["alpha"])


def per_gaussian_partials(r, n, items_base=0):
    """Sums the GPU per-intersection partials per (view, Gaussian) item, in
    float64, using the emission-order ranges of the cumsum (items are emitted
    in the order of the item_order buffer)."""
    part = r.read_buffer("partials").reshape(-1, 12)[:, :9].astype(np.float64)
    counts = r.read_buffer("counts").astype(np.int64)
    cum = r.read_buffer("cumsum").astype(np.int64)
    order = r.read_buffer("item_order").astype(np.int64)
    items = counts.shape[0]
    assert np.array_equal(np.sort(order), np.arange(items))
    emitted = counts[order]                      # counts in emission order
    assert np.array_equal(np.cumsum(emitted), cum)
    out = np.zeros((items, 9))
    seg_item = np.repeat(order, emitted)          # item of every emitted intersection
    np.add.at(out, seg_item, part[: cum[-1]])
    return out


def test_small_view_backward_partials_and_gradients(sky, orc):
    P, cams, tgt, cfg = small_case()
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([0])
    grads = r.backward()
    s = oracle_settings(orc, cfg)
    ref = orc.view_pipeline(P, cams[0], tgt[0], s, 0, mode=0)
    gpu9 = per_gaussian_partials(r, P.shape[1])
    ref9, mass = ref["bw"]["gsum9"], ref["bw"]["gabs9"]
    # per (tile, intersection) sums differ only in f32 summation order
    assert np.all(np.abs(gpu9 - ref9) <= 2e-5 * mass + 1e-9)
    g_ref = orc.geom(P, cams[0], s, 0, ref9.astype(np.float32))
    for lo, hi in [(0, 3), (3, 6), (6, 10), (10, 11), (11, 14)]:
        a, b = grads[lo:hi], g_ref[lo:hi]
        scale = np.max(np.abs(b))
        assert scale > 0
        assert np.all(np.abs(a - b) <= 1e-3 * np.abs(b) + 1e-4 * scale), (lo, hi)
    assert np.all(grads[14:] == 0)


def test_reference_mode_fixed_point_sums_bit_exact(sky, orc):
    P, cams, tgt, cfg = small_case()
    r = make(sky, P, cams, tgt, backward_mode=1, **cfg)
    r.forward([0])
    grads = r.backward()
    s = oracle_settings(orc, cfg)
    ref = orc.view_pipeline(P, cams[0], tgt[0], s, 0, mode=1)
    tg = r.read_buffer("tile_grads").reshape(-1, 54)
    assert np.array_equal(tg, ref["bw"]["tile_grads"])
    gs = ref["bw"]["gsum54"]
    scale = np.float32(1.0 / 65536.0)
    # opacity and SH planes come straight from the exact i64 sums
    assert np.array_equal(grads[10], gs[:, 0].astype(np.float32) * scale)
    sh = (gs[:, 6:].astype(np.float32) * scale).T
    assert np.array_equal(grads[11:14], sh[0:3])


def test_adam_step_matches_oracle_given_the_same_gradients(sky, orc):
    P, cams, tgt, cfg = small_case()
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([0])
    g = r.backward()
    p0 = r.params()
    st = r.trainStep([0])
    assert st.iteration == 1 and st.sh_updated == 0
    sc = r.read_buffer("step_scalars")
    lr = sc[0:5]
    b1, b2, eps, bc1, bc2 = sc[5:10]
    p1 = r.params()
    m1, m2 = r.moments()
    exp_p, exp_m1, exp_m2 = p0.copy(), np.zeros_like(p0), np.zeros_like(p0)
    groups = [(0, 3, lr[0]), (3, 6, lr[1]), (6, 10, lr[2]), (10, 11, lr[3])]
    for lo, hi, l in groups:
        pp = np.ascontiguousarray(exp_p[lo:hi])
        a, b = np.ascontiguousarray(exp_m1[lo:hi]), np.ascontiguousarray(exp_m2[lo:hi])
        orc.adam(pp, a, b, np.ascontiguousarray(g[lo:hi]), l, b1, b2, eps, bc1, bc2)
        exp_p[lo:hi], exp_m1[lo:hi], exp_m2[lo:hi] = pp, a, b
    assert np.array_equal(p1, exp_p)
    assert np.array_equal(m1, exp_m1) and np.array_equal(m2, exp_m2)


def clustered_case(n=20000):
    P = scenes.scene_clusters(n, seed=1003, clusters=16, center_range=1.0, cluster_sigma=0.25,
                              logscale_mean=-3.8)
    cams = scenes.cameras_orbit(3, 3.5, 240, 176)
    tgt = [scenes.target_uniform(240, 176, seed=2100 + k) for k in range(3)]
    cfg = dict(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=16)
    return P, cams, tgt, cfg


def test_batched_views_match_per_view_oracle_sh3(sky, orc):
    P, cams, tgt, cfg = clustered_case()
    n = P.shape[1]
    r = make(sky, P, cams, tgt, **cfg)
    views = [2, 0, 1]
    r.forward(views)
    s = oracle_settings(orc, cfg)
    rgba = r.read_buffer("color").reshape(-1, 4)
    counts = r.read_buffer("counts").astype(np.int64)
    tile_base = isect_base = pix = 0
    for k, v in enumerate(views):
        ref = orc.view_pipeline(P, cams[v], tgt[v], s, 3, mode=0)
        ref["group_tile_base"] = 0
        check_view(r, ref, n, k, tile_base, k * n, isect_base)
        npx = cams[v]["width"] * cams[v]["height"]
        assert np.array_equal(rgba[pix:pix + npx], ref["fw"]["rgba"])
        tw, th = orc.tiles_wh(cams[v], 16)
        tile_base += tw * th
        # sorted by tile, a view's intersections follow those of the views
        # before it in the sort group (emission interleaves them by depth)
        isect_base += int(counts[k * n:(k + 1) * n].sum())
        pix += npx


def test_two_sort_groups_match_per_view_oracle(sky, orc):
    """Three 1920x1080 views at 8-pixel tiles: 32,400 tiles each, so the
    step splits into two sort groups (views 0-1 and view 2; a group holds at
    most 65,536 tiles).  Items are emitted per group in depth order and the
    intersections sorted on the tile field only: keys, tile ranges, item
    lists and images must still be those of the oracle's per-view full-key
    sort, and the per-item partial sums its gradients."""
    P = scenes.scene_clusters(20000, seed=1011, clusters=16, center_range=1.0, cluster_sigma=0.25,
                              logscale_mean=-3.8)
    cams = scenes.cameras_orbit(3, 3.5, 1920, 1080)
    tgt = [scenes.target_uniform(1920, 1080, seed=2200 + k) for k in range(3)]
    cfg = dict(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=8)
    n = P.shape[1]
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([0, 1, 2])
    groups = r.read_buffer("groups").reshape(-1, 2)
    assert groups.shape[0] == 2
    s = oracle_settings(orc, cfg)
    rgba = r.read_buffer("color").reshape(-1, 4)
    counts = r.read_buffer("counts").astype(np.int64)
    tw, th = orc.tiles_wh(cams[0], 8)
    tile_base = isect_base = pix = 0
    refs = []
    for k in range(3):
        ref = orc.view_pipeline(P, cams[k], tgt[k], s, 3, mode=0)
        refs.append(ref)
        ref["group_tile_base"] = 0 if k < 2 else 2 * tw * th
        if k == 2:
            assert isect_base == int(groups[1, 0])
        check_view(r, ref, n, k, tile_base, k * n, isect_base)
        npx = 1920 * 1080
        assert np.array_equal(rgba[pix:pix + npx], ref["fw"]["rgba"])
        tile_base += tw * th
        isect_base += int(counts[k * n:(k + 1) * n].sum())
        pix += npx
    assert isect_base == int(groups[1, 1])
    r.backward()
    gpu9 = per_gaussian_partials(r, n)
    for k in range(3):
        ref9, mass = refs[k]["bw"]["gsum9"], refs[k]["bw"]["gabs9"]
        assert np.all(np.abs(gpu9[k * n:(k + 1) * n] - ref9) <= 2e-5 * mass + 1e-9)


def test_batched_gradients_are_sum_of_per_view(sky):
    P, cams, tgt, cfg = clustered_case(8000)
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([0, 1, 2])
    gb = r.backward()
    per = []
    for v in range(3):
        r.forward([v])
        per.append(r.backward())
    expect = (per[0] + per[1]) + per[2]
    # position (0-2), logit (10) and SH (11-58) are added per view in view
    # order: exactly the sum
    exact = np.r_[0:3, 10:59]
    assert np.array_equal(gb[exact], expect[exact])
    # log sigma (3-5) and the quaternion (6-9) come from one pass of the
    # covariance chain over dL/dC3 summed across the views, the per-view runs
    # from one pass each: equal up to f32 rounding of the linear chain
    cov = np.r_[3:10]
    scale = max(float(np.abs(p[cov]).max()) for p in per)
    assert np.max(np.abs(gb[cov] - expect[cov])) <= 1e-5 * scale


def test_gradients_are_deterministic(sky):
    P, cams, tgt, cfg = clustered_case(8000)
    r = make(sky, P, cams, tgt, **cfg)
    r.forward([0, 1])
    g1 = r.backward()
    r.forward([0, 1])
    g2 = r.backward()
    assert np.array_equal(g1, g2)
