"""Pins of the CPU oracle (no GPU): its primitives against numpy/float64,
analytic known-answer cases, its fixed point and tile-range rules, and its
exact adjoint against FP64 central finite differences."""
import math

import numpy as np
import pytest

from skyfall import scenes

SH_C0 = 0.28209479177387814


def test_expf_within_one_ulp(orc):
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(-87, 88, 400_000), rng.uniform(-12, 0, 400_000),
                        np.linspace(-87, 88, 200_001)]).astype(np.float32)
    y = orc.expf(x).astype(np.float64)
    ref = np.exp(x.astype(np.float64))
    ulp = np.spacing(ref.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(y - ref) / ulp) <= 1.0
    assert orc.expf(np.array([-100.0, 100.0, np.nan], np.float32)).tolist()[:2] == [0.0, np.inf]


def test_round_f16_is_round_to_nearest_even(orc):
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(0, 1, 200_000), rng.normal(0, 3e4, 20_000),
                        rng.uniform(-1e-6, 1e-6, 20_000),
                        [65504, 65519.99, 65520, -65520, 6.1e-5, 5.96e-8, 2.98e-8, 2.99e-8]]).astype(np.float32)
    y = orc.round_f16(x)
    with np.errstate(over="ignore"):  # 65520 and beyond round to infinity, as intended
        ref = x.astype(np.float16).astype(np.float32)
    assert np.array_equal(y, ref)


def single_gaussian(pos=(0.0, 0.0, 0.0), sigma=0.05, logit=0.0, color=0.7):
    P = np.zeros((59, 1), np.float32)
    P[0:3, 0] = pos
    P[3:6, 0] = math.log(sigma)
    P[9, 0] = 1.0                      # quaternion (0, 0, 0, 1)
    P[10, 0] = logit
    P[11:14, 0] = (color - 0.5) / SH_C0
    return P


def test_single_isotropic_gaussian_closed_form(orc):
    """An isotropic Gaussian on the optical axis: conic, radius, tile count and
    every pixel of the image follow in closed form."""
    cam = scenes.cameras_single(256, 256, 3.0)[0]
    s = orc.settings(round_f16=0, nthreads=1, w_l2=1.0, w_l1=0.0, w_ssim=0.0)
    P = single_gaussian()
    out = orc.view_pipeline(P, cam, None, s, 0)
    rec = out["pr"]["rec"][0]
    f = float(cam["focal"][0])
    c = (f * 0.05 / 3.0) ** 2 + 0.3
    assert rec[0] == pytest.approx(128.0, abs=1e-4) and rec[1] == pytest.approx(128.0, abs=1e-4)
    assert rec[2] == pytest.approx(1.0 / c, rel=1e-5)
    assert abs(rec[3]) < 1e-7
    assert rec[4] == pytest.approx(1.0 / c, rel=1e-5)
    radius = math.ceil(3.0 * math.sqrt(c))
    assert rec[10] == radius
    x0, x1 = math.floor((128 - radius) / 16), math.ceil((128 + radius) / 16)
    assert out["pr"]["counts"][0] == (x1 - x0) ** 2
    ys, xs = np.mgrid[0:256, 0:256]
    d2 = (xs + 0.5 - 128.0) ** 2 + (ys + 0.5 - 128.0) ** 2
    a = np.minimum(0.5 * np.exp(-0.5 * d2 / c), 0.999)
    a[a < 1 / 255] = 0
    # pixels outside the Gaussian's tile rectangle are not rendered at all
    inrect = (xs // 16 >= x0) & (xs // 16 < x1) & (ys // 16 >= x0) & (ys // 16 < x1)
    a[~inrect] = 0
    img = out["fw"]["rgba"][:, 0].reshape(256, 256)
    assert np.max(np.abs(img - 0.7 * a)) < 2e-6
    assert np.max(np.abs(out["fw"]["alpha"].reshape(256, 256) - a)) < 2e-6


def test_two_splats_composite_front_to_back(orc):
    cam = scenes.cameras_single(64, 64, 3.0)[0]
    s = orc.settings(round_f16=0, nthreads=1)
    # the farther splat has the lower index: the depth key must put it second
    P = np.concatenate([single_gaussian((0, 0, 1.5), 0.08, 1.0, 0.2),
                        single_gaussian((0, 0, -0.5), 0.08, 0.5, 0.9)], axis=1)
    out = orc.view_pipeline(P, cam, None, s, 0)
    keys = out["tl"]["keys_sorted"]
    assert np.all(np.diff(keys.astype(np.int64)) >= 0)
    rec = out["pr"]["rec"]
    assert rec[0, 9] == pytest.approx(4.5) and rec[1, 9] == pytest.approx(2.5)
    p = 32 * 64 + 32          # pixel (32, 32), centre at (32.5, 32.5)
    def alpha(i):
        dx = 32.5 - rec[i, 0]
        dy = 32.5 - rec[i, 1]
        sv = 0.5 * (rec[i, 2] * dx * dx + rec[i, 4] * dy * dy) + rec[i, 3] * dx * dy
        return min(rec[i, 5] * math.exp(-sv), 0.999)
    a_front, a_back = alpha(1), alpha(0)
    expect = 0.9 * a_front + 0.2 * a_back * (1 - a_front)
    assert out["fw"]["rgba"][p, 0] == pytest.approx(expect, rel=1e-5)


def test_stable_sort_keeps_index_order_on_equal_keys(orc):
    cam = scenes.cameras_single(64, 64, 3.0)[0]
    s = orc.settings(round_f16=0, nthreads=1)
    # depths 3.9, 3.1, 3.4: the same integer depth 3, so equal keys per tile
    P = np.concatenate([single_gaussian((0, 0, 0.9), 0.05), single_gaussian((0, 0, 0.1), 0.05),
                        single_gaussian((0, 0, 0.4), 0.05)], axis=1)
    out = orc.view_pipeline(P, cam, None, s, 0)
    ks, gs = out["tl"]["keys_sorted"], out["tl"]["gidx_sorted"]
    for key in np.unique(ks):
        assert list(gs[ks == key]) == [0, 1, 2]


def test_tile_offsets_are_first_index_with_backfill(orc):
    P = scenes.scene_uniform(4096, seed=7)
    cam = scenes.cameras_single(200, 136, 3.0)[0]
    s = orc.settings(nthreads=4)
    out = orc.view_pipeline(P, cam, None, s, 0)
    ks, off = out["tl"]["keys_sorted"], out["tl"]["offsets"]
    tiles = ks >> 16
    T = off.shape[0] - 1
    expect = np.searchsorted(tiles, np.arange(T + 1), side="left")
    assert np.array_equal(off, expect.astype(np.uint32))
    assert off[-1] == ks.shape[0]


def test_reference_mode_sums_fixed_point_per_intersection(orc):
    """Reference mode: the i64 per-Gaussian sums equal the sums of the i32
    per-(tile, intersection) values."""
    P = scenes.scene_uniform(2048, seed=3)
    cam = scenes.cameras_single(96, 96, 3.0)[0]
    s = orc.settings(nthreads=4, w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    tgt = scenes.target_uniform(96, 96)
    out = orc.view_pipeline(P, cam, tgt, s, 0, mode=1)
    tg, gs = out["bw"]["tile_grads"], out["bw"]["gsum54"]
    gidx = out["tl"]["gidx_sorted"]
    acc = np.zeros_like(gs)
    np.add.at(acc, gidx, tg.astype(np.int64))
    assert np.array_equal(acc, gs)
    assert np.count_nonzero(tg) > 0


def _fd_scene():
    P = scenes.scene_uniform(600, seed=11)
    P[3:6] += 1.2            # larger splats: more pixels per Gaussian
    cam = scenes.cameras_single(96, 96, 3.0)[0]
    return P, cam


def test_oracle_exact_adjoint_matches_fp64_finite_differences(orc):
    P, cam = _fd_scene()
    deg = 0
    s = orc.settings(round_f16=0, nthreads=4, w_l2=1.0, w_l1=0.2, w_ssim=0.0)
    tgt = scenes.target_uniform(96, 96, seed=5)
    out = orc.view_pipeline(P, cam, tgt, s, deg, mode=0)
    g = orc.geom(P, cam, s, deg, out["bw"]["gsum9"].astype(np.float32))
    rng = np.random.default_rng(0)
    P64 = P.astype(np.float64)
    planes = [0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13]
    cand = [(p, i) for p in planes for i in range(P.shape[1]) if abs(g[p, i]) > 1e-3]
    picks = [cand[k] for k in rng.choice(len(cand), size=min(96, len(cand)), replace=False)]
    h = 1e-4
    checked, bad = 0, []
    for p, i in picks:
        Pp, Pm = P64.copy(), P64.copy()
        Pp[p, i] += h
        Pm[p, i] -= h
        lp, sp = orc.loss_f64(Pp, cam, s, deg, tgt)
        lm, sm = orc.loss_f64(Pm, cam, s, deg, tgt)
        _, s0 = orc.loss_f64(P64, cam, s, deg, tgt)
        if not (sp == sm == s0):
            continue          # a discrete decision flips inside [-h, h]
        fd = (lp - lm) / (2 * h)
        checked += 1
        if abs(g[p, i] - fd) > 1e-3 * abs(fd) + 1e-6:
            bad.append((p, i, float(g[p, i]), fd))
    assert checked >= 40
    assert not bad, bad[:5]


def test_logf_within_two_ulp(orc):
    """The oracle's (and the kernels') log: within 2 ulp of the f64 log over
    normal and subnormal arguments, exact specials."""
    rng = np.random.default_rng(5)
    x = np.concatenate([
        np.exp(rng.uniform(-87, 88, 200000)).astype(np.float32),
        rng.uniform(0.5, 2.0, 100000).astype(np.float32),
        (rng.uniform(0, 1, 2000) * 1e-40).astype(np.float32),
        np.array([1.0, 2.0, 0.5, 1e-6, 0.1, 3.4e38], np.float32),
    ])
    x = x[x > 0]
    got = orc.logf(x).astype(np.float64)
    want = np.log(x.astype(np.float64))
    ulp = np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    err = np.abs(got - want) / ulp
    assert err.max() <= 2.0, err.max()
    assert orc.logf(np.array([1.0], np.float32))[0] == 0.0
    sp = orc.logf(np.array([0.0, -1.0, np.inf], np.float32))
    assert sp[0] == -np.inf and np.isnan(sp[1]) and sp[2] == np.inf
