"""TEST INFRASTRUCTURE ONLY: numpy restatement of the reference's
densification path, used by tests/ as the checker of the device version.

Follows Skyfall-Viewer's
  - importance-accum.wgsl:19-40 and densify-accum.wgsl:19-46 (per-step
    statistics),
  - metric-map.wgsl:32-147 with computePixelLossStats / accumulateMetricCounts
    / generateMultiViewScores (src/renderers/gaussian-renderer.ts:2706-2788),
  - performDensification (gaussian-renderer.ts:3211-3433),
  - applyMultiViewPrune (gaussian-renderer.ts:2800-2915).
The reference draws its random numbers from Math.random(); this restatement
uses the same counter-based generator as the library (draw r of Gaussian i
at iteration t), so clone/split samples can be compared value by value.  The
prune selection follows the Efraimidis-Spirakis form of weighted sampling
without replacement; `sequential_weighted_sample` restates the reference's
one-draw-at-a-time loop for the distribution check.
"""
from __future__ import annotations

import math

import numpy as np

U64 = np.uint64
_G = U64(0x9E3779B97F4A7C15)
_M1 = U64(0xBF58476D1CE4E5B9)
_M2 = U64(0x94D049BB133111EB)
_M3 = U64(0xD1B54A32D192ED03)


def counter_uniform(seed: int, iteration: int, index, draw: int) -> np.ndarray:
    """Uniform doubles in (0, 1): splitmix64 finaliser of a linear mix of
    (seed, iteration, index, draw); 53 bits, offset by half an ulp."""
    idx = np.asarray(index, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (U64(seed) * _G + U64(iteration) * _M3 + idx * _M2 + U64(draw) * _M1 + _G)
        z = (z ^ (z >> U64(30))) * _M1
        z = (z ^ (z >> U64(27))) * _M2
        z = z ^ (z >> U64(31))
    return ((z >> U64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


# ---- per-step statistics --------------------------------------------------

def importance_update(stats: np.ndarray, counts: np.ndarray, radius: np.ndarray,
                      decay: float = 0.98) -> np.ndarray:
    """accumulate_importance (importance-accum.wgsl:19-40), f32."""
    s = stats.astype(np.float32).copy()
    d = np.float32(decay)
    s[:, 0] *= d
    s[:, 1] *= d
    s[:, 2] *= d
    vis = counts > 0
    s[vis, 0] += counts[vis].astype(np.float32)
    s[vis, 1] += np.float32(1.0)
    s[vis, 2] = np.maximum(s[vis, 2], radius[vis].astype(np.float32))
    return s


def densify_accum_update(acc: np.ndarray, g9: np.ndarray) -> np.ndarray:
    """accumulate_grads (densify-accum.wgsl:19-46) from per-Gaussian
    gradients (dcolor rgb, dlogit, dconic a b c, dmean2d x y)."""
    a = acc.astype(np.float64).copy()
    g = g9.astype(np.float64)
    n2d = np.sqrt(g[:, 7] ** 2 + g[:, 8] ** 2)
    nc = np.sqrt(g[:, 4] ** 2 + g[:, 5] ** 2 + g[:, 6] ** 2)
    hit = (n2d > 1e-10) | (nc > 1e-10)
    a[hit, 0] += n2d[hit]
    a[hit, 1] = 0.0
    a[hit, 2] += nc[hit]
    a[hit, 3] += 1.0
    return a


# ---- multi-view scores ------------------------------------------------------

def metric_view(rgba: np.ndarray, target: np.ndarray, last: np.ndarray, offsets: np.ndarray,
                gidx_sorted: np.ndarray, rec: np.ndarray, width: int, height: int,
                tile_size: int, n: int, threshold: float = 0.1):
    """One view: (hits per Gaussian u32, mean L1) following compute_metric_map,
    computePixelLossStats, threshold_metric_map and accumulate_metric_counts."""
    f32 = np.float32
    rgb = rgba[:, :3].astype(f32)
    t = target.reshape(-1, 3).astype(f32)
    d = np.abs(rgb - t)
    l1 = ((d[:, 0] + d[:, 1]) + d[:, 2]) / f32(3.0)
    fin = np.isfinite(l1)
    counts = np.zeros(n, np.uint32)
    if not fin.any():
        return counts, 0.0
    mn, mx = l1[fin].min(), l1[fin].max()
    mean = float(l1[fin].astype(np.float64).sum()) / l1.size
    inv = f32(1.0 / (float(mx) - float(mn))) if mx > mn else f32(0.0)
    value = (l1 - mn) * inv
    flagged = np.nonzero(value > f32(threshold))[0]
    tx = (width + tile_size - 1) // tile_size
    a = rec[:, 2].astype(f32)
    b = rec[:, 3].astype(f32)
    c = rec[:, 4].astype(f32)
    for p in flagged:
        x, y = int(p % width), int(p // width)
        tile = (y // tile_size) * tx + (x // tile_size)
        start, end = int(offsets[tile]), int(offsets[tile + 1])
        if start >= end:
            continue
        lst = int(last[p])
        if lst < start:
            continue
        fin_k = min(lst, end - 1)
        g = gidx_sorted[start:fin_k + 1].astype(np.int64)
        dx = f32(x + 0.5) - rec[g, 0]
        dy = f32(y + 0.5) - rec[g, 1]
        s = f32(0.5) * ((a[g] * dx) * dx + (c[g] * dy) * dy) + (b[g] * dx) * dy
        ok = (s >= 0) & (s <= 6)
        np.add.at(counts, g[ok], 1)
    return counts, mean


def combine_scores(views) -> tuple[np.ndarray, np.ndarray]:
    """generateMultiViewScores: importance (u32) and pruning (f32, one
    rounding per view as the reference's Float32Array) over views in order."""
    imp = None
    pr = None
    for counts, mean in views:
        if imp is None:
            imp = np.zeros(counts.shape[0], np.uint64)
            pr = np.zeros(counts.shape[0], np.float32)
        imp += counts
        pr = (pr.astype(np.float64) + counts.astype(np.float64) * mean).astype(np.float32)
    return imp.astype(np.uint32), pr


# ---- densification ---------------------------------------------------------

def densify_decide(params: np.ndarray, acc: np.ndarray, importance: np.ndarray,
                   sample_count: int, grad_px: float, grad_abs_px: float,
                   size_threshold: float, min_visibility: float, importance_threshold: float,
                   max_new_ratio: float = 0.1) -> np.ndarray:
    """performDensification :3248-3318: the applied action per Gaussian
    (0 none, 1 clone, 2 split)."""
    n = params.shape[1]
    denom = acc[:, 3].astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        avg = acc[:, 0].astype(np.float64) / denom
        avg_abs = acc[:, 2].astype(np.float64) / denom
    ms = np.exp(params[3:6].astype(np.float64)).max(axis=0)
    imp = importance.astype(np.float64) / max(1.0, float(sample_count))
    ok = ~(denom < max(1.0, min_visibility)) & (imp > importance_threshold)
    clone = ok & (ms <= size_threshold) & (avg >= grad_px)
    split = ok & ~clone & (ms > size_threshold) & (avg_abs >= grad_abs_px)
    score = np.where(clone, avg / grad_px if grad_px > 1e-8 else avg,
                     avg_abs / grad_abs_px if grad_abs_px > 1e-8 else avg_abs)
    cand = np.nonzero(clone | split)[0]
    action = np.zeros(n, np.uint32)
    if cand.size == 0:
        return action
    order = cand[np.argsort(-score[cand], kind="stable")]
    allowed = min(max(1, math.floor(n * max_new_ratio)), cand.size)
    sel = order[:allowed]
    action[sel] = np.where(clone[sel], 1, 2)
    return action


def densify_build(params: np.ndarray, m1: np.ndarray, m2: np.ndarray, action: np.ndarray,
                  seed: int, iteration: int):
    """performDensification :3325-3420: survivors in order, then clones and
    split samples per candidate in index order, zero moments for new ones."""
    keep = action != 2
    newp = [params[:, keep]]
    new1 = [m1[:, keep]]
    new2 = [m2[:, keep]]
    red = math.log(0.8 * 2.0)
    for i in np.nonzero(action)[0]:
        p = params[:, i].astype(np.float32)
        sig = np.exp(p[3:6].astype(np.float64))
        pos = p[0:3].astype(np.float64)
        u = lambda r: float(counter_uniform(seed, iteration, i, r))  # noqa: E731
        if action[i] == 1:
            mag = sig.max() * 0.25 * (0.5 + u(0) * 0.5)
            d = np.array([u(1) * 2 - 1, u(2) * 2 - 1, u(3) * 2 - 1])
            nrm = math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) or 1.0
            q = p.copy()
            q[0:3] = (pos + d / nrm * mag).astype(np.float32)
            outs = [q]
        else:
            x, y, z, w = (float(v) for v in p[6:10])
            x2, y2, z2 = x + x, y + y, z + z
            xx, xy, xz, yy, yz, zz = x * x2, x * y2, x * z2, y * y2, y * z2, z * z2
            wx, wy, wz = w * x2, w * y2, w * z2
            R = np.array([[1 - (yy + zz), xy - wz, xz + wy],
                          [xy + wz, 1 - (xx + zz), yz - wx],
                          [xz - wy, yz + wx, 1 - (xx + yy)]])
            outs = []
            for smp in range(2):
                u1, u2, u3, u4 = (u(4 + 4 * smp + k) for k in range(4))
                r1, r3 = math.sqrt(-2 * math.log(u1)), math.sqrt(-2 * math.log(u3))
                l = np.array([r1 * math.cos(2 * math.pi * u2) * sig[0],
                              r1 * math.sin(2 * math.pi * u2) * sig[1],
                              r3 * math.cos(2 * math.pi * u4) * sig[2]])
                q = p.copy()
                q[0:3] = (pos + R @ l).astype(np.float32)
                q[3:6] = (p[3:6].astype(np.float64) - red).astype(np.float32)
                outs.append(q)
        for q in outs:
            newp.append(q[:, None])
            new1.append(np.zeros((params.shape[0], 1), np.float32))
            new2.append(np.zeros((params.shape[0], 1), np.float32))
    return (np.concatenate(newp, axis=1), np.concatenate(new1, axis=1),
            np.concatenate(new2, axis=1))


# ---- scored prune -------------------------------------------------------------

def prune_keys(params: np.ndarray, pruning: np.ndarray, base: int, imp_stats: np.ndarray | None,
               min_opacity: float, max_scale: float, max_screen_radius: float,
               use_screen: bool, seed: int, iteration: int, opacity_bonus: float = 0.35,
               scale_bonus: float = 0.25, screen_bonus: float = 0.25):
    """applyMultiViewPrune :2820-2886: prunable flags, weights and the
    selection keys -log(u) / w (inf for Gaussians that are not prunable)."""
    n = params.shape[1]
    sc = pruning[:base].astype(np.float64)
    finite = sc[np.isfinite(sc)]
    if finite.size:
        lo, hi = float(finite.min()), float(finite.max())
    else:
        lo, hi = 0.0, 1.0
    rng = max(1e-6, hi - lo)
    norm = np.zeros(n, np.float32)
    norm[:base] = ((sc - lo) / rng).astype(np.float32)
    op = 1.0 / (1.0 + np.exp(-params[10].astype(np.float64)))
    low = op < min_opacity
    large = np.exp(params[3:6].astype(np.float64)).max(axis=0) > max_scale
    screen = np.zeros(n, bool)
    if use_screen and max_screen_radius < 9999 and imp_stats is not None:
        r = imp_stats[:, 2]
        screen = np.isfinite(r) & (r.astype(np.float64) > max_screen_radius)
    prunable = low | large | screen
    ws = np.where(np.isfinite(norm), norm.astype(np.float64), 0.0)
    ws = ws + np.where(low, opacity_bonus, 0.0) + np.where(large, scale_bonus, 0.0) + \
        np.where(screen, screen_bonus, 0.0)
    ws = np.minimum(0.999, np.maximum(0.0, ws))
    w = 1.0 / (1e-6 + (1.0 - ws))
    u = counter_uniform(seed, iteration, np.arange(n), 64)
    keys = np.where(prunable, -np.log(u) / w, np.inf)
    return prunable, w, keys


def prune_budget(num_prunable: int, base_count: int, prune_ratio: float = 0.5,
                 max_ratio: float = 0.02) -> int:
    """removeBudget of applyMultiViewPrune :2888-2891."""
    if num_prunable == 0:
        return 0
    max_removals = max(1, math.floor(base_count * max_ratio))
    desired = max(1, math.floor(num_prunable * prune_ratio))
    return min(num_prunable, desired, max_removals)


def sequential_weighted_sample(weights: np.ndarray, budget: int, rng: np.random.Generator):
    """The reference's selection loop (:2893-2909): budget draws, each with
    probability proportional to the remaining weights."""
    w = weights.astype(np.float64).copy()
    total = w.sum()
    chosen = []
    for _ in range(budget):
        if total <= 0:
            break
        target = rng.random() * total
        acc = 0.0
        for i in range(w.size):
            if w[i] == 0:
                continue
            acc += w[i]
            if target <= acc:
                chosen.append(i)
                total -= w[i]
                w[i] = 0
                break
    return chosen
