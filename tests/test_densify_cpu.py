"""CPU checks of the densification oracle (oracle/densify.py): the counter
generator against a big-integer restatement, the vectorised candidate rule
against a literal loop over performDensification's steps, and the
weighted-sampling form used for the prune against the reference's
one-draw-at-a-time loop."""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle import densify as D

MASK = (1 << 64) - 1


def _uniform_bigint(seed, it, i, r):
    z = (seed * 0x9E3779B97F4A7C15 + it * 0xD1B54A32D192ED03 + i * 0x94D049BB133111EB
         + r * 0xBF58476D1CE4E5B9 + 0x9E3779B97F4A7C15) & MASK
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
    z = z ^ (z >> 31)
    return ((z >> 11) + 0.5) / 2.0 ** 53


def test_counter_uniform_matches_bigint():
    idx = np.arange(0, 5000, 7)
    for seed, it, r in [(0, 0, 0), (0x5EED, 500, 3), (2**63 + 5, 12345, 64)]:
        got = D.counter_uniform(seed, it, idx, r)
        want = np.array([_uniform_bigint(seed, it, int(i), r) for i in idx])
        assert np.array_equal(got, want)
        assert (got > 0).all() and (got < 1).all()


def _decide_literal(params, acc, importance, sample_count, grad_px, grad_abs_px, size_thr,
                    min_vis, imp_thr, max_new_ratio):
    """performDensification :3256-3318 step by step."""
    n = params.shape[1]
    cands = []
    for i in range(n):
        denom = float(acc[i, 3])
        if denom < max(1.0, min_vis):
            continue
        avg = float(acc[i, 0]) / denom
        avg_abs = float(acc[i, 2]) / denom
        ms = max(math.exp(float(params[3, i])), math.exp(float(params[4, i])),
                 math.exp(float(params[5, i])))
        imp = float(importance[i]) / max(1, sample_count)
        if imp <= imp_thr:
            continue
        if ms <= size_thr and avg >= grad_px:
            cands.append((i, 1, avg / grad_px if grad_px > 1e-8 else avg))
        elif ms > size_thr and avg_abs >= grad_abs_px:
            cands.append((i, 2, avg_abs / grad_abs_px if grad_abs_px > 1e-8 else avg_abs))
    action = np.zeros(n, np.uint32)
    if not cands:
        return action
    allowed = min(max(1, math.floor(n * max_new_ratio)), len(cands))
    cands.sort(key=lambda c: -c[2])  # stable, like Array.prototype.sort
    for i, a, _ in cands[:allowed]:
        action[i] = a
    return action


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_decide_matches_literal_loop(seed):
    rng = np.random.default_rng(seed)
    n = 400
    params = rng.normal(size=(59, n)).astype(np.float32)
    params[3:6] = rng.uniform(-6, -1, size=(3, n)).astype(np.float32)
    acc = np.zeros((n, 4), np.float32)
    acc[:, 3] = rng.integers(0, 40, n)
    acc[:, 0] = (rng.uniform(0, 0.2, n) * acc[:, 3]).astype(np.float32)
    acc[:, 2] = (rng.uniform(0, 0.8, n) * acc[:, 3]).astype(np.float32)
    # equal scores to exercise the stable order
    acc[10:20, :] = acc[10]
    importance = rng.integers(0, 200, n).astype(np.uint32)
    args = (params, acc, importance, 10, 0.003 * 32, 0.015 * 32,
            float(np.median(np.exp(params[3:6].astype(np.float64)).max(axis=0))), 5.0, 5.0, 0.1)
    got = D.densify_decide(*args)
    want = _decide_literal(*args)
    assert np.array_equal(got, want)
    assert (got == 1).any() and (got == 2).any()


def test_build_layout():
    rng = np.random.default_rng(7)
    n = 50
    params = rng.normal(size=(59, n)).astype(np.float32)
    m1 = rng.normal(size=(59, n)).astype(np.float32)
    m2 = rng.uniform(size=(59, n)).astype(np.float32)
    action = np.zeros(n, np.uint32)
    action[[3, 9, 20]] = 1
    action[[5, 30]] = 2
    P, M1, M2 = D.densify_build(params, m1, m2, action, 0x5EED, 700)
    keep = action != 2
    assert P.shape[1] == n - 2 + 3 + 4
    assert np.array_equal(P[:, :n - 2], params[:, keep])
    assert np.array_equal(M1[:, :n - 2], m1[:, keep])
    assert not M1[:, n - 2:].any() and not M2[:, n - 2:].any()
    # clones keep everything but the position; splits shrink the scale
    assert np.array_equal(P[3:, n - 2], params[3:, 3])
    red = np.float32(math.log(1.6))
    assert np.allclose(P[3:6, n - 2 + 1], params[3:6, 5] - red, atol=1e-6)
    assert np.array_equal(P[6:, n - 2 + 1], params[6:, 5])


def test_efraimidis_spirakis_matches_sequential_draws():
    """Weighted sampling without replacement: sorting -log(u)/w and taking
    the first k gives the same inclusion probabilities as k sequential draws
    proportional to the remaining weights."""
    w = np.array([1.0, 2.0, 3.0, 5.0, 10.0, 1000.0 / 1.5])
    k = 2
    trials = 20000
    rng = np.random.default_rng(11)
    seq = np.zeros(w.size)
    for _ in range(trials):
        for i in D.sequential_weighted_sample(w, k, rng):
            seq[i] += 1
    es = np.zeros(w.size)
    for t in range(trials):
        u = D.counter_uniform(99, t, np.arange(w.size), 64)
        es[np.argsort(-np.log(u) / w, kind="stable")[:k]] += 1
    assert np.abs(seq / trials - es / trials).max() < 0.02


def test_prune_budget_rule():
    assert D.prune_budget(0, 1000) == 0
    assert D.prune_budget(1, 1000) == 1
    assert D.prune_budget(100, 1000) == 20      # max(1, floor(0.02 * 1000))
    assert D.prune_budget(10, 1000) == 5        # floor(0.5 * 10)
    assert D.prune_budget(3, 10) == 1


def test_importance_and_accum_updates():
    stats = np.array([[10.0, 2.0, 5.0, 0.0], [1.0, 1.0, 9.0, 0.0]], np.float32)
    out = D.importance_update(stats, np.array([3, 0], np.uint32), np.array([7.0, 100.0], np.float32))
    d = np.float32(0.98)
    assert out[0, 0] == np.float32(np.float32(10.0) * d) + np.float32(3)
    assert out[0, 2] == np.maximum(np.float32(5.0) * d, np.float32(7.0))
    assert out[1, 2] == np.float32(9.0) * d      # invisible: decay only
    acc = D.densify_accum_update(np.zeros((2, 4)), np.array([[0] * 7 + [3, 4], [0] * 9], float))
    assert acc[0].tolist() == [5.0, 0.0, 0.0, 1.0] and acc[1].tolist() == [0, 0, 0, 0]
