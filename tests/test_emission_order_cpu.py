"""The emission-order scheme of the step, checked on the CPU (no GPU).

The reference emits intersection keys (tile << 16) | depth16 in (view,
Gaussian) item order, each item's tiles in row-major order of its rectangle,
and sorts the full keys stably.  The library instead sorts each sort group's
items stably by depth16, emits in that order, and sorts the intersections
stably on the tile field only.  Because a tile belongs to one view, both give
the same permutation of (item, tile) pairs; these tests check that on random
items, with ties in depth, several views per sort group and several groups.
"""
import numpy as np


def emit(items, order):
    """Keys and items of all intersections, items in `order`."""
    keys, owners = [], []
    for it in order:
        view, depth16, x0, y0, x1, y1, tiles_x, key_tile_base = items[it]
        for ty in range(y0, y1):
            for tx in range(x0, x1):
                keys.append(((key_tile_base + ty * tiles_x + tx) << 16) | depth16)
                owners.append(it)
    return np.array(keys, np.uint64), np.array(owners, np.int64)


def random_step(rng, views, n, tiles_x, tiles_y, views_per_group):
    items = []
    for v in range(views):
        key_tile_base = (v % views_per_group) * tiles_x * tiles_y
        for g in range(n):
            depth16 = int(rng.integers(0, 6))          # few distinct depths: many ties
            x0 = int(rng.integers(0, tiles_x)); y0 = int(rng.integers(0, tiles_y))
            x1 = min(tiles_x, x0 + int(rng.integers(0, 4)))
            y1 = min(tiles_y, y0 + int(rng.integers(0, 4)))
            items.append((v, depth16, x0, y0, x1, y1, tiles_x, key_tile_base))
    return items


def test_depth_ordered_emission_with_tile_sort_equals_full_key_sort():
    rng = np.random.default_rng(11)
    for trial in range(20):
        views, n, tx, ty, vpg = 5, 60, 7, 5, 2
        items = random_step(rng, views, n, tx, ty, vpg)
        groups = [list(range(v0 * n, min(views, v0 + vpg) * n)) for v0 in range(0, views, vpg)]
        # reference: item order, stable sort of the full keys, per sort group
        ref = []
        for grp in groups:
            k, o = emit(items, grp)
            ref.append(o[np.argsort(k, kind="stable")])
        # library: per group a stable sort of the items by depth16, emission in
        # that order, a stable sort on the tile field alone
        lib = []
        for grp in groups:
            order = sorted(grp, key=lambda it: items[it][1])   # Python's sort is stable
            k, o = emit(items, order)
            lib.append(o[np.argsort(k >> 16, kind="stable")])
            # the sorted keys (tile and depth fields) are the reference's too
            assert np.array_equal(np.sort(k, kind="stable"), k[np.argsort(k >> 16, kind="stable")])
        for a, b in zip(ref, lib):
            assert np.array_equal(a, b)


def test_item_pass_key_carries_count_and_depth():
    """The item key is (min(count, 0xFFFF) << 16) | depth16: sorting on the
    low 16 bits orders by depth; the scan reads counts from the high half
    and gathers only saturated ones."""
    rng = np.random.default_rng(12)
    depth = rng.integers(0, 1 << 16, 1000).astype(np.uint32)
    count = rng.integers(0, 70000, 1000).astype(np.uint32)
    key = (np.minimum(count, 0xFFFF) << 16) | depth
    order = np.argsort(key & 0xFFFF, kind="stable")
    assert np.array_equal(order, np.argsort(depth, kind="stable"))
    hi = key[order] >> 16
    got = np.where(hi < 0xFFFF, hi, count[order])
    assert np.array_equal(got, count[order])
