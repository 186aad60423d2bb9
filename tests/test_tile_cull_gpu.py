"""Culled intersection lists (SkyConfig.tile_cull) on the GPU.

With tile_cull the backward and training steps list, per Gaussian, only the
tiles of its rectangle that its alpha >= 1/255 ellipse reaches.  A tile left
out holds no pixel where the Gaussian passes the rasterisers' pre-filter, so
it changes no pixel, no partial sum and no statistic: these tests train the
same scene with and without culling and require the parameters, Adam
moments, losses, densification statistics and images to be bit-identical,
for every tile size, the graph-captured step and a step split into two sort
groups (the reference backward mode keeps the reference's lists); and the
culled lists to be ordered sub-lists of the reference's.
"""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu


def make(sky, P, cams, targets, **cfg):
    r = sky.GaussianRenderer(**cfg)
    r.load_points(P)
    r.setTrainingCameras(cams)
    r.setTrainingImages(targets)
    return r


def scene(seed):
    # clusters of mid-sized splats whose opacities span the range, so that
    # many rectangles hold tiles the alpha >= 1/255 ellipse does not reach
    return scenes.scene_clusters(20000, seed=seed, clusters=16, center_range=1.0, cluster_sigma=0.25,
                                 logscale_mean=-3.4)


def train(sky, P, cams, tgts, cull, steps, view_sets, **cfg):
    r = make(sky, P, cams, tgts, **cfg)
    r.setTileCull(cull)
    assert r.getConfig().tile_cull == (1 if cull else 0)
    losses, isects = [], []
    for k in range(steps):
        st = r.trainStep(view_sets[k % len(view_sets)])
        losses.append(st.loss)
        isects.append(st.num_intersections)
    out = dict(params=r.params(), moments=r.moments(), stats=r.densifyStats(), losses=losses,
               isects=isects)
    r.forward(view_sets[0])
    out["color"] = r.read_buffer("color")
    out["loss_fwd"] = r.forward(view_sets[0])
    out["grads"] = r.backward()
    r.close()
    return out


def assert_same(a, b):
    assert a["losses"] == b["losses"]
    assert np.array_equal(a["params"].view(np.uint32), b["params"].view(np.uint32))
    for x, y in zip(a["moments"], b["moments"]):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    for x, y in zip(a["stats"], b["stats"]):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    assert np.array_equal(a["color"].view(np.uint32), b["color"].view(np.uint32))
    assert a["loss_fwd"] == b["loss_fwd"]
    assert np.array_equal(a["grads"].view(np.uint32), b["grads"].view(np.uint32))


@pytest.mark.parametrize("ts,mode,graph", [(16, 0, 0), (8, 0, 0), (32, 0, 0), (16, 1, 0), (16, 0, 1)])
def test_culled_lists_train_bit_identically(sky, ts, mode, graph):
    P = scene(1701)
    cams = scenes.cameras_orbit(4, 3.5, 320, 240)
    tgts = [scenes.target_uniform(320, 240, seed=2700 + k) for k in range(4)]
    cfg = dict(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.2, tile_size=ts,
               backward_mode=mode, use_graph=graph)
    sets = [[0, 1, 2, 3], [1, 3], [2]]
    full = train(sky, P, cams, tgts, False, 5, sets, **cfg)
    cull = train(sky, P, cams, tgts, True, 5, sets, **cfg)
    assert_same(full, cull)
    if mode == 1:
        # the reference backward's sums depend on its batches of list
        # entries, so it keeps the reference's lists
        assert cull["isects"] == full["isects"]
        return
    # and the lists really are shorter
    assert all(c < f for c, f in zip(cull["isects"], full["isects"]))
    assert sum(cull["isects"]) < 0.9 * sum(full["isects"])


def test_culled_lists_with_two_sort_groups(sky):
    """Three 1920x1080 views at 8-pixel tiles split into two sort groups."""
    P = scene(1702)
    cams = scenes.cameras_orbit(3, 3.5, 1920, 1080)
    tgts = [scenes.target_uniform(1920, 1080, seed=2710 + k) for k in range(3)]
    cfg = dict(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=8)
    full = train(sky, P, cams, tgts, False, 2, [[0, 1, 2]], **cfg)
    cull = train(sky, P, cams, tgts, True, 2, [[0, 1, 2]], **cfg)
    assert_same(full, cull)
    assert cull["isects"][0] < full["isects"][0]


def test_culled_lists_are_ordered_sublists(sky):
    """Per tile, the culled list is the reference list with some entries
    dropped, in the same order; per item, its count is at most its
    rectangle's area; a render (which always lists every tile) after a
    culled step gives the reference lists again."""
    P = scene(1703)
    cams = scenes.cameras_orbit(2, 3.5, 320, 240)
    tgts = [scenes.target_uniform(320, 240, seed=2720 + k) for k in range(2)]
    cfg = dict(sh_degree=3, sh_degree_interval=0, w_l2=1.0, w_l1=0.2, w_ssim=0.0, tile_size=16)
    r = make(sky, P, cams, tgts, **cfg)
    r.forward([0, 1])
    off_f = r.read_buffer("tile_offsets").astype(np.int64)
    flat_f = r.read_buffer("flatten").astype(np.int64)
    counts_f = r.read_buffer("counts").astype(np.int64)
    r.setTileCull(True)
    r.backward()  # a backward step lists the culled tiles (parameters unchanged)
    off_c = r.read_buffer("tile_offsets").astype(np.int64)
    flat_c = r.read_buffer("flatten").astype(np.int64)
    counts_c = r.read_buffer("counts").astype(np.int64)
    assert off_c[-1] < off_f[-1]
    assert np.all(counts_c <= counts_f) and counts_c.sum() == off_c[-1]
    for t in range(off_f.size - 1):
        lf = flat_f[off_f[t]:off_f[t + 1]]
        lc = flat_c[off_c[t]:off_c[t + 1]]
        pos = 0  # lf is walked once
        for item in lc:
            while pos < lf.size and lf[pos] != item:
                pos += 1
            assert pos < lf.size, (t, item)
            pos += 1
    r.forward([0, 1])
    assert np.array_equal(r.read_buffer("tile_offsets").astype(np.int64), off_f)
    assert np.array_equal(r.read_buffer("flatten").astype(np.int64), flat_f)
    r.close()
