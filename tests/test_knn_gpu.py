"""GPU k-NN scale initialisation (grid search) against the oracle's
all-pairs scan of knn-init.wgsl: mean distances and the f16 log sigmas must
be identical; every other parameter is re-read through f16."""
import numpy as np
import pytest

from skyfall import scenes

pytestmark = pytest.mark.gpu


def f16(a):
    return a.astype(np.float32).astype(np.float16).astype(np.float32)


@pytest.mark.parametrize("kind", ["uniform", "clusters", "duplicates"])
def test_knn_matches_all_pairs(sky, orc, kind):
    if kind == "uniform":
        P = scenes.scene_uniform(6000, seed=1401)
    elif kind == "clusters":
        P = scenes.scene_clusters(6000, seed=1402)
    else:
        # many points collapse onto the same f16 position
        P = scenes.scene_uniform(3000, seed=1403)
        P[0:3] = np.round(P[0:3] * 20.0) / 20.0
    r = sky.GaussianRenderer()
    r.load_points(P)
    ext = r.getStatus().scene_extent
    dens = r.initializeKnnAndSync()
    want_d, want_ls = orc.knn_init(P, ext)
    assert np.array_equal(dens, want_d)
    Q = r.params()
    for k in range(3, 6):
        assert np.array_equal(Q[k], want_ls)
    other = [k for k in range(59) if k not in (3, 4, 5)]
    assert np.array_equal(Q[other], f16(P[other]))


@pytest.mark.parametrize("n", [1, 2, 4])
def test_knn_tiny_scenes(sky, orc, n):
    P = scenes.scene_uniform(64, seed=1404)[:, :n].copy()
    r = sky.GaussianRenderer()
    r.load_points(P)
    dens = r.initializeKnnAndSync(scene_extent=2.0)
    want_d, want_ls = orc.knn_init(P, 2.0)
    assert np.array_equal(dens, want_d)
    assert np.array_equal(r.params()[3], want_ls)
