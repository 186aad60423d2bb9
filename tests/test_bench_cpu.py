"""Host logic of bench.py that the reported numbers rest on: the matched-loss
interpolation, the algorithmic bytes per stage, the scaling of the small
case's measured DRAM bytes to the bench's launch, and the rasterizers' work
shares from the pair counters."""
import json

import pytest


@pytest.fixture(scope="module")
def bench():
    import bench as b
    return b


def test_interp_time_crossing_and_edges(bench):
    curve = [(0.0, 1.0), (1.0, 0.5), (2.0, 0.25)]
    assert bench.interp_time(curve, 0.75) == pytest.approx(0.5)   # halfway down the first leg
    assert bench.interp_time(curve, 0.5) == pytest.approx(1.0)    # an evaluation itself
    assert bench.interp_time(curve, 0.3) == pytest.approx(1.8)
    assert bench.interp_time(curve, 0.1) is None                  # never reached
    assert bench.interp_time([(0.0, 0.2), (1.0, 0.1)], 0.3) == 0.0  # below from the start


def test_algo_bytes_per_unit_figures(bench):
    # backward: 100 B per intersection (record, item index, partial), 28 B per pixel
    assert bench.algo_bytes("backward", 1, 1, 10, 3) == 10 * 100 + 3 * 28
    assert bench.algo_bytes("forward", 1, 1, 10, 3) == 10 * 60 + 3 * 60
    assert bench.algo_bytes("sort", 1, 1, 10, 0) == 10 * 36
    assert bench.algo_bytes("preprocess", 5, 2, 0, 0) == 5 * 236 + 10 * 72
    with pytest.raises(KeyError):
        bench.algo_bytes("nonexistent", 1, 1, 1, 1)


def test_measured_traffic_scales_the_small_case(bench):
    d = json.loads((bench.REPO / "profiles" / "traffic.json").read_text())
    for stage in ("backward", "forward", "geom_adam"):
        e = d[stage]
        small = e["small_case"]
        # at the small case itself the scale is one: the measured bytes come back
        got, src = bench.measured_traffic(stage, e["bench_workload"], small["n"], small["views"],
                                          small["isect_per_launch"], small["pixels_per_launch"])
        assert got == pytest.approx(e["bytes_per_launch"])
        assert e["kernel"] in src and "profiles/traffic.json" in src
        # twice the work of every kind: twice the bytes
        got2, _ = bench.measured_traffic(stage, e["bench_workload"], 2 * small["n"], small["views"],
                                         2 * small["isect_per_launch"], 2 * small["pixels_per_launch"])
        assert got2 == pytest.approx(2 * e["bytes_per_launch"])
    # another workload has no capture to scale from
    assert bench.measured_traffic("backward", "another/ts16/cull", 1, 1, 1.0, 1.0) == (None, None)


def test_measured_traffic_of_the_bench_step(bench):
    """The default step (1M Gaussians, 16 views of 1920x1080, 56.4M culled
    intersections): the backward's traffic is the small case's bytes times
    the algorithmic-byte ratio, below the algorithmic bytes themselves."""
    isect, pix = 56.36e6, 16 * 1920 * 1080
    got, _ = bench.measured_traffic("backward", "train1080/ts16/cull", 1_000_000, 16, isect, pix)
    algo = bench.algo_bytes("backward", 1_000_000, 16, isect, pix)
    assert 0.3 * algo < got < algo


def test_pair_stats_shares(bench):
    # forward: 64 evaluated, 32 contributing, 4 warp entries; backward: 100
    # evaluated, 40 contributing, 2 entries, 1 of them without a contribution
    s = bench.pair_stats([64, 32, 4, 100, 40, 2, 1, 0])
    assert s["forward"]["lane_use"] == pytest.approx(64 / 128)
    assert s["forward"]["contributing_share"] == pytest.approx(0.5)
    assert s["backward"]["slot_use"] == pytest.approx(100 / 128)
    assert s["backward"]["contributing_share"] == pytest.approx(0.4)
    assert s["backward"]["entries_without_contribution"] == pytest.approx(0.5)
    # per step over two steps
    s2 = bench.pair_stats([64, 32, 4, 100, 40, 2, 1, 0], steps=2)
    assert s2["backward"]["pairs_evaluated"] == pytest.approx(50)
    assert bench.pair_stats(None) is None
    assert bench.pair_stats([1, 1, 0, 1, 1, 1, 0, 0]) is None  # no forward entries counted
