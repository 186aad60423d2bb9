"""Autotuner of the batched trainer: tile size and splat-batch depths.

The tile size (8, 16 or 32 pixels) is fixed when a context is created (it
sets the CTA shape of the rasterizers and the tile grid of every view).  The
splat-batch depths -- how many splat records the forward (64, 128, 256) and
the 16x16-tile backward (32, 64, 128) stage in shared memory per batch -- are
kernel variants chosen per step, so they are tuned on a live context.  None
of the three changes a result: images are identical across tile sizes and
depths, gradients differ across tile sizes only in summation order and not
at all across depths, so every candidate does equal work.

`pick_tile_size` builds one context per candidate size on the same scene,
cameras and targets and times a few training steps of the given view sets
with CUDA events on the library's stream.  `autotune` then tunes the forward
depth and the backward depth in turn on the fastest size's context
(coordinate descent: 3 + 2 + 2 timed candidates instead of 27).
"""
from __future__ import annotations

FWD_BATCHES = (64, 128, 256)
BWD_BATCHES = (32, 64, 128)


def _time_steps(r, view_sets, warmup: int) -> float:
    import torch
    stream = torch.cuda.ExternalStream(r.stream())
    for k in range(warmup):
        r.trainStep(view_sets[k % len(view_sets)])
    r.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for vs in view_sets:
        r.trainStep(vs)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / len(view_sets)


def pick_tile_size(make_renderer, view_sets, sizes=(8, 16, 32), warmup: int = 2):
    """make_renderer(tile_size) -> a loaded GaussianRenderer (cameras and
    targets set).  Returns (best tile size, {size: ms per step})."""
    times = {}
    for ts in sizes:
        r = make_renderer(ts)
        try:
            times[ts] = _time_steps(r, view_sets, warmup)
        finally:
            r.close()
    best = min(times, key=times.get)
    return best, times


def autotune(make_renderer, view_sets, sizes=(8, 16, 32), fwd_batches=FWD_BATCHES,
             bwd_batches=BWD_BATCHES, warmup: int = 2):
    """Tile size, then forward and backward splat-batch depths.  Returns
    (tile_size, fwd_batch, bwd_batch, timings) with timings in ms per step:
    {"tile": {size: ms}, "fwd_batch": {depth: ms}, "bwd_batch": {depth: ms}}.
    The backward depth only applies to 16x16 tiles; for other sizes it is
    reported as 0 (default) without timing."""
    ts, tile_times = pick_tile_size(make_renderer, view_sets, sizes, warmup)
    r = make_renderer(ts)
    try:
        fwd_times, bwd_times = {}, {}
        fb, bb = 0, 0
        for d in fwd_batches:
            r.setBatchDepth(d, bb)
            fwd_times[d] = _time_steps(r, view_sets, warmup)
        fb = min(fwd_times, key=fwd_times.get)
        if ts == 16:
            for d in bwd_batches:
                r.setBatchDepth(fb, d)
                bwd_times[d] = _time_steps(r, view_sets, warmup)
            bb = min(bwd_times, key=bwd_times.get)
    finally:
        r.close()
    return ts, fb, bb, {"tile": tile_times, "fwd_batch": fwd_times, "bwd_batch": bwd_times}


__all__ = ["pick_tile_size", "autotune", "FWD_BATCHES", "BWD_BATCHES"]
