"""Tile-size autotuner for the batched trainer.

The tile size (8, 16 or 32 pixels) is fixed when a context is created (it
sets the CTA shape of the rasterizers and the tile grid of every view), and
the splat-batch depth of each rasterizer follows from it (256 records per
forward batch; 64 per backward batch for 8x8 and 16x16 tiles, 16 for 32x32).
`pick_tile_size` builds one context per candidate on the same scene,
cameras and targets, times a few training steps of the given view sets with
CUDA events on the library's stream, and returns the fastest size with all
timings.  Images are identical across tile sizes; gradients differ only in
summation order, so the candidates do equal work.
"""
from __future__ import annotations


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


__all__ = ["pick_tile_size"]
