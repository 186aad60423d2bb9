"""The backward's per-block ellipse test, checked on the CPU (no GPU).

Before the exact backward walks a batch of splats, each splat's bounding-box
block mask is narrowed block by block: an 8x8 pixel block is dropped when the
minimum of s = 0.5 (a dx^2 + c dy^2) + b dx dy over the block's rectangle of
pixel centres, evaluated in f32 along the rectangle's edges, exceeds
1.001 smax.  Dropping a block that holds a pixel with f32 s <= smax would
lose that pixel's contribution.  This test restates the test's f32
arithmetic (ellipse_mask in kernels.cu) in numpy, one rounding per
operation, and checks it against the kernels' own f32 evaluation of s at
every pixel centre of the block, on random splats with anisotropy up to the
test's conditioning limit (b^2 <= 0.98 a c) and means on both sides of the
block's edges.
"""
import numpy as np

f = np.float32


def kernel_s(a, b, c, mx, my, px, py):
    """The rasterisers' f32 evaluation of s at a pixel centre."""
    dx = px - mx
    dy = py - my
    s1 = (a * dx) * dx
    s2 = (c * dy) * dy
    so2 = f(0.5) * (s1 + s2)
    return so2 + (b * dx) * dy


def block_dropped(a, b, c, mx, my, smax, x0, y0, bw, bh):
    cond = (a > 0) & (c > 0) & (b * b <= f(0.98) * (a * c))
    ku = -(b / c)
    kv = -(b / a)

    def s_at(u, v):
        return f(0.5) * ((a * u) * u + (c * v) * v) + (b * u) * v

    def clamp(x, lo, hi):
        return np.minimum(np.maximum(x, lo), hi)

    cx = f(x0) + f(0.5)
    cy = f(y0) + f(0.5)
    u0 = cx - mx
    u1 = (cx + f(bw - 1)) - mx
    v0 = cy - my
    v1 = (cy + f(bh - 1)) - my
    holds_mean = (u0 <= 0) & (u1 >= 0) & (v0 <= 0) & (v1 >= 0)
    smin = s_at(u0, clamp(ku * u0, v0, v1))
    smin = np.minimum(smin, s_at(u1, clamp(ku * u1, v0, v1)))
    smin = np.minimum(smin, s_at(clamp(kv * v0, u0, u1), v0))
    smin = np.minimum(smin, s_at(clamp(kv * v1, u0, u1), v1))
    return cond & ~holds_mean & (smin > f(1.001) * smax)


def random_splats(rng, n, x0, y0):
    l1 = f(0.3) + rng.exponential(20.0, n).astype(f)
    l2 = f(0.3) + (rng.exponential(3.0, n) * (rng.random(n) < 0.5)).astype(f)
    th = (rng.random(n) * np.pi).astype(f)
    ct, st = np.cos(th), np.sin(th)
    c00 = l1 * ct * ct + l2 * st * st
    c11 = l1 * st * st + l2 * ct * ct
    c01 = (l1 - l2) * ct * st
    det = c00 * c11 - c01 * c01
    a, c, b = (c11 / det).astype(f), (c00 / det).astype(f), (-c01 / det).astype(f)
    op = (rng.random(n) * 0.99 + 0.005).astype(f)
    smax = (np.log(f(255) * op) + f(1e-3)).astype(f)
    mx = (rng.random(n) * 60 - 26).astype(f) + f(x0)
    my = (rng.random(n) * 60 - 26).astype(f) + f(y0)
    return a, b, c, mx, my, smax


def test_dropped_blocks_hold_no_pixel_within_smax():
    rng = np.random.default_rng(11)
    total_dropped = 0
    for x0, y0 in ((0, 0), (1000, 500), (3832, 2152)):
        a, b, c, mx, my, smax = random_splats(rng, 60000, x0, y0)
        live = smax > 0
        drop = block_dropped(a, b, c, mx, my, smax, x0, y0, 8, 8) & live
        reach = np.zeros_like(drop)
        for yy in range(8):
            for xx in range(8):
                s = kernel_s(a, b, c, mx, my, f(x0 + xx) + f(0.5), f(y0 + yy) + f(0.5))
                reach |= (s >= 0) & (s <= smax)
        assert not (drop & reach).any()
        # and the test is not vacuous: it drops nearly every block no pixel reaches
        assert drop.sum() >= 0.95 * (live & ~reach).sum()
        total_dropped += int(drop.sum())
    assert total_dropped > 50000


def test_ill_conditioned_conics_are_never_dropped():
    # |b| close to sqrt(a c): the rounding bound no longer holds, the mask stays
    a = np.array([1.0, 4.0], f)
    c = np.array([1.0, 0.25], f)
    b = np.sqrt(a * c) * f(0.995)
    smax = np.array([0.5, 0.5], f)
    mx = np.array([-30.0, -30.0], f)
    my = np.array([-30.0, -30.0], f)
    assert not block_dropped(a, b, c, mx, my, smax, 0, 0, 8, 8).any()
