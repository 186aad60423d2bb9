"""The ellipse tests that skip work, checked on the CPU (no GPU).

Both use the analytic x-extent of the ellipse s = 0.5 (a dx^2 + c dy^2) +
b dx dy <= 1.001 smax within a band of pixel rows.  Before the exact backward
walks a batch of splats, each splat's bounding-box block mask is narrowed: an
8x8 pixel block is dropped when its pixel-centre columns miss that extent
within its 8 rows.  With culled intersection lists, each tile row of a
Gaussian's rectangle lists only the tiles whose columns meet the extent
within the row.  Dropping a block or tile that holds a pixel with f32
s <= smax would lose that pixel's contribution.  These tests restate the f32
arithmetic (ellipse_rows, band_extent, ellipse_band_mask and row_span in
kernels.cu) in numpy, one rounding per operation, and check it against the
rasterisers' own f32 evaluation of s at every pixel centre, on random splats
with anisotropy up to the conditioning limit (b^2 <= 0.98 a c) and means on
both sides of the edges.  The kernels evaluate the extents' square roots and
quotients with sqrt.approx and the fast division (relative errors below
2^-22); the tests run the restatement exact and with every square root and
quotient moved by a relative 2e-6 in the direction that narrows the extent.
"""
import numpy as np
import pytest

f = np.float32


def kernel_s(a, b, c, mx, my, px, py):
    """The rasterisers' f32 evaluation of s at a pixel centre."""
    dx = px - mx
    dy = py - my
    s1 = (a * dx) * dx
    s2 = (c * dy) * dy
    so2 = f(0.5) * (s1 + s2)
    return so2 + (b * dx) * dy


def down(x, rel):
    """x moved by the relative amount rel towards -inf (an approximate
    square root or quotient at its worst for a narrowing extent)."""
    return (x - f(rel) * np.abs(x)).astype(f) if rel else x


def up(x, rel):
    return (x + f(rel) * np.abs(x)).astype(f) if rel else x


def band_extent(a, b, c, mx, my, smax, v0, v1, rel=0.0, vr_sign=1.0):
    """ellipse_rows + band_extent (kernels.cu) in f32, elementwise: whether
    the band of pixel-centre rows with dy in [v0, v1] meets the ellipse, and
    its x-extent [ul, ur] relative to the mean there (margins included).
    rel > 0 perturbs every square root and quotient adversarially (vr_sign
    picks the direction of the edge maximum's abscissa)."""
    L = f(1.001) * smax
    det = a * c - b * b
    U = down(np.sqrt(down(f(2) * c * L / det, rel)), rel)
    two_a_l = f(2) * a * L
    V = down(np.sqrt(down(two_a_l / det, rel)), rel)
    v_margin = f(1.01) * V + f(0.05)
    u_margin = f(0.01) * U + f(0.05)
    v_right = -b * U / c
    v_right = (up(v_right, rel) if vr_sign > 0 else down(v_right, rel)) if rel else v_right
    meets = ~((v1 < -v_margin) | (v0 > v_margin))
    w0, w1 = np.maximum(v0, -V), np.minimum(v1, V)
    vr = np.minimum(np.maximum(v_right, w0), w1)
    vl = np.minimum(np.maximum(-v_right, w0), w1)
    # a band beyond E's top or bottom row (within the margin): that row's extent
    beyond = w0 > w1
    tip = np.where(v0 > 0, V, -V)
    vr = np.where(beyond, tip, vr)
    vl = np.where(beyond, tip, vl)
    dr = np.maximum(two_a_l - det * vr * vr, f(0))
    dl = np.maximum(two_a_l - det * vl * vl, f(0))
    ur = down((-b * vr + down(np.sqrt(dr), rel)) / a, rel) + u_margin
    ul = up((-b * vl - down(np.sqrt(dl), rel)) / a, rel) - u_margin
    return meets, ul, ur


def block_dropped(a, b, c, mx, my, smax, x0, y0, bw, bh, rel=0.0, vr_sign=1.0):
    """ellipse_band_mask's decision for one bw x bh block at (x0, y0)."""
    cond = (a > 0) & (c > 0) & (b * b <= f(0.98) * (a * c)) & (smax > 0)
    with np.errstate(invalid="ignore", divide="ignore"):
        cy = f(y0) + f(0.5)
        meets, ul, ur = band_extent(a, b, c, mx, my, smax, cy - my, (cy + f(bh - 1)) - my,
                                    rel, vr_sign)
        xl, xr = mx + ul, mx + ur
        cx = f(x0) + f(0.5)
        kept = meets & (xr >= cx) & (xl <= cx + f(bw - 1))
    return cond & ~kept


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


@pytest.mark.parametrize("rel,vr_sign,bw,bh", [(0.0, 1.0, 8, 8), (2e-6, 1.0, 8, 8), (2e-6, -1.0, 8, 8),
                                              (2e-6, 1.0, 8, 4), (2e-6, -1.0, 8, 4)])
def test_dropped_blocks_hold_no_pixel_within_smax(rel, vr_sign, bw, bh):
    """8x8 blocks (backward) and 8x4 blocks (forward), exact and with the
    approximate operations' worst case."""
    rng = np.random.default_rng(11)
    total_dropped = 0
    for x0, y0 in ((0, 0), (1000, 500), (3832, 2152)):
        a, b, c, mx, my, smax = random_splats(rng, 60000, x0, y0)
        live = smax > 0
        drop = block_dropped(a, b, c, mx, my, smax, x0, y0, bw, bh, rel, vr_sign) & live
        reach = np.zeros_like(drop)
        for yy in range(bh):
            for xx in range(bw):
                s = kernel_s(a, b, c, mx, my, f(x0 + xx) + f(0.5), f(y0 + yy) + f(0.5))
                reach |= (s >= 0) & (s <= smax)
        assert not (drop & reach).any()
        # and the test is not vacuous: it drops nearly every block no pixel reaches
        assert drop.sum() >= 0.95 * (live & ~reach).sum()
        total_dropped += int(drop.sum())
    assert total_dropped > 50000


def row_span(a, b, c, mx, my, smax, ty, x0, x1, ts, rel=0.0, vr_sign=1.0):
    """row_span (kernels.cu) in f32: the listed tiles [lo, lo + len) of tile
    row ty of the rectangle [x0, x1)."""
    cy = f(ty * ts) + f(0.5)
    meets, ul, ur = band_extent(a, b, c, mx, my, smax, cy - my, (cy + f(ts - 1)) - my, rel, vr_sign)
    if not meets:
        return x0, 0
    fts = f(ts)
    t_lo = np.ceil(up(((mx + ul) - (fts - f(0.5))) / fts, rel))
    t_hi = np.floor(down(((mx + ur) - f(0.5)) / fts, rel))
    flo, fhi = max(t_lo, f(x0)), min(t_hi, f(x1 - 1))
    if not fhi >= flo:
        return x0, 0
    return int(flo), int(fhi) - int(flo) + 1


@pytest.mark.parametrize("ts,rel,vr_sign", [(8, 0.0, 1.0), (16, 0.0, 1.0), (32, 0.0, 1.0),
                                             (16, 2e-6, 1.0), (16, 2e-6, -1.0), (8, 2e-6, 1.0)])
def test_row_spans_list_every_reached_tile(ts, rel, vr_sign):
    """The culled intersection lists: per tile row of a Gaussian's rectangle,
    the analytic span of its ellipse must hold every tile with a pixel whose
    f32 s passes the pre-filter, and list few tiles beyond those."""
    rng = np.random.default_rng(20 + ts)
    a, b, c, mx, my, smax = random_splats(rng, 1500, 1000, 500)
    l_max = np.maximum(1.0 / a, 1.0 / c) * 4.0  # generous radius for the rectangle
    reached = listed = 0
    for i in range(a.size):
        if not (smax[i] > 0 and b[i] * b[i] <= f(0.98) * (a[i] * c[i])):
            continue
        rad = int(np.ceil(3 * np.sqrt(l_max[i])))
        x0, x1 = int(np.floor((mx[i] - rad) / ts)), int(np.ceil((mx[i] + rad) / ts))
        y0, y1 = int(np.floor((my[i] - rad) / ts)), int(np.ceil((my[i] + rad) / ts))
        for ty in range(y0, y1):
            lo, n = row_span(a[i], b[i], c[i], mx[i], my[i], smax[i], ty, x0, x1, ts, rel, vr_sign)
            listed += n
            ys = f(ty * ts) + f(0.5) + np.arange(ts, dtype=f)
            for tx in range(x0, x1):
                xs = f(tx * ts) + f(0.5) + np.arange(ts, dtype=f)
                X, Y = np.meshgrid(xs, ys)
                s = kernel_s(a[i], b[i], c[i], mx[i], my[i], X, Y)
                if ((s >= 0) & (s <= smax[i])).any():
                    reached += 1
                    assert lo <= tx < lo + n, (i, ty, tx, lo, n)
    assert reached > 1000
    assert listed <= 1.1 * reached


def test_bands_beyond_the_extreme_rows_get_the_tip_extent():
    """A band of rows wholly beyond E's top or bottom row but within the
    row margin (the f32 rounding allowance) still 'meets' E; its extent is
    that of the extreme row: it holds the tip -b v / a at v = +-V and every
    pixel of the band that passes the f32 pre-filter."""
    rng = np.random.default_rng(31)
    a, b, c, mx, my, smax = random_splats(rng, 40000, 0, 0)
    keep = (smax > 0) & (b * b <= f(0.98) * (a * c))
    a, b, c, mx, my, smax = (x[keep] for x in (a, b, c, mx, my, smax))
    L = f(1.001) * smax
    det = a * c - b * b
    V = np.sqrt(f(2) * a * L / det)
    vm = f(1.01) * V + f(0.05)
    for side in (1.0, -1.0):
        # a one-row band strictly between V and the margin, below or above
        t = rng.random(a.size).astype(f)
        vb = (f(side) * (V + (vm - V) * (f(0.05) + f(0.9) * t))).astype(f)
        beyond = np.abs(vb) > V
        meets, ul, ur = band_extent(a, b, c, mx, my, smax, vb, vb)
        assert meets[beyond].all()
        tipu = -b * (f(side) * V) / a
        assert ((ul <= tipu) & (tipu <= ur))[beyond].all()
        # pixels of that row: any that passes the f32 test lies in the extent
        for du in np.linspace(-40, 40, 161, dtype=f):
            px, py = mx + du, my + vb
            s = kernel_s(a, b, c, mx, my, px, py)
            ok = (s >= 0) & (s <= smax) & beyond
            rel = px - mx
            assert not (ok & ((rel < ul) | (rel > ur))).any()


def test_ill_conditioned_conics_are_never_dropped():
    # |b| close to sqrt(a c): the rounding bound no longer holds, the mask stays
    a = np.array([1.0, 4.0], f)
    c = np.array([1.0, 0.25], f)
    b = np.sqrt(a * c) * f(0.995)
    smax = np.array([0.5, 0.5], f)
    mx = np.array([-30.0, -30.0], f)
    my = np.array([-30.0, -30.0], f)
    assert not block_dropped(a, b, c, mx, my, smax, 0, 0, 8, 8).any()
