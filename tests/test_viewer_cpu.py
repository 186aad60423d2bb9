"""Known answers for the viewer-frame restatement in the oracle
(orc_view_render): one isotropic splat in front of the camera, and the
"over" order of two splats at different depths."""
import math

import numpy as np

from skyfall import scenes

SH_C0 = 0.28209479177387814


def splat_params(points):
    """(59, n) planes: position, isotropic log sigma, identity rotation,
    opacity logit, DC colour; `points` = [(x, y, z, sigma, logit, rgb)]."""
    P = np.zeros((59, len(points)), np.float32)
    for i, (x, y, z, sig, logit, rgb) in enumerate(points):
        P[0:3, i] = (x, y, z)
        P[3:6, i] = math.log(sig)
        P[9, i] = 1.0                       # quaternion w
        P[10, i] = logit
        P[11:14, i] = [(c - 0.5) / SH_C0 for c in rgb]
    return P


def test_single_splat_closed_form(orc):
    W = H = 64
    cam = scenes.cameras_single(W, H, 3.0)[0]
    f = float(cam["focal"][0])
    sig, logit = 0.02, 1.0
    P = splat_params([(0.0, 0.0, 0.0, sig, logit, (0.25, 0.5, 0.75))])
    out = orc.view_render(P, cam, 1.0, 0, round16=0)
    img = out["rgba"].reshape(H, W, 4)
    var = (f * sig / 3.0) ** 2 + 0.3          # C2D diagonal at depth 3
    conic = 1.0 / var
    radius = math.ceil(3.0 * math.sqrt(var))
    op = 1.0 / (1.0 + math.exp(-logit))
    assert out["splats"][0, 9] == radius
    cx = cy = W / 2.0
    for y in range(H):
        for x in range(W):
            px, py = x + 0.5, y + 0.5
            inside = cx - radius <= px < cx + radius and cy - radius <= py < cy + radius
            a = op * math.exp(-0.5 * conic * ((px - cx) ** 2 + (py - cy) ** 2)) if inside else 0.0
            want = [0.25 * a, 0.5 * a, 0.75 * a, a]
            assert np.allclose(img[y, x], want, atol=2e-6), (x, y, img[y, x], want)


def test_far_splat_is_drawn_first(orc):
    W = H = 32
    cam = scenes.cameras_single(W, H, 3.0)[0]
    # camera at z = -3 looking at +z: the splat at z = +1 is farther
    near = (0.0, 0.0, -1.0, 0.05, 0.0, (1.0, 0.0, 0.0))
    far = (0.0, 0.0, 1.0, 0.05, 0.0, (0.0, 0.0, 1.0))
    for order in ([near, far], [far, near]):
        out = orc.view_render(splat_params(order), cam, 1.0, 0, round16=0)
        img = out["rgba"].reshape(H, W, 4)
        c = img[H // 2, W // 2]
        # both splats cover the centre pixel with alpha ~ sigmoid(0) = 0.5
        # times the Gaussian falloff; red (near) is over blue (far)
        assert c[0] > c[2] > 0.0
        k = out["keys"]
        iz_near = order.index(near)
        assert k[iz_near] > k[1 - iz_near]        # ascending key = far first


def test_culled_and_empty(orc):
    W = H = 16
    cam = scenes.cameras_single(W, H, 3.0)[0]
    behind = (0.0, 0.0, -10.0, 0.05, 2.0, (1.0, 1.0, 1.0))   # behind the camera
    out = orc.view_render(splat_params([behind]), cam, 1.0, 0, round16=0)
    assert out["keys"][0] == 0xFFFFFFFF
    assert not out["rgba"].any()
