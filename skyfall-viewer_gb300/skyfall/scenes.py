"""Seeded synthetic scenes and cameras for the benchmark and parity workloads.

The reference trains on COLMAP captures; the workloads here are synthetic
stand-ins with the shapes and value distributions of the benchmark configs:

* small single view: N = 16,384 Gaussians, means U[-1,1]^3, log-scales
  N(-4, 0.3), normalised N(0,1)^4 quaternions, logits N(0,1), SH degree 0
  with colours U[0,1]; one 256x256 pinhole camera, 60 deg fov, distance 3.
* clustered: N Gaussians around 64 cluster centres U[-2,2]^3 (sigma 0.3),
  log-scales N(-4.5, 0.5), SH degree 3 (DC colours U[0,1], higher orders
  N(0, 0.05)), logits N(0, 1.5); cameras on an orbit or a Fibonacci sphere.

Random numbers: SplitMix64 counters (one stream per quantity) feeding
Box-Muller, so every host regenerates the same bits.  Parameters are
rounded to f16-representable values, the reference's storage format, so the
f16 packing of the reference is lossless on them.
"""
from __future__ import annotations

import math

import numpy as np

SH_C0 = 0.28209479177387814
GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def splitmix64(seed: int, stream: int, n: int) -> np.ndarray:
    """n SplitMix64 outputs of the generator seeded with (seed, stream)."""
    with np.errstate(over="ignore"):
        s0 = _mix(np.array([(seed * 0x100000001B3 + stream * 0xD6E8FEB86659FD93) & (2**64 - 1)],
                           dtype=np.uint64))[0]
        idx = np.arange(1, n + 1, dtype=np.uint64)
        return _mix(s0 + idx * GOLDEN)


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """U[0, 1) doubles with 53 random bits."""
    return (splitmix64(seed, stream, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """Standard normal doubles by Box-Muller (cosine branch)."""
    u1 = 1.0 - uniform(seed, 2 * stream, n)      # (0, 1]
    u2 = uniform(seed, 2 * stream + 1, n)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def f16(a: np.ndarray) -> np.ndarray:
    return np.asarray(a, dtype=np.float64).astype(np.float16).astype(np.float32)


def _assemble(pos, logscale, quat, logit, sh) -> np.ndarray:
    n = pos.shape[0]
    P = np.zeros((59, n), dtype=np.float32)
    P[0:3] = f16(pos.T)
    P[3:6] = f16(logscale.T)
    P[6:10] = f16(quat.T)
    P[10] = f16(logit)
    P[11:59] = f16(sh.T)
    return P


def random_quats(seed: int, stream: int, n: int) -> np.ndarray:
    q = normal(seed, stream, 4 * n).reshape(n, 4)
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def scene_uniform(n: int = 16384, seed: int = 1001) -> np.ndarray:
    """Small single-view scene: 59 x n f32 parameter planes (SH degree 0)."""
    pos = uniform(seed, 1, 3 * n).reshape(n, 3) * 2.0 - 1.0
    logscale = -4.0 + 0.3 * normal(seed, 2, 3 * n).reshape(n, 3)
    quat = random_quats(seed, 3, n)
    logit = normal(seed, 4, n)
    sh = np.zeros((n, 48))
    sh[:, 0:3] = (uniform(seed, 5, 3 * n).reshape(n, 3) - 0.5) / SH_C0
    return _assemble(pos, logscale, quat, logit, sh)


def scene_clusters(n: int, seed: int = 1002, clusters: int = 64, center_range: float = 2.0,
                   cluster_sigma: float = 0.3, logscale_mean: float = -4.5,
                   logscale_sigma: float = 0.5, logit_sigma: float = 1.5, sh_degree: int = 3,
                   sh_rest_sigma: float = 0.05) -> np.ndarray:
    """Clustered scene: n Gaussians around `clusters` centres."""
    centers = (uniform(seed, 10, 3 * clusters).reshape(clusters, 3) * 2.0 - 1.0) * center_range
    which = (uniform(seed, 11, n) * clusters).astype(np.int64).clip(0, clusters - 1)
    pos = centers[which] + cluster_sigma * normal(seed, 12, 3 * n).reshape(n, 3)
    logscale = logscale_mean + logscale_sigma * normal(seed, 13, 3 * n).reshape(n, 3)
    quat = random_quats(seed, 14, n)
    logit = logit_sigma * normal(seed, 15, n)
    sh = np.zeros((n, 48))
    sh[:, 0:3] = (uniform(seed, 16, 3 * n).reshape(n, 3) - 0.5) / SH_C0
    ncoef = (sh_degree + 1) ** 2
    if ncoef > 1:
        sh[:, 3:3 * ncoef] = sh_rest_sigma * normal(seed, 17, (3 * ncoef - 3) * n).reshape(n, -1)
    return _assemble(pos, logscale, quat, logit, sh)


# ---------------------------------------------------------------------------
# Cameras
# ---------------------------------------------------------------------------

def look_at(eye, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """World->camera matrix (column-major, 16 f32) with camera x right, y up,
    z forward: the convention under which the reference's pinhole projection
    puts pixel y = H - cy - fy * y / z."""
    eye = np.asarray(eye, dtype=np.float64)
    f = np.asarray(target, dtype=np.float64) - eye
    f /= np.linalg.norm(f)
    upv = np.asarray(up, dtype=np.float64)
    if abs(np.dot(f, upv)) > 0.999:
        upv = np.array([0.0, 0.0, 1.0])
    r = np.cross(upv, f)
    r /= np.linalg.norm(r)
    u = np.cross(f, r)
    R = np.stack([r, u, f])          # rows
    t = -R @ eye
    M = np.eye(4)
    M[:3, :3] = R
    M[:3, 3] = t
    return M.T.reshape(-1).astype(np.float32)   # column-major


def pinhole(view: np.ndarray, fx: float, fy: float, cx: float, cy: float, w: int, h: int) -> dict:
    """Camera dict with the projection of get_pinhole_projection_matrix
    (src/camera/training-camera.ts:29-52), f64 arithmetic, f32 storage."""
    sx, sy = 2.0 * fx / w, -2.0 * fy / h
    ox, oy = 2.0 * cx / w - 1.0, 1.0 - 2.0 * cy / h
    P = np.zeros(16, dtype=np.float64)
    P[0 * 4 + 0] = sx
    P[1 * 4 + 1] = sy
    P[2 * 4 + 0] = ox
    P[2 * 4 + 1] = oy
    P[2 * 4 + 2] = 1.0
    P[2 * 4 + 3] = 1.0
    return dict(view=np.asarray(view, dtype=np.float32), proj=P.astype(np.float32),
                focal=np.array([fx, fy], dtype=np.float32), width=int(w), height=int(h))


def camera_fov(eye, w: int, h: int, fov_y_deg: float = 60.0, target=(0.0, 0.0, 0.0)) -> dict:
    f = (h / 2.0) / math.tan(math.radians(fov_y_deg) / 2.0)
    return pinhole(look_at(eye, target), f, f, w / 2.0, h / 2.0, w, h)


def cameras_single(w: int = 256, h: int = 256, distance: float = 3.0) -> list[dict]:
    return [camera_fov((0.0, 0.0, -distance), w, h)]


def cameras_orbit(count: int, radius: float, w: int, h: int, height: float = 0.8) -> list[dict]:
    out = []
    for k in range(count):
        a = 2.0 * math.pi * k / count
        out.append(camera_fov((radius * math.cos(a), height, radius * math.sin(a)), w, h))
    return out


def cameras_fibonacci(count: int, radius: float, w: int, h: int) -> list[dict]:
    out = []
    ga = math.pi * (3.0 - math.sqrt(5.0))
    for k in range(count):
        y = 1.0 - 2.0 * (k + 0.5) / count
        r = math.sqrt(max(0.0, 1.0 - y * y))
        out.append(camera_fov((radius * r * math.cos(ga * k), radius * y, radius * r * math.sin(ga * k)), w, h))
    return out


def cameras_mixed(count: int, radius: float, seed: int = 2004) -> list[dict]:
    """`count` cameras on a Fibonacci sphere with resolutions drawn uniformly
    from 640x480, 1280x720 and 1920x1080."""
    sizes = [(640, 480), (1280, 720), (1920, 1080)]
    pick = (uniform(seed, 1, count) * 3).astype(np.int64).clip(0, 2)
    base = cameras_fibonacci(count, radius, 16, 16)
    out = []
    for cam, k in zip(base, pick):
        w, h = sizes[int(k)]
        f = (h / 2.0) / math.tan(math.radians(60.0) / 2.0)
        out.append(pinhole(cam["view"], f, f, w / 2.0, h / 2.0, w, h))
    return out


def target_uniform(w: int, h: int, seed: int = 2001) -> np.ndarray:
    """Seeded U[0,1] RGB f32 image, (h, w, 3)."""
    return uniform(seed, 1, w * h * 3).astype(np.float32).reshape(h, w, 3)
