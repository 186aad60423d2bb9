"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the C++ oracle (oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, and only as the checker or the timed CPU baseline; the product
never imports it.  build() compiles oracle.cpp with g++ (-ffp-contract=off)
into oracle/_build/liboracle.so.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.cpp"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
               "-shared", "-pthread", str(SRC), "-o", str(LIB)]
        subprocess.run(cmd, check=True)
    return LIB


class OrcCam(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("focal", C.c_float * 2),
                ("width", C.c_uint32), ("height", C.c_uint32)]


class OrcSettings(C.Structure):
    _fields_ = [("tile_size", C.c_uint32), ("near_plane", C.c_float), ("far_plane", C.c_float),
                ("radius_clip", C.c_float), ("eps2d", C.c_float), ("bg", C.c_float * 3),
                ("w_l2", C.c_float), ("w_l1", C.c_float), ("w_ssim", C.c_float),
                ("round_f16", C.c_uint32), ("nthreads", C.c_uint32)]


_lib = None
P = C.c_void_p


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_project.argtypes = [P, C.c_uint64, C.c_uint32, P, P, C.c_int, P, P, P, P, P]
        L.orc_tiles.argtypes = [P, P, P, C.c_uint32, P, P, P, P, P, P, P, P]
        L.orc_forward.argtypes = [P, C.c_uint32, P, P, P, P, P, P, P, P]
        L.orc_loss.argtypes = [P, P, P, P, P, P]
        L.orc_backward.argtypes = [P, C.c_uint32, P, P, C.c_int, C.c_int, P, P, P, P, P, P, P, P, P, P, P]
        L.orc_geom.argtypes = [P, C.c_uint64, C.c_uint32, P, P, C.c_int, C.c_int, P, P, C.c_uint64]
        L.orc_adam.argtypes = [P, P, P, P, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_float,
                               C.c_float, C.c_float]
        L.orc_loss_f64.argtypes = [P, C.c_uint64, C.c_uint32, P, P, C.c_int, P, P]
        L.orc_loss_f64.restype = C.c_double
        L.orc_expf.argtypes = [P, P, C.c_uint64]
        L.orc_round_f16.argtypes = [P, P, C.c_uint64]
        L.orc_view_render.argtypes = [P, C.c_uint64, C.c_uint32, P, C.c_float, C.c_uint32,
                                      C.c_uint32, P, P, P]
        L.orc_logf.argtypes = [P, P, C.c_uint64]
        L.orc_knn_init.argtypes = [P, C.c_uint64, C.c_uint32, C.c_float, P, P, C.c_uint32]
        _lib = L
    return _lib


def ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def cam_struct(cam: dict) -> OrcCam:
    c = OrcCam()
    c.view = (C.c_float * 16)(*np.asarray(cam["view"], np.float32).reshape(16))
    c.proj = (C.c_float * 16)(*np.asarray(cam["proj"], np.float32).reshape(16))
    c.focal = (C.c_float * 2)(*np.asarray(cam["focal"], np.float32).reshape(2))
    c.width, c.height = int(cam["width"]), int(cam["height"])
    return c


def settings(cfg=None, nthreads: int | None = None, **kw) -> OrcSettings:
    """Oracle settings from a SkyConfig-like object (attribute access) or
    keyword overrides; defaults are the reference's."""
    d = dict(tile_size=16, near_plane=0.2, far_plane=10000.0, radius_clip=512.0, eps2d=0.3,
             bg=(0.0, 0.0, 0.0), w_l2=0.0, w_l1=0.8, w_ssim=0.2, round_f16=1)
    if cfg is not None:
        for k in ("tile_size", "near_plane", "far_plane", "radius_clip", "eps2d", "w_l2", "w_l1", "w_ssim"):
            d[k] = getattr(cfg, k)
        d["bg"] = tuple(cfg.background)
        d["round_f16"] = cfg.round_params_f16
    d.update(kw)
    s = OrcSettings()
    for k, v in d.items():
        if k == "bg":
            s.bg = (C.c_float * 3)(*v)
        else:
            setattr(s, k, v)
    s.nthreads = nthreads if nthreads is not None else (os.cpu_count() or 1)
    return s


def expf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    lib().orc_expf(ptr(x), ptr(y), x.size)
    return y


def round_f16(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    lib().orc_round_f16(ptr(x), ptr(y), x.size)
    return y


def tiles_wh(cam, ts):
    return (cam["width"] + ts - 1) // ts, (cam["height"] + ts - 1) // ts


def project(params: np.ndarray, cam: dict, s: OrcSettings, sh_deg: int) -> dict:
    params = np.ascontiguousarray(params, np.float32)
    n = params.shape[1]
    rec = np.empty((n, 12), np.float32)
    counts = np.empty(n, np.uint32)
    rects = np.empty((n, 4), np.uint32)
    raw = np.empty((n, 3), np.float32)
    dirs = np.empty((n, 3), np.float32)
    c = cam_struct(cam)
    lib().orc_project(ptr(params), n, n, C.byref(c), C.byref(s), sh_deg, ptr(rec), ptr(counts),
                      ptr(rects), ptr(raw), ptr(dirs))
    return dict(rec=rec, counts=counts, rects=rects, raw=raw, dirs=dirs)


def tiles(pr: dict, cam: dict, s: OrcSettings) -> dict:
    n = pr["counts"].shape[0]
    I = int(pr["counts"].astype(np.uint64).sum())
    tw, th = tiles_wh(cam, s.tile_size)
    out = dict(cumsum=np.empty(n, np.uint32), keys_emit=np.empty(I, np.uint32),
               gidx_emit=np.empty(I, np.uint32), keys_sorted=np.empty(I, np.uint32),
               gidx_sorted=np.empty(I, np.uint32), offsets=np.empty(tw * th + 1, np.uint32))
    c = cam_struct(cam)
    lib().orc_tiles(ptr(pr["rec"]), ptr(pr["counts"]), ptr(pr["rects"]), n, C.byref(c), C.byref(s),
                    ptr(out["cumsum"]), ptr(out["keys_emit"]), ptr(out["gidx_emit"]),
                    ptr(out["keys_sorted"]), ptr(out["gidx_sorted"]), ptr(out["offsets"]))
    return out


def forward(pr: dict, tl: dict, cam: dict, s: OrcSettings) -> dict:
    n = pr["rec"].shape[0]
    P = cam["width"] * cam["height"]
    out = dict(rgba=np.empty((P, 4), np.float32), alpha=np.empty(P, np.float32),
               last=np.empty(P, np.uint32), tprod=np.empty(P, np.float32))
    c = cam_struct(cam)
    lib().orc_forward(ptr(pr["rec"]), n, C.byref(c), C.byref(s), ptr(tl["gidx_sorted"]),
                      ptr(tl["offsets"]), ptr(out["rgba"]), ptr(out["alpha"]), ptr(out["last"]),
                      ptr(out["tprod"]))
    return out


def loss(fw: dict, target: np.ndarray, cam: dict, s: OrcSettings) -> dict:
    P = cam["width"] * cam["height"]
    t = np.ascontiguousarray(target, np.float32).reshape(P, 3)
    res = np.empty((P, 4), np.float32)
    l = C.c_double()
    c = cam_struct(cam)
    lib().orc_loss(ptr(fw["rgba"]), ptr(t), C.byref(c), C.byref(s), ptr(res), C.byref(l))
    return dict(residual=res, loss=l.value)


def backward(pr: dict, tl: dict, fw: dict, ls: dict, cam: dict, s: OrcSettings, mode: int,
             sh_deg: int) -> dict:
    n = pr["rec"].shape[0]
    I = tl["keys_sorted"].shape[0]
    c = cam_struct(cam)
    out = {}
    if mode == 0:
        out["gsum9"] = np.zeros((n, 9), np.float64)
        out["gabs9"] = np.zeros((n, 9), np.float64)
        lib().orc_backward(ptr(pr["rec"]), n, C.byref(c), C.byref(s), 0, sh_deg, ptr(pr["dirs"]),
                           ptr(tl["gidx_sorted"]), ptr(tl["offsets"]), ptr(fw["alpha"]),
                           ptr(fw["last"]), ptr(fw["tprod"]), ptr(ls["residual"]), ptr(out["gsum9"]),
                           ptr(out["gabs9"]),
                           None, None)
    else:
        out["tile_grads"] = np.zeros((I, 54), np.int32)
        out["gsum54"] = np.zeros((n, 54), np.int64)
        lib().orc_backward(ptr(pr["rec"]), n, C.byref(c), C.byref(s), 1, sh_deg, ptr(pr["dirs"]),
                           ptr(tl["gidx_sorted"]), ptr(tl["offsets"]), ptr(fw["alpha"]),
                           ptr(fw["last"]), ptr(fw["tprod"]), ptr(ls["residual"]), None, None,
                           ptr(out["tile_grads"]),
                           ptr(out["gsum54"]))
    return out


def geom(params: np.ndarray, cam: dict, s: OrcSettings, sh_deg: int, g9: np.ndarray,
         grads: np.ndarray | None = None, with_sh: bool = True) -> np.ndarray:
    """Exact adjoint; accumulates into grads (59, n) f32 (allocated if None)."""
    params = np.ascontiguousarray(params, np.float32)
    n = params.shape[1]
    if grads is None:
        grads = np.zeros((59, n), np.float32)
    g9f = np.ascontiguousarray(g9, np.float32)
    c = cam_struct(cam)
    lib().orc_geom(ptr(params), n, n, C.byref(c), C.byref(s), sh_deg, int(with_sh), ptr(g9f),
                   ptr(grads), n)
    return grads


def adam(p, m1, m2, g, lr, beta1, beta2, eps, bc1_rcp, bc2_sqrt_rcp):
    """In place on contiguous f32 arrays."""
    lib().orc_adam(ptr(p), ptr(m1), ptr(m2), ptr(g), p.size, lr, beta1, beta2, eps, bc1_rcp,
                   bc2_sqrt_rcp)


def loss_f64(params64: np.ndarray, cam: dict, s: OrcSettings, sh_deg: int, target: np.ndarray):
    p = np.ascontiguousarray(params64, np.float64)
    n = p.shape[1]
    t = np.ascontiguousarray(target, np.float32).reshape(-1, 3)
    sig = C.c_uint64()
    c = cam_struct(cam)
    v = lib().orc_loss_f64(ptr(p), n, n, C.byref(c), C.byref(s), sh_deg, ptr(t), C.byref(sig))
    return v, sig.value


def logf(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    lib().orc_logf(ptr(x), ptr(y), x.size)
    return y


def knn_init(params: np.ndarray, extent: float, nthreads: int | None = None):
    """All-pairs k-NN init: (density, f16 log sigma) per Gaussian."""
    params = np.ascontiguousarray(params, np.float32)
    n = params.shape[1]
    dens = np.empty(n, np.float32)
    ls = np.empty(n, np.float32)
    lib().orc_knn_init(ptr(params), C.c_uint64(n), n, C.c_float(extent), ptr(dens), ptr(ls),
                       nthreads or os.cpu_count() or 1)
    return dens, ls


def view_render(params: np.ndarray, cam: dict, scaling: float = 1.0, sh_deg: int = 3,
                round16: int = 1) -> dict:
    """Viewer frame: rgba (H*W, 4) f32, per-Gaussian splat records and keys."""
    params = np.ascontiguousarray(params, np.float32)
    n = params.shape[1]
    P = cam["width"] * cam["height"]
    out = dict(rgba=np.empty((P, 4), np.float32), splats=np.empty((n, 12), np.float32),
               keys=np.empty(n, np.uint32))
    c = cam_struct(cam)
    lib().orc_view_render(ptr(params), C.c_uint64(n), n, C.byref(c), C.c_float(scaling), sh_deg,
                          round16, ptr(out["rgba"]), ptr(out["splats"]), ptr(out["keys"]))
    return out


def view_pipeline(params, cam, target, s: OrcSettings, sh_deg: int, mode: int = 0) -> dict:
    """Projection -> tiles -> forward -> loss -> backward for one view."""
    pr = project(params, cam, s, sh_deg)
    tl = tiles(pr, cam, s)
    fw = forward(pr, tl, cam, s)
    out = dict(pr=pr, tl=tl, fw=fw)
    if target is not None:
        ls = loss(fw, target, cam, s)
        out["ls"] = ls
        out["bw"] = backward(pr, tl, fw, ls, cam, s, mode, sh_deg)
    return out
