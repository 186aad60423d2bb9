"""Host-side mirror of the reference's GaussianRenderer training API.

Method names, argument meaning and defaults follow the object returned by
get_renderer (src/renderers/gaussian-renderer.ts:30-58, 4110-4153); each call
goes straight to the C-ABI (include/skyfall.h).  Differences that follow from
the host: calls are synchronous (the reference returns Promises), images are
numpy arrays (the reference binds GPU textures), and camera choice in
train() comes from a seeded generator instead of Math.random().
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L


@dataclass
class TrainingParams:
    """TrainingParams (gaussian-renderer.ts:100-107)."""
    lr_means: float
    lr_sh: float
    lr_opacity: float
    lr_scale: float
    lr_rotation: float
    sh_update_interval: int


@dataclass
class LossWeights:
    """LossWeights (gaussian-renderer.ts:110-114)."""
    w_l2: float
    w_l1: float
    w_ssim: float


@dataclass
class TrainingStatus:
    """TrainingStatus (gaussian-renderer.ts:117-123)."""
    isTraining: bool
    currentIteration: int
    targetIterations: int
    iterationsPerSecond: float
    gaussianCount: int


def to_sky_camera(cam) -> L.SkyCamera:
    if isinstance(cam, L.SkyCamera):
        return cam
    c = L.SkyCamera()
    c.view = (C.c_float * 16)(*np.asarray(cam["view"], dtype=np.float32).reshape(16))
    c.proj = (C.c_float * 16)(*np.asarray(cam["proj"], dtype=np.float32).reshape(16))
    c.focal = (C.c_float * 2)(*np.asarray(cam["focal"], dtype=np.float32).reshape(2))
    c.width = int(cam["width"])
    c.height = int(cam["height"])
    return c


class GaussianRenderer:
    """A skyfall context: one scene, its cameras and targets, its optimizer."""

    def __init__(self, config: L.SkyConfig | None = None, **overrides):
        self._L = L.lib()
        self.config = config if config is not None else L.default_config(**overrides)
        h = C.c_void_p()
        L.check(self._L.sky_create(C.byref(self.config), C.byref(h)))
        self._h = h
        self._cams: list[L.SkyCamera] = []
        self._stop = False
        self._training = False
        self._target_iters = 0
        self._ips = 0.0
        self.last_stats = L.SkyStepStats()

    # -- lifecycle ----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.sky_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scene --------------------------------------------------------------
    def load_points(self, params: np.ndarray) -> None:
        """params: (59, N) f32 planes (see SKY_PLANE_*)."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.ndim != 2 or p.shape[0] != L.SKY_NUM_PLANES:
            raise ValueError("params must be (59, N)")
        L.check(self._L.sky_load_points(self._h, L.ptr(p), p.shape[1], p.shape[1]))

    def load_packed(self, gaussians: np.ndarray, sh: np.ndarray | None) -> None:
        """Reference storage: gaussians (N, 6) u32 words, sh (N, 24) u32 words."""
        g = np.ascontiguousarray(gaussians, dtype=np.uint32)
        s = None if sh is None else np.ascontiguousarray(sh, dtype=np.uint32)
        L.check(self._L.sky_load_packed(self._h, L.ptr(g), L.ptr(s), g.shape[0]))

    def loadPly(self, path) -> tuple[int, int]:
        """loadPlyFile + reloadPointCloud: returns (N, SH degree of the file)."""
        n, d = C.c_uint32(), C.c_uint32()
        L.check(self._L.sky_load_ply(self._h, str(path).encode(), C.byref(n), C.byref(d)))
        return n.value, d.value

    def savePly(self, path, sh_degree: int = 3) -> None:
        L.check(self._L.sky_save_ply(self._h, str(path).encode(), sh_degree))

    def initializeKnnAndSync(self, scene_extent: float = 0.0) -> np.ndarray:
        """k-NN scale initialisation; returns the per-Gaussian mean distance
        to the three nearest neighbours."""
        d = np.empty(self.getGaussianCount(), np.float32)
        L.check(self._L.sky_knn_init(self._h, scene_extent, L.ptr(d)))
        return d

    def saveCheckpoint(self, path) -> None:
        L.check(self._L.sky_save_checkpoint(self._h, str(path).encode()))

    def loadCheckpoint(self, path) -> None:
        L.check(self._L.sky_load_checkpoint(self._h, str(path).encode()))

    def setTrainingCameras(self, cameras) -> None:
        self._cams = [to_sky_camera(c) for c in cameras]
        arr = (L.SkyCamera * len(self._cams))(*self._cams)
        L.check(self._L.sky_set_cameras(self._h, arr, len(self._cams)))

    def setTrainingImages(self, images) -> None:
        for i, img in enumerate(images):
            self.setTrainingImage(i, img)

    def setTrainingImage(self, camera: int, image: np.ndarray) -> None:
        a = np.ascontiguousarray(image, dtype=np.float32)
        if a.ndim != 3 or a.shape[2] < 3:
            raise ValueError("image must be (H, W, 3)")
        a = np.ascontiguousarray(a[:, :, :3])
        L.check(self._L.sky_set_target(self._h, camera, L.ptr(a), a.shape[1], a.shape[0]))

    # -- hot path -----------------------------------------------------------
    def buildTrainingTiles(self, camera: int = 0) -> None:
        """Project, emit, sort and range the tiles of one camera (the forward
        of that camera also runs; the tile buffers stay readable)."""
        self.render([camera])

    def render(self, cameras, with_alpha: bool = True):
        cams = np.ascontiguousarray(np.atleast_1d(cameras), dtype=np.uint32)
        px = sum(self._cams[int(c)].width * self._cams[int(c)].height for c in cams)
        rgba = np.empty((px, 4), dtype=np.float32)
        alpha = np.empty(px, dtype=np.float32) if with_alpha else None
        L.check(self._L.sky_render(self._h, L.ptr(cams), len(cams), L.ptr(rgba), L.ptr(alpha)))
        return rgba, alpha

    def forward(self, cameras) -> float:
        cams = np.ascontiguousarray(np.atleast_1d(cameras), dtype=np.uint32)
        loss = C.c_double()
        L.check(self._L.sky_forward(self._h, L.ptr(cams), len(cams), C.byref(loss)))
        return loss.value

    def backward(self) -> np.ndarray:
        n = self.getGaussianCount()
        g = np.empty((L.SKY_NUM_PLANES, n), dtype=np.float32)
        L.check(self._L.sky_backward(self._h, L.ptr(g), n))
        return g

    def trainStep(self, cameras) -> L.SkyStepStats:
        cams = np.ascontiguousarray(np.atleast_1d(cameras), dtype=np.uint32)
        st = L.SkyStepStats()
        L.check(self._L.sky_step(self._h, L.ptr(cams), len(cams), C.byref(st)))
        self.last_stats = st
        return st

    def train(self, numIterations: int, views_per_step: int = 1) -> None:
        """train(n) (gaussian-renderer.ts:3744-3854): n steps, a seeded
        random camera per step; stopTraining() ends the loop between steps."""
        import time
        if self._training or numIterations <= 0:
            return
        self._training, self._stop = True, False
        self._target_iters = numIterations
        t0 = time.perf_counter()
        done = 0
        try:
            for _ in range(numIterations):
                if self._stop:
                    break
                st = L.SkyStepStats()
                L.check(self._L.sky_train(self._h, 1, views_per_step, C.byref(st)))
                self.last_stats = st
                done += 1
        finally:
            dt = time.perf_counter() - t0
            self._ips = done / dt if dt > 0 else 0.0
            self._training, self._stop = False, False

    def stopTraining(self) -> None:
        if self._training:
            self._stop = True

    # -- prune / densify / opacity reset -----------------------------------
    def prune(self, minOpacity: float = 0.005, maxScale: float = float("inf"),
              max_remove_ratio: float = 0.0, mask: np.ndarray | None = None) -> int:
        p = L.SkyPruneParams(minOpacity, maxScale, max_remove_ratio, 0)
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
        removed = C.c_uint32()
        L.check(self._L.sky_prune(self._h, C.byref(p), L.ptr(m), C.byref(removed)))
        return self.getGaussianCount()

    def resetOpacity(self, maxOpacity: float = 0.1) -> None:
        L.check(self._L.sky_reset_opacity(self._h, maxOpacity))

    def frame(self, camera, gaussian_scaling: float = 1.0, sh_degree: int | None = None,
              round_params_f16: bool = True, as_u8: bool = False) -> np.ndarray:
        """frame(encoder, view) of the viewer, headless: the (H, W, 4) RGBA
        image (f32, or u8 with as_u8) of the quad-splat render from `camera`."""
        cam = to_sky_camera(camera)
        vs = L.SkyViewSettings()
        L.lib().sky_view_settings_default(C.byref(vs))
        vs.gaussian_scaling = gaussian_scaling
        vs.sh_degree = self.config.sh_degree if sh_degree is None else sh_degree
        vs.round_params_f16 = 1 if round_params_f16 else 0
        h, w = int(cam.height), int(cam.width)
        if as_u8:
            out = np.empty((h, w, 4), np.uint8)
            L.check(self._L.sky_view_render(self._h, C.byref(cam), C.byref(vs), None, L.ptr(out)))
        else:
            out = np.empty((h, w, 4), np.float32)
            L.check(self._L.sky_view_render(self._h, C.byref(cam), C.byref(vs), L.ptr(out), None))
        return out

    def densifyStats(self) -> tuple[np.ndarray, np.ndarray]:
        """(grad_accum, importance_stats), each (N, 4) f32: the densify
        accumulator and the importance statistics the training steps gather."""
        n = self.getGaussianCount()
        g = np.zeros((n, 4), np.float32)
        i = np.zeros((n, 4), np.float32)
        L.check(self._L.sky_densify_stats(self._h, L.ptr(g), L.ptr(i)))
        return g, i

    def scoreViews(self, cameras=None) -> tuple[np.ndarray, np.ndarray]:
        """Multi-view scores (generateMultiViewScores): per Gaussian the u32
        error-pixel hits and the f32 pruning score; cameras=None samples
        min(10, cameras) with the context's seeded generator."""
        n = self.getGaussianCount()
        imp = np.zeros(n, np.uint32)
        pr = np.zeros(n, np.float32)
        if cameras is None:
            L.check(self._L.sky_score_views(self._h, None, 0, L.ptr(imp), L.ptr(pr)))
        else:
            cams = np.ascontiguousarray(np.atleast_1d(cameras), dtype=np.uint32)
            L.check(self._L.sky_score_views(self._h, L.ptr(cams), len(cams), L.ptr(imp), L.ptr(pr)))
        return imp, pr

    @staticmethod
    def densifyParams(**overrides) -> L.SkyDensifyParams:
        p = L.SkyDensifyParams()
        L.lib().sky_densify_default(C.byref(p))
        for k, v in overrides.items():
            setattr(p, k, v)
        return p

    def densify(self, params: L.SkyDensifyParams | None = None, **overrides) -> tuple[int, int]:
        """performDensification: returns (cloned, split)."""
        p = params if params is not None else self.densifyParams(**overrides)
        cl, sp = C.c_uint32(), C.c_uint32()
        L.check(self._L.sky_densify(self._h, C.byref(p), C.byref(cl), C.byref(sp)))
        return cl.value, sp.value

    @staticmethod
    def scoredPruneParams(**overrides) -> L.SkyScoredPruneParams:
        p = L.SkyScoredPruneParams()
        L.lib().sky_scored_prune_default(C.byref(p))
        for k, v in overrides.items():
            setattr(p, k, v)
        return p

    def pruneScored(self, params: L.SkyScoredPruneParams | None = None, **overrides) -> int:
        """applyMultiViewPrune: returns the number of Gaussians removed."""
        p = params if params is not None else self.scoredPruneParams(**overrides)
        removed = C.c_uint32()
        L.check(self._L.sky_prune_scored(self._h, C.byref(p), C.byref(removed)))
        return removed.value

    def setSchedule(self, enabled: bool = True, **overrides) -> L.SkySchedule:
        """TrainingController schedule run by train(): densify/prune/opacity
        reset windows and thresholds (defaults of DEFAULT_TRAINING_SCHEDULE)."""
        s = L.SkySchedule()
        L.lib().sky_schedule_default(C.byref(s))
        s.enabled = 1 if enabled else 0
        for k, v in overrides.items():
            if k == "densify":
                for dk, dv in v.items():
                    setattr(s.densify, dk, dv)
            else:
                setattr(s, k, v)
        L.check(self._L.sky_set_schedule(self._h, C.byref(s)))
        return s

    # -- parameters and status ---------------------------------------------
    def getTrainingParams(self) -> TrainingParams:
        c = self.config
        return TrainingParams(c.lr_means, c.lr_sh, c.lr_opacity, c.lr_scale, c.lr_rotation,
                              c.sh_update_interval)

    def setTrainingParams(self, **params) -> None:
        for k, v in params.items():
            if k not in TrainingParams.__dataclass_fields__:
                raise KeyError(k)
            setattr(self.config, k, v)
        L.check(self._L.sky_set_config(self._h, C.byref(self.config)))

    def getConfig(self) -> L.SkyConfig:
        """The context's configuration as the library holds it."""
        c = L.SkyConfig()
        c.struct_size = C.sizeof(L.SkyConfig)
        L.check(self._L.sky_get_config(self._h, C.byref(c)))
        return c

    def setBatchDepth(self, fwd_batch: int = 0, bwd_batch: int = 0) -> None:
        """Splat-batch depths of the rasterizers (0 = default); results do not
        depend on them, only speed (see skyfall.autotune)."""
        self.config.fwd_batch = fwd_batch
        self.config.bwd_batch = bwd_batch
        L.check(self._L.sky_set_config(self._h, C.byref(self.config)))

    def setTileCull(self, on: bool) -> None:
        """Intersection lists of backward and training steps limited to the
        tiles each Gaussian's alpha >= 1/255 ellipse reaches (exact: images,
        loss, gradients and parameters are bit-identical either way; renders
        keep every tile of the rectangle)."""
        self.config.tile_cull = 1 if on else 0
        L.check(self._L.sky_set_config(self._h, C.byref(self.config)))

    def setBatchScaling(self, on: bool) -> None:
        """Adam hyperparameters of a step of B views: off, those of one view
        (the reference's); on, learning rates x sqrt(B) and betas to the
        power B (Zhao et al. 2024), bias correction counted in views.  Steps
        of one view are unchanged either way."""
        self.config.batch_scaling = 1 if on else 0
        L.check(self._L.sky_set_config(self._h, C.byref(self.config)))

    def getLossWeights(self) -> LossWeights:
        return LossWeights(self.config.w_l2, self.config.w_l1, self.config.w_ssim)

    def setLossWeights(self, **w) -> None:
        for k, v in w.items():
            if k not in LossWeights.__dataclass_fields__:
                raise KeyError(k)
            setattr(self.config, k, v)
        L.check(self._L.sky_set_config(self._h, C.byref(self.config)))

    def getStatus(self) -> L.SkyStatus:
        st = L.SkyStatus()
        L.check(self._L.sky_get_status(self._h, C.byref(st)))
        return st

    def getTrainingStatus(self) -> TrainingStatus:
        st = self.getStatus()
        return TrainingStatus(self._training, int(st.iteration), self._target_iters, self._ips,
                              int(st.num_gaussians))

    def getGaussianCount(self) -> int:
        n = C.c_uint32()
        L.check(self._L.sky_get_count(self._h, C.byref(n)))
        return n.value

    def params(self) -> np.ndarray:
        n = self.getGaussianCount()
        out = np.empty((L.SKY_NUM_PLANES, n), dtype=np.float32)
        L.check(self._L.sky_get_params(self._h, L.ptr(out), n))
        return out

    def moments(self):
        n = self.getGaussianCount()
        m1 = np.empty((L.SKY_NUM_PLANES, n), dtype=np.float32)
        m2 = np.empty((L.SKY_NUM_PLANES, n), dtype=np.float32)
        L.check(self._L.sky_get_moments(self._h, L.ptr(m1), L.ptr(m2), n))
        return m1, m2

    def read_buffer(self, name: str) -> np.ndarray:
        which = L.BUF[name]
        size = C.c_uint64()
        L.check(self._L.sky_read_buffer(self._h, which, None, 0, C.byref(size)))
        dt = np.dtype(L.BUF_DTYPE[name])
        out = np.empty(size.value // dt.itemsize, dtype=dt)
        if size.value:
            L.check(self._L.sky_read_buffer(self._h, which, L.ptr(out), size.value, C.byref(size)))
        return out

    def sync(self) -> None:
        L.check(self._L.sky_sync(self._h))

    # -- profiling (profiledTrainStep / TrainingProfiler) -------------------
    def stream(self) -> int:
        s = C.c_void_p()
        L.check(self._L.sky_get_stream(self._h, C.byref(s)))
        return s.value or 0

    def enableProfiling(self, enabled: bool = True) -> None:
        L.check(self._L.sky_set_profiling(self._h, int(enabled)))

    def stageTimes(self) -> tuple[dict, int]:
        """Summed milliseconds per stage and the number of timed steps."""
        arr = (C.c_double * len(L.STAGES))()
        steps = C.c_uint64()
        L.check(self._L.sky_get_stage_times(self._h, arr, len(L.STAGES), C.byref(steps)))
        return dict(zip(L.STAGES, list(arr))), steps.value
