"""skyfall: GB300 Gaussian-splat render-and-train hot path behind a C-ABI.

The compute path is libskyfall.so (sm_103a CUDA kernels, built in-tree by
skyfall.build); this package is its Python host mirror of the reference's
GaussianRenderer API plus seeded synthetic scenes.
"""
from . import _lib, scenes
from ._lib import SkyError, default_config, lib
from .renderer import GaussianRenderer, LossWeights, TrainingParams, TrainingStatus

__all__ = ["GaussianRenderer", "LossWeights", "SkyError", "TrainingParams", "TrainingStatus",
           "_lib", "default_config", "lib", "scenes"]
