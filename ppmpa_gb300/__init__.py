"""ppmpa_gb300 -- GB300-native (sm_103a) hot path of ppm-pa.

Progressive photon mapping with the probabilistic approach: photon emission
and bounce tracing, the per-pass photon map and its in-radius gather, the
eye-hit radiance estimate, the PA radius shrink and the running average of
pass images, all on one GPU behind the C ABI of include/ppm_api.h.
"""
from . import scene
from .api import MIXED, PLAIN, Batch, Context, RenderConfig
from ._lib import PPMError

__all__ = ["scene", "Batch", "Context", "RenderConfig", "PLAIN", "MIXED", "PPMError"]
