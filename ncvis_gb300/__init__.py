"""GB300-native NCVis engine: drop-in for stat-ml/ncvis's ``ncvis`` module.

``import ncvis_gb300 as ncvis`` gives the reference's ``NCVis`` class and
``find_ab_params``; the work runs in hand-written sm_103a CUDA kernels in
libncvis_gb300.so (C ABI: include/ncvis_gb300.h).
"""
from .api import DISTANCES, NCVis, default_noise_plan, find_ab_params
from ._lib import NcvisError, library_path

__all__ = ["NCVis", "find_ab_params", "default_noise_plan", "DISTANCES", "NcvisError",
           "library_path"]
__version__ = "0.1.0"
