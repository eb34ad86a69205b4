"""ctypes binding of libncvis_gb300.so (C ABI declared in include/ncvis_gb300.h).

The library is loaded from the package directory.  If it is missing it is
built with nvcc (ncvis_gb300/_build.py); if that is impossible the import of
any engine entry point fails loudly -- there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _build

NCVIS_OK = 0
NCVIS_INVALID_ARGUMENT = 1
NCVIS_CUDA_ERROR = 2
NCVIS_UNSUPPORTED = 3
NCVIS_DEVICE_TIMEOUT = 4
NCVIS_INTERNAL = 5

KNN_FP32 = 0
KNN_BF16_RERANK = 1
KNN_IVF = 2
KNN_CALLER_ORDER = 0x100  # flag: exact BF16 search in the caller's row order
SGD_HOGWILD = 0
SGD_REPLAY = 1
SGD_HOGWILD_UNSTAGED = 2


class NcvisParams(C.Structure):
    _fields_ = [
        ("d", C.c_size_t),
        ("n_threads", C.c_size_t),
        ("n_neighbors", C.c_size_t),
        ("M", C.c_size_t),
        ("ef_construction", C.c_size_t),
        ("random_seed", C.c_size_t),
        ("n_epochs", C.c_int),
        ("n_init_epochs", C.c_int),
        ("a", C.c_float),
        ("b", C.c_float),
        ("alpha", C.c_float),
        ("alpha_Q", C.c_float),
        ("n_noise", C.POINTER(C.c_size_t)),
        ("distance", C.c_int),
    ]


class NcvisOptions(C.Structure):
    _fields_ = [
        ("knn_precision", C.c_int),
        ("rerank_factor", C.c_int),
        ("sgd_mode", C.c_int),
        ("replay_stream", C.POINTER(C.c_int32)),
        ("replay_len", C.c_size_t),
        ("stream", C.c_void_p),
        ("sgd_chains", C.c_int),
        ("ivf_lists", C.c_int),
        ("ivf_probe", C.c_int),
        ("wait_limit_cycles", C.c_longlong),
        ("inject_stall", C.c_int),
        ("arena_limit", C.c_size_t),
        ("init_sequential_stats", C.c_int),
        ("knn_order_cells", C.c_int),
    ]


class NcvisStageTimes(C.Structure):
    _fields_ = [
        ("h2d_ms", C.c_float),
        ("preprocess_ms", C.c_float),
        ("knn_ms", C.c_float),
        ("rerank_ms", C.c_float),
        ("symmetrize_ms", C.c_float),
        ("build_edges_ms", C.c_float),
        ("init_ms", C.c_float),
        ("optimize_ms", C.c_float),
        ("d2h_ms", C.c_float),
        ("total_ms", C.c_float),
        ("n_edges", C.c_int64),
        ("k", C.c_int64),
        ("knn_order_ms", C.c_float),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class NcvisError(RuntimeError):
    """A non-zero status from the engine; `code` is the NCVIS_* status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


_vp = C.c_void_p
_sz = C.c_size_t
_lock = threading.Lock()
_lib = None

# name -> (restype, argtypes); every exported symbol of include/ncvis_gb300.h.
SIGNATURES = {
    "ncvis_create": (_vp, [C.POINTER(NcvisParams), C.POINTER(NcvisOptions)]),
    "ncvis_destroy": (None, [_vp]),
    "ncvis_set_options": (C.c_int, [_vp, C.POINTER(NcvisOptions)]),
    "ncvis_fit_transform": (C.c_int, [_vp, _vp, _sz, _sz, _vp]),
    "ncvis_fit_transform_device": (C.c_int, [_vp, _vp, _sz, _sz, _vp]),
    "ncvis_fit_transform_batched_device": (C.c_int, [_vp, _vp, _sz, _vp, _sz, _vp, _vp]),
    "ncvis_last_error": (C.c_char_p, [_vp]),
    "ncvis_get_last_error": (C.c_char_p, []),
    "ncvis_get_stage_times": (C.c_int, [_vp, C.POINTER(NcvisStageTimes)]),
    "ncvis_knn_device": (C.c_int, [_vp, _sz, _sz, C.c_int, _sz, C.c_int, C.c_int, _vp, _vp, _vp]),
    "ncvis_knn_ivf_device": (C.c_int, [_vp, _sz, _sz, C.c_int, _sz, C.c_int, C.c_int, C.c_int,
                                       _vp, _vp, _vp]),
    "ncvis_symmetrize_device": (C.c_int, [_sz, _sz, _vp, _vp, _vp, _vp, _vp, _vp,
                                          C.POINTER(_sz), _vp]),
    "ncvis_init_embedding_device": (C.c_int, [_sz, _sz, _vp, _vp, C.c_uint64, C.c_int, C.c_float,
                                              C.c_int, _vp, _vp]),
    "ncvis_optimize_device": (C.c_int, [_sz, _sz, _sz, _vp, _vp, _vp, _vp, C.c_uint64, C.c_int,
                                        C.c_int, C.c_int, C.POINTER(_sz), C.c_float, C.c_float,
                                        C.c_float, C.c_float, C.c_int, _vp]),
    "ncvis_optimize_staged_device": (C.c_int, [_sz, _sz, _sz, _vp, _vp, _vp, _vp, C.c_uint64,
                                               C.c_int, C.c_int, C.c_int, C.POINTER(_sz),
                                               C.c_float, C.c_float, C.c_float, C.c_float,
                                               C.c_int, C.c_int, _vp]),
    "ncvis_optimize_replay_device": (C.c_int, [_sz, _sz, _vp, _vp, _sz, _sz, _vp, _sz, _vp, _vp,
                                               C.c_int, C.c_int, _sz, C.c_float, C.c_float,
                                               C.c_float, C.c_float, _vp]),
    "ncvis_nce_loss_device": (C.c_int, [_sz, _sz, _sz, _vp, _vp, _vp, _vp, _sz, C.c_float,
                                        C.c_float, C.c_uint64, C.c_uint32, C.c_uint64, _vp, _vp]),
    "ncvis_nce_grad_device": (C.c_int, [_sz, _sz, _sz, _vp, _vp, _vp, _vp, _sz, C.c_float,
                                        C.c_float, C.c_uint64, C.c_uint32, C.c_uint64, _vp, _vp,
                                        _vp, _vp]),
    "ncvis_nce_noise_device": (C.c_int, [_sz, _sz, _vp, _sz, C.c_uint64, C.c_uint32, C.c_uint64,
                                         _vp, _vp]),
    "ncvis_nce_loss_device_noalloc": (C.c_int, [_sz, _sz, _sz, _vp, _vp, _vp, _vp, _sz,
                                                C.c_float, C.c_float, C.c_uint64, C.c_uint32,
                                                C.c_uint64, _vp, _vp]),
    "ncvis_trustworthiness_device": (C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_int,
                                               C.c_void_p, C.c_size_t, C.c_size_t,
                                               C.POINTER(C.c_double), C.c_void_p]),
    "ncvis_measure_update_rate": (C.c_int, [C.c_size_t, C.c_size_t, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.c_void_p]),
    "ncvis_kernel_launch_count": (C.c_uint64, []),
    "ncvis_version": (C.c_char_p, []),
}


def library_path() -> str:
    return _build.LIB


def lib():
    """The loaded engine library (built on first use if needed)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            if not os.path.exists(path):
                raise ImportError(f"libncvis_gb300.so is missing at {path}")
            L = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def error_of(rc: int, handle=None):
    """The NcvisError for a non-zero status (None for NCVIS_OK), with the
    message the library recorded for it."""
    if rc == NCVIS_OK:
        return None
    L = lib()
    msg = L.ncvis_last_error(handle) if handle else L.ncvis_get_last_error()
    return NcvisError(rc, (msg or b"").decode(errors="replace") or f"ncvis status {rc}")


def check(rc: int, handle=None) -> None:
    """Raise NcvisError for a non-zero status."""
    err = error_of(rc, handle)
    if err:
        raise err
