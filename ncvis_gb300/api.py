"""Python API of the GB300 NCVis engine, a drop-in for the reference's
``ncvis.NCVis`` (wrapper/ncvis.pyx:48-163).

The parameter policy is the reference's: the a/b curve fit
(wrapper/ncvis.pyx:7-24, 137-141), the default noise schedule
(wrapper/ncvis.pyx:103-123), the thread default (:125-126) and the distance
names (:128-135), with the same ValueErrors.  ``fit_transform`` makes one call
into libncvis_gb300.so, as the reference makes one call into its C++ engine
(wrapper/ncvis.pyx:45-46, 159-163).  numpy input runs through the host-buffer
entry point; a CUDA torch tensor runs through the device-buffer entry point
on the current torch stream and returns a CUDA tensor.

Keyword-only extras select the engine's modes: ``knn_precision`` ("fp32",
the plain drop-in; "bf16" for tensor-core distances with an exact FP32
rerank; "ivf" for the approximate search over k-means cells, with
``ivf_lists`` cells and ``ivf_probe`` cells searched per cell, 0 = defaults),
``rerank_factor``, ``sgd_mode`` ("hogwild": parallel chains with the
noise samples staged in shared-memory windows of the embedding where N is
large enough; "hogwild_unstaged": every noise row read from the whole
embedding; "replay" with a recorded ``replay_stream``) and ``sgd_chains``;
``knn_order`` (the "bf16" search sweeps rows ordered by k-means cell; False
keeps the caller's order, same candidates up to exact ties),
``wait_limit_cycles`` (limit of the tensor-core kernel's waits),
``arena_limit`` (largest device arena, bytes; 0 = no limit) and
``init_sequential_stats`` (init's statistics summed as the reference's one
thread sums them instead of in FP64).
"""
from __future__ import annotations

import ctypes as C
from multiprocessing import cpu_count

import numpy as np

from . import _lib


def find_ab_params(spread: float = 1.0, min_dist: float = 0.1):
    """Fit a, b of the embedding kernel 1 / (1 + a x^(2b)) to an offset
    exponential decay, as the reference does (wrapper/ncvis.pyx:7-24, after
    UMAP's curve fit)."""
    from scipy.optimize import curve_fit

    def curve(x, a, b):
        return 1.0 / (1.0 + a * x ** (2 * b))

    xv = np.linspace(0, spread * 3, 300)
    yv = np.zeros(xv.shape)
    yv[xv < min_dist] = 1.0
    yv[xv >= min_dist] = np.exp(-(xv[xv >= min_dist] - min_dist) / spread)
    params, _ = curve_fit(curve, xv, yv)
    return params[0], params[1]


def default_noise_plan(n_epochs: int, n_negative: int = 5) -> np.ndarray:
    """Noise samples per epoch rising as the cube of training progress and
    summing to about n_epochs * n_negative, at least 1 (wrapper/ncvis.pyx:103-112).
    With one epoch the reference's plan is 0 / 0, and its cast of NaN to uintp
    depends on the machine (2^63 on x86-64, 0 and so 1 on Arm); here it is 1."""
    plan = np.linspace(0, 1, n_epochs)
    plan = plan ** 3
    total = plan.sum()
    if total > 0:
        plan /= total
        plan *= n_epochs * n_negative
    plan = plan.round().astype(np.uintp)
    plan[plan < 1] = 1
    return plan


MAX_NOISE = 1 << 24  # noise samples per edge and epoch the engine accepts


DISTANCES = {
    "euclidean": 0,      # squared_L2
    "cosine": 2,         # cosine_similarity
    "correlation": 3,    # correlation
    "inner_product": 1,  # inner_product
}

_PRECISIONS = {"fp32": _lib.KNN_FP32, "bf16": _lib.KNN_BF16_RERANK, "ivf": _lib.KNN_IVF}
_SGD_MODES = {"hogwild": _lib.SGD_HOGWILD, "replay": _lib.SGD_REPLAY,
              "hogwild_unstaged": _lib.SGD_HOGWILD_UNSTAGED}


class NCVis:
    def __init__(self, d=2, n_threads=-1, n_neighbors=15, M=8, ef_construction=100,
                 random_seed=42, n_epochs=50, n_init_epochs=20, spread=1., min_dist=0.4, a=None,
                 b=None, alpha=1., alpha_Q=1., n_noise=None, distance="euclidean", *,
                 knn_precision="fp32", rerank_factor=0, sgd_mode="hogwild", replay_stream=None,
                 sgd_chains=0, ivf_lists=0, ivf_probe=0, knn_order=True, wait_limit_cycles=0,
                 arena_limit=0, init_sequential_stats=False):
        """Creates a new NCVis instance; arguments as in the reference
        (wrapper/ncvis.pyx:49-101).  M and ef_construction configure HNSW in
        the reference and are accepted and ignored (the kNN here is exact);
        n_threads bounds host-side work only."""
        self.d = d
        if n_noise is None:
            negative_plan = default_noise_plan(n_epochs)
        elif type(n_noise) is np.ndarray:
            if len(n_noise.shape) != 1:
                raise ValueError(
                    "n_noise should have exactly one dimension, but shape {} was passed".format(
                        n_noise.shape))
            if n_noise.size and (n_noise.min() < 0 or n_noise.max() > MAX_NOISE):
                raise ValueError("n_noise entries should be in [0, {}], but [{}, {}] was passed"
                                 .format(MAX_NOISE, n_noise.min(), n_noise.max()))
            negative_plan = n_noise.astype(np.uintp)
            n_epochs = negative_plan.size
        elif type(n_noise) is int:
            if n_noise < 1:
                raise ValueError("n_noise should be at least 1, but {} was passed".format(n_noise))
            if n_noise > MAX_NOISE:
                raise ValueError("n_noise should be at most {}, but {} was passed".format(
                    MAX_NOISE, n_noise))
            negative_plan = np.full(n_epochs, n_noise).astype(np.uintp)
        else:
            raise ValueError("n_noise has unsupported type")

        if n_threads < 1:
            n_threads = cpu_count()

        if distance not in DISTANCES:
            raise ValueError("Unsupported distance, expected one of: "
                             f"{set(DISTANCES)}, but got {distance}")

        if (a is None) or (b is None):
            if (a is None) and (b is None):
                a, b = find_ab_params(spread, min_dist)
            else:
                raise ValueError("Expected (a, b) to be (float, float) or (None, None), "
                                 f"but got (a, b) = ({a}, {b})")
        if knn_precision not in _PRECISIONS:
            raise ValueError(f"knn_precision must be one of {sorted(_PRECISIONS)}")
        if sgd_mode not in _SGD_MODES:
            raise ValueError(f"sgd_mode must be one of {sorted(_SGD_MODES)}")
        if int(ivf_lists) < 0 or int(ivf_probe) < 0:
            raise ValueError("ivf_lists and ivf_probe must be non-negative")
        if int(rerank_factor) < 0 or int(sgd_chains) < 0:
            raise ValueError("rerank_factor and sgd_chains must be non-negative")
        if int(wait_limit_cycles) < 0 or int(arena_limit) < 0:
            raise ValueError("wait_limit_cycles and arena_limit must be non-negative")

        self.n_epochs = int(n_epochs)
        self.noise_plan = np.ascontiguousarray(negative_plan, dtype=np.uintp)
        self.a, self.b = float(a), float(b)
        self._noise_c = (C.c_size_t * max(1, self.n_epochs))(*[int(v) for v in self.noise_plan])
        self._params = _lib.NcvisParams(
            d=d, n_threads=n_threads, n_neighbors=n_neighbors, M=M,
            ef_construction=ef_construction, random_seed=random_seed, n_epochs=self.n_epochs,
            n_init_epochs=n_init_epochs, a=self.a, b=self.b, alpha=alpha, alpha_Q=alpha_Q,
            n_noise=C.cast(self._noise_c, C.POINTER(C.c_size_t)), distance=DISTANCES[distance])
        self._replay = None
        if replay_stream is not None:
            self._replay = np.ascontiguousarray(replay_stream, dtype=np.int32)
        precision = _PRECISIONS[knn_precision] | (0 if knn_order else _lib.KNN_CALLER_ORDER)
        self._options = _lib.NcvisOptions(
            knn_precision=precision, rerank_factor=int(rerank_factor),
            sgd_mode=_SGD_MODES[sgd_mode],
            replay_stream=(self._replay.ctypes.data_as(C.POINTER(C.c_int32))
                           if self._replay is not None else None),
            replay_len=0 if self._replay is None else int(self._replay.size),
            stream=None, sgd_chains=int(sgd_chains), ivf_lists=int(ivf_lists),
            ivf_probe=int(ivf_probe), wait_limit_cycles=int(wait_limit_cycles), inject_stall=0,
            arena_limit=int(arena_limit), init_sequential_stats=int(bool(init_sequential_stats)))
        L = _lib.lib()
        self._h = L.ncvis_create(C.byref(self._params), C.byref(self._options))
        if not self._h:
            raise _lib.NcvisError(_lib.NCVIS_INVALID_ARGUMENT,
                                  (L.ncvis_get_last_error() or b"").decode())

    def __del__(self):
        h = getattr(self, "_h", None)
        if not h:
            return
        self._h = None
        try:
            _lib.lib().ncvis_destroy(h)
        except (TypeError, AttributeError):
            pass  # interpreter shutdown: the module's globals are already gone

    def _set_stream(self, stream_ptr):
        self._options.stream = stream_ptr
        _lib.check(_lib.lib().ncvis_set_options(self._h, C.byref(self._options)), self._h)

    def set_options(self, **fields):
        """Changes fields of the engine's options struct (ncvis_options in
        include/ncvis_gb300.h) for the next calls, e.g. arena_limit or
        wait_limit_cycles."""
        for name, value in fields.items():
            if name not in dict(_lib.NcvisOptions._fields_) or name in ("replay_stream",
                                                                         "replay_len", "stream"):
                raise ValueError(f"unknown or fixed option {name!r}")
            setattr(self._options, name, int(value))
        _lib.check(_lib.lib().ncvis_set_options(self._h, C.byref(self._options)), self._h)

    def fit_transform(self, X):
        """Builds an embedding for the rows of X [n_samples, n_high_dimensions]
        and returns Y [n_samples, d] float32 (wrapper/ncvis.pyx:145-163)."""
        L = _lib.lib()
        if _is_cuda_tensor(X):
            import torch
            Xc = X.detach().to(torch.float32).contiguous()
            Y = torch.empty((Xc.shape[0], self.d), dtype=torch.float32, device=Xc.device)
            with torch.cuda.device(Xc.device):
                self._set_stream(torch.cuda.current_stream().cuda_stream)
                rc = L.ncvis_fit_transform_device(self._h, Xc.data_ptr(), Xc.shape[0],
                                                  Xc.shape[1] if Xc.dim() > 1 else 0,
                                                  Y.data_ptr())
                err = _lib.error_of(rc, self._h)
                self._set_stream(None)
            if err:
                raise err
            return Y
        Xn = np.ascontiguousarray(X, dtype=np.float32)
        if Xn.ndim != 2:
            raise ValueError("X must be a 2-D array [n_samples, n_features]")
        Y = np.empty((Xn.shape[0], self.d), dtype=np.float32)
        rc = L.ncvis_fit_transform(self._h, Xn.ctypes.data, Xn.shape[0], Xn.shape[1],
                                   Y.ctypes.data)
        _lib.check(rc, self._h)
        return Y

    def fit_transform_batched(self, Xs, seeds=None):
        """Embeds several independent datasets in one run (each as if it were
        embedded alone, with its own seed) and returns one Y per dataset.
        numpy inputs give numpy outputs; CUDA tensors give CUDA tensors.  The
        neighbour count is clamped by the smallest dataset; d <= 4; the kNN
        follows knn_precision ("ivf" searches each problem exactly); the
        replay mode is not available here."""
        import torch
        L = _lib.lib()
        cuda_in = all(_is_cuda_tensor(x) for x in Xs)
        if cuda_in:
            dev = Xs[0].device
            parts = [x.detach().to(torch.float32).contiguous() for x in Xs]
        else:
            dev = torch.device("cuda", torch.cuda.current_device())
            parts = [torch.from_numpy(np.ascontiguousarray(x, dtype=np.float32)) for x in Xs]
        if not parts or any(p.dim() != 2 for p in parts):
            raise ValueError("Xs must be a non-empty list of 2-D arrays")
        D = parts[0].shape[1]
        if any(p.shape[1] != D for p in parts):
            raise ValueError("all datasets must have the same number of features")
        sizes = [p.shape[0] for p in parts]
        offsets = np.zeros(len(parts) + 1, dtype=np.int64)
        offsets[1:] = np.cumsum(sizes)
        X = torch.cat(parts).to(dev)
        Y = torch.empty((int(offsets[-1]), self.d), dtype=torch.float32, device=dev)
        seed_arr = None
        if seeds is not None:
            seed_arr = np.ascontiguousarray(seeds, dtype=np.uint64)
            if seed_arr.shape != (len(parts),):
                raise ValueError("one seed per dataset")
        with torch.cuda.device(dev):
            self._set_stream(torch.cuda.current_stream().cuda_stream)
            rc = L.ncvis_fit_transform_batched_device(
                self._h, X.data_ptr(), D, offsets.ctypes.data, len(parts),
                seed_arr.ctypes.data if seed_arr is not None else None, Y.data_ptr())
            err = _lib.error_of(rc, self._h)
            self._set_stream(None)
        if err:
            raise err
        out = torch.split(Y, sizes)
        if cuda_in:
            return list(out)
        torch.cuda.current_stream(dev).synchronize()
        return [y.cpu().numpy() for y in out]

    def stage_times(self) -> dict:
        """Device times (ms) of the stages of the last fit_transform."""
        t = _lib.NcvisStageTimes()
        _lib.check(_lib.lib().ncvis_get_stage_times(self._h, C.byref(t)), self._h)
        return t.as_dict()


def _is_cuda_tensor(x) -> bool:
    mod = type(x).__module__
    return mod.startswith("torch") and getattr(x, "is_cuda", False)
