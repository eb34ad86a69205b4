# cython: language_level=3
"""NCVisWrapper over libncvis_gb300.so: the class the reference's Cython module
defines over its C++ engine (wrapper/ncvis.pyx:26-46), with the same
constructor arguments and fit_transform(X, Y), driving the GPU engine through
its C ABI.  The reference's `NCVis` policy class (a/b fit, noise plan,
distances, wrapper/ncvis.pyx:48-163) sits unchanged on top of it.

Differences, both deliberate: an argument the engine refuses raises
ValueError from the constructor (the reference's constructor throws a C++
exception, translated by `except +`), and a failing fit_transform raises
RuntimeError (the reference's .pxd has no `except +` there, so a throw ends
the interpreter).  fit_transform releases the GIL while the engine runs."""
import numpy as np

from cncvis_gb300 cimport (ncvis_create, ncvis_destroy, ncvis_fit_transform, ncvis_get_last_error,
                            ncvis_handle, ncvis_last_error, ncvis_params)


cdef class NCVisWrapper:
    cdef ncvis_handle h
    cdef size_t d

    def __cinit__(self, size_t d, size_t n_threads, size_t n_neighbors, size_t M,
                  size_t ef_construction, size_t random_seed, int n_epochs, int n_init_epochs,
                  float a, float b, float alpha, float alpha_Q, object n_noise, int distance):
        cdef size_t[::1] plan
        self.h = NULL
        if isinstance(n_noise, int):
            if n_noise < 0:
                raise ValueError("n_noise must be non-negative")
            plan = np.full(max(n_epochs, 1), n_noise, dtype=np.uintp)
        elif isinstance(n_noise, np.ndarray):
            if n_noise.ndim != 1:
                raise ValueError("Expected 1D n_noise array.")
            n_epochs = n_noise.shape[0]
            plan = np.ascontiguousarray(n_noise.astype(np.uintp)) if n_epochs else \
                np.zeros(1, dtype=np.uintp)
        else:
            raise ValueError("n_noise must be an int or a 1-D numpy array")
        cdef ncvis_params p
        p.d = d
        p.n_threads = n_threads
        p.n_neighbors = n_neighbors
        p.M = M
        p.ef_construction = ef_construction
        p.random_seed = random_seed
        p.n_epochs = n_epochs
        p.n_init_epochs = n_init_epochs
        p.a = a
        p.b = b
        p.alpha = alpha
        p.alpha_Q = alpha_Q
        p.n_noise = &plan[0]
        p.distance = distance
        self.h = ncvis_create(&p, NULL)  # copies the plan
        if self.h == NULL:
            raise ValueError(ncvis_get_last_error().decode(errors="replace"))
        self.d = d

    def __dealloc__(self):
        if self.h != NULL:
            ncvis_destroy(self.h)
            self.h = NULL

    def fit_transform(self, float[:, ::1] X, float[:, ::1] Y):
        """X [N, D] and Y [N, d] C-contiguous float32 host arrays; Y is written."""
        cdef int rc
        cdef size_t N = X.shape[0], D = X.shape[1]
        if Y.shape[0] != X.shape[0] or <size_t>Y.shape[1] != self.d:
            raise ValueError("Y must have shape (X.shape[0], d)")
        cdef const float *xp = &X[0, 0] if N > 0 and D > 0 else NULL
        cdef float *yp = &Y[0, 0] if N > 0 else NULL
        with nogil:
            rc = ncvis_fit_transform(self.h, xp, N, D, yp)
        if rc != 0:
            raise RuntimeError(ncvis_last_error(self.h).decode(errors="replace"))
