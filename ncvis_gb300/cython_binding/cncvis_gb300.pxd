# Cython declarations of the engine's C ABI (include/ncvis_gb300.h): what the
# reference's wrapper/cncvis.pxd declares for the C++ class ncvis::NCVis
# (wrapper/cncvis.pxd:1-11), here for libncvis_gb300.so.  Only the fields and
# functions the wrapper uses are listed; the header is the definition.
from libc.stdint cimport int32_t

cdef extern from "ncvis_gb300.h" nogil:
    ctypedef struct ncvis_params:
        size_t d
        size_t n_threads
        size_t n_neighbors
        size_t M
        size_t ef_construction
        size_t random_seed
        int n_epochs
        int n_init_epochs
        float a
        float b
        float alpha
        float alpha_Q
        const size_t *n_noise
        int distance
    ctypedef struct ncvis_options:
        int knn_precision
        int rerank_factor
        int sgd_mode
    ctypedef struct ncvis_engine:
        pass
    ctypedef ncvis_engine *ncvis_handle
    ncvis_handle ncvis_create(const ncvis_params *params, const ncvis_options *options)
    void ncvis_destroy(ncvis_handle h)
    int ncvis_fit_transform(ncvis_handle h, const float *X, size_t N, size_t D, float *Y)
    const char *ncvis_last_error(ncvis_handle h)
    const char *ncvis_get_last_error()
