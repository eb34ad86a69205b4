"""The drop-in boundary without a GPU: libncvis_gb300.so builds for sm_103a,
loads, and exports every function include/ncvis_gb300.h declares with the
binding's signatures; the C++ header compiles against it.  No compute call
is made (there is no GPU here)."""
import ctypes
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "ncvis_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b(ncvis_[a-z_0-9]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from ncvis_gb300 import _lib
    L = _lib.lib()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), "ctypes binding and header disagree"


def test_library_is_sm103a_only():
    from ncvis_gb300 import _build
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.NVCC_FLAGS)
    assert os.path.exists(_build.LIB)


def test_version_string():
    from ncvis_gb300 import _lib
    assert b"sm_103a" in _lib.lib().ncvis_version()


def test_cpp_header_compiles():
    """include/ncvis.hpp (the reference-shaped C++ class) compiles and links."""
    src = os.path.join(ROOT, "tests", "harness", "cpp_api_check.cpp")
    out = os.path.join(ROOT, "tests", "harness", "_cpp_api_check")
    from ncvis_gb300 import _build
    lib_dir = os.path.dirname(_build.LIB)
    r = subprocess.run(["g++", "-std=c++14", "-I", os.path.join(ROOT, "include"), src, "-o", out,
                        "-L", lib_dir, "-lncvis_gb300", f"-Wl,-rpath,{lib_dir}"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # Argument errors are reported without touching the GPU.
    r = subprocess.run([out], capture_output=True, text=True)
    os.remove(out)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ok" in r.stdout


def test_create_refuses_noise_above_bound():
    """ncvis_create checks the noise plan on the host (no GPU call): an entry
    above 2^24 returns NULL with a message; 2^24 itself is accepted."""
    import ctypes as C
    from ncvis_gb300 import _lib
    L = _lib.lib()
    for top, ok in (((1 << 24) + 1, False), (1 << 24, True), ((1 << 63), False)):
        plan = (C.c_size_t * 3)(1, top, 2)
        p = _lib.NcvisParams(d=2, n_threads=1, n_neighbors=15, M=16, ef_construction=200,
                             random_seed=42, n_epochs=3, n_init_epochs=20, a=1.0, b=1.0,
                             alpha=1.0, alpha_Q=1.0, n_noise=C.cast(plan, C.POINTER(C.c_size_t)),
                             distance=0)
        h = L.ncvis_create(C.byref(p), None)
        if ok:
            assert h
            L.ncvis_destroy(h)
        else:
            assert not h
            assert b"n_noise entries must be at most 16777216" in L.ncvis_get_last_error()


def test_c_header_links_from_c99(tmp_path):
    """include/ncvis_gb300.h is plain C (C99, strict warnings): a C program
    includes it, links libncvis_gb300.so and runs its host-only calls."""
    from ncvis_gb300 import _build
    src = tmp_path / "c_check.c"
    src.write_text(
        '#include <stdio.h>\n#include <string.h>\n#include "ncvis_gb300.h"\n'
        "int main(void) {\n"
        "    size_t plan[2] = {1, 2};\n"
        "    ncvis_params p;\n"
        "    ncvis_handle h;\n"
        "    memset(&p, 0, sizeof p);\n"
        "    p.d = 2; p.n_neighbors = 15; p.random_seed = 42; p.n_epochs = 2;\n"
        "    p.n_init_epochs = 20; p.a = 1.f; p.b = 1.f; p.alpha = 1.f; p.alpha_Q = 1.f;\n"
        "    p.n_noise = plan; p.distance = NCVIS_COSINE_SIMILARITY;\n"
        "    h = ncvis_create(&p, NULL);\n"
        "    if (!h) { printf(\"create: %s\\n\", ncvis_get_last_error()); return 1; }\n"
        "    ncvis_destroy(h);\n"
        "    printf(\"ok %s\\n\", ncvis_version());\n"
        "    return 0;\n"
        "}\n")
    exe = str(tmp_path / "c_check")
    lib_dir = os.path.dirname(_build.LIB)
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Wpedantic", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", exe, "-L", lib_dir,
                        "-lncvis_gb300", f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("ok "), r.stdout + r.stderr


def test_options_are_checked_on_the_host():
    """ncvis_create and ncvis_set_options refuse unknown modes, negative counts
    and a replay length without a stream (no GPU call is made)."""
    import ctypes as C
    from ncvis_gb300 import _lib
    L = _lib.lib()
    plan = (C.c_size_t * 2)(1, 2)
    p = _lib.NcvisParams(d=2, n_threads=1, n_neighbors=15, M=16, ef_construction=200,
                         random_seed=42, n_epochs=2, n_init_epochs=20, a=1.0, b=1.0, alpha=1.0,
                         alpha_Q=1.0, n_noise=C.cast(plan, C.POINTER(C.c_size_t)), distance=0)
    bad = [dict(knn_precision=3), dict(knn_precision=-1), dict(sgd_mode=3), dict(rerank_factor=-1),
           dict(sgd_chains=-2), dict(ivf_lists=-1), dict(ivf_probe=-1), dict(replay_len=5)]
    for kw in bad:
        h = L.ncvis_create(C.byref(p), C.byref(_lib.NcvisOptions(**kw)))
        assert not h, kw
        assert b"[ncvis] options:" in L.ncvis_get_last_error(), kw
    good = _lib.NcvisOptions(knn_precision=2, sgd_mode=2, rerank_factor=4, sgd_chains=8,
                             ivf_lists=16, ivf_probe=8)
    h = L.ncvis_create(C.byref(p), C.byref(good))
    assert h
    try:
        assert L.ncvis_set_options(h, C.byref(_lib.NcvisOptions(sgd_mode=7))) == _lib.NCVIS_INVALID_ARGUMENT
        assert b"sgd_mode" in L.ncvis_last_error(h)
        assert L.ncvis_set_options(h, C.byref(_lib.NcvisOptions())) == 0
    finally:
        L.ncvis_destroy(h)
