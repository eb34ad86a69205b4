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
