"""Build recipe of the Cython binding (ncvis_gb300_cy.NCVisWrapper): cythonize
ncvis_gb300_cy.pyx against cncvis_gb300.pxd and compile it with the C
compiler against include/ncvis_gb300.h, linked to libncvis_gb300.so (found
through an rpath to the package directory).  Needs Cython, which the
reference's own build uses; the ctypes binding (ncvis_gb300._lib) needs
nothing beyond the library."""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
INCLUDE = os.path.join(os.path.dirname(PKG), "include")


def build(out_dir: str) -> str:
    """Compiles the extension module into out_dir; returns its path."""
    from ncvis_gb300 import _build
    lib = _build.build()
    os.makedirs(out_dir, exist_ok=True)
    c_file = os.path.join(out_dir, "ncvis_gb300_cy.c")
    subprocess.run([sys.executable, "-m", "cython", "-3", "-I", HERE,
                    os.path.join(HERE, "ncvis_gb300_cy.pyx"), "-o", c_file],
                   check=True, capture_output=True, text=True)
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(out_dir, "ncvis_gb300_cy" + suffix)
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O2", "-shared", "-fPIC", "-I", sysconfig.get_paths()["include"], "-I", INCLUDE,
           c_file, "-L", os.path.dirname(lib), "-lncvis_gb300",
           "-Wl,-rpath," + os.path.dirname(lib), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compiling the Cython binding failed:\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else os.path.join(PKG, "_build", "cython")))
