"""The Cython binding (ncvis_gb300/cython_binding): the reference's NCVisWrapper
(wrapper/ncvis.pyx:26-46, wrapper/cncvis.pxd:1-11) over the engine's C ABI,
cythonized and compiled here, imported, and driven through its error paths,
which need no GPU: the constructor refuses what the engine refuses
(ValueError), and fit_transform reports the reference's errors
(src/ncvis.cpp:364-369) as RuntimeError.  Cython is absent on the GPU
machines; there the ctypes binding is the tested one."""
import importlib.util

import numpy as np
import pytest

pytest.importorskip("Cython")


@pytest.fixture(scope="module")
def cy(tmp_path_factory):
    from ncvis_gb300.cython_binding import build
    path = build.build(str(tmp_path_factory.mktemp("cython")))
    spec = importlib.util.spec_from_file_location("ncvis_gb300_cy", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _args(n_noise, distance=0):
    from ncvis_gb300.api import find_ab_params
    a, b = find_ab_params(1.0, 0.4)
    return (2, 1, 15, 16, 200, 42, 50, 20, a, b, 1.0, 1.0, n_noise, distance)


def test_constructs_with_reference_arguments(cy):
    from ncvis_gb300.api import default_noise_plan
    cy.NCVisWrapper(*_args(default_noise_plan(50)))
    cy.NCVisWrapper(*_args(3))


def test_constructor_refuses_bad_arguments(cy):
    with pytest.raises(ValueError, match="n_noise"):
        cy.NCVisWrapper(*_args(np.full(50, 1 << 25, dtype=np.uintp)))
    with pytest.raises(ValueError, match="1D"):
        cy.NCVisWrapper(*_args(np.ones((5, 10), dtype=np.uintp)))
    with pytest.raises(ValueError):
        cy.NCVisWrapper(*_args("three"))


def test_fit_transform_reports_reference_errors(cy):
    w = cy.NCVisWrapper(*_args(3))
    with pytest.raises(RuntimeError, match="at least one element"):
        w.fit_transform(np.zeros((0, 3), np.float32), np.zeros((0, 2), np.float32))
    with pytest.raises(ValueError, match="shape"):
        w.fit_transform(np.zeros((4, 3), np.float32), np.zeros((4, 3), np.float32))
