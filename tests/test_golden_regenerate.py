"""The golden fixtures come from the reference's own code: where the
reference build exists (oracle/_ref, made by oracle/build_ref.sh from the
reference's unmodified sources), tests/golden/make_golden.py is run into a
temporary folder and every array must equal the committed one bit for bit.
Skipped where the reference build is absent (it needs the reference
checkout, which only the development machine has)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def test_fixtures_regenerate_from_the_reference(tmp_path):
    from oracle import oracle as O
    if not O.ref_available():
        pytest.skip("reference build (oracle/_ref) not present")
    r = subprocess.run([sys.executable, os.path.join(GOLDEN, "make_golden.py"), str(tmp_path)],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    names = sorted(f for f in os.listdir(GOLDEN) if f.endswith(".npz"))
    assert names == sorted(f for f in os.listdir(tmp_path) if f.endswith(".npz"))
    for name in names:
        a, b = np.load(os.path.join(GOLDEN, name)), np.load(tmp_path / name)
        assert sorted(a.files) == sorted(b.files), name
        for key in a.files:
            x, y = a[key], b[key]
            assert x.dtype == y.dtype and x.shape == y.shape, (name, key)
            assert x.tobytes() == y.tobytes(), (name, key)
