"""The engine's introsort (ncvis_gb300/csrc/introsort.cuh, compiled as host
C++) gives the same permutation as this toolchain's std::sort with the
reference's comparator (src/knntable.cpp:81-83), ties included: random keys
with few or many distinct values, sorted, reversed, zig-zag and sawtooth
rows, pairs of equal keys as symmetrization makes them, and median-of-three
adversaries that exhaust the depth budget so the heap-sort fallback runs
(tests/harness/sort_check.cpp).  The symmetrized CSR is bit-exact only if
the tie order matches, so this is the CPU half of that parity bar; the GPU
half is tests/test_gpu_symmetrize.py."""
import os
import subprocess

from conftest import ROOT


def test_introsort_matches_std_sort(tmp_path):
    src = os.path.join(ROOT, "tests", "harness", "sort_check.cpp")
    exe = str(tmp_path / "sort_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "ncvis_gb300", "csrc"),
                        src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok "), r.stdout
    assert int(r.stdout.split()[1]) >= 20000


def test_staged_row_merge_matches_reference_steps(tmp_path):
    """The staged row merge (ncvis_gb300/csrc/merge_row.cuh, the per-row body
    of the GPU symmetrization) against a direct statement of the reference's
    append order, index sort and in-place deduplication
    (src/knntable.cpp:40-49, 81-93), over plain arrays and over strided
    views like the GPU's shared-memory rows (tests/harness/merge_check.cpp)."""
    src = os.path.join(ROOT, "tests", "harness", "merge_check.cpp")
    exe = str(tmp_path / "merge_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "ncvis_gb300", "csrc"),
                        src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok "), r.stdout
    assert int(r.stdout.split()[1]) >= 20000


def test_data_parallel_row_sort_matches_std_sort(tmp_path):
    """The data-parallel restatement behind the GPU's warp-per-row merge:
    std::sort's Hoare partitions computed from position lists, each leaf
    range stably sorted, and the in-place deduplication as a fixpoint of one
    parallel step, against std::sort with the reference's comparator and the
    sequential merge (src/knntable.cpp:81-93), on random, tie-heavy and
    adversarial rows that exhaust the depth budget
    (tests/harness/partition_check.cpp)."""
    src = os.path.join(ROOT, "tests", "harness", "partition_check.cpp")
    exe = str(tmp_path / "partition_check")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "ncvis_gb300", "csrc"),
                        src, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok "), r.stdout
    assert int(r.stdout.split()[1]) >= 20000
