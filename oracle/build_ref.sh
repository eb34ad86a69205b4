#!/usr/bin/env bash
# Builds oracle/_ref/libncvis_ref.so: the reference's own src/ncvis.cpp and
# src/knntable.cpp, compiled where they lie, with the reference's compiler
# flags (setup.py:124-126), the brute-force hnswlib stand-in and the pcg-cpp
# forwarding shim under oracle/shim, plus oracle/ref_driver.cpp.
#
# Test infrastructure only: it needs the reference checkout and pyarrow's
# vendored pcg-cpp, so it runs where both exist and is skipped elsewhere.  The
# checkout is NCVIS_REFERENCE_ROOT when set, else a directory named
# `reference` beside this repository.  Output goes to oracle/_ref/ only.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF_ROOT="${NCVIS_REFERENCE_ROOT:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_ROOT/src/ncvis.cpp" ]; then
    echo "build_ref: reference sources not found under $REF_ROOT; skipped" >&2
    exit 0
fi
PYARROW_INC="$(python3 -c 'import pyarrow; print(pyarrow.get_include())' 2>/dev/null || true)"
if [ -z "$PYARROW_INC" ] || [ ! -f "$PYARROW_INC/arrow/vendored/pcg/pcg_random.hpp" ]; then
    echo "build_ref: pyarrow's vendored pcg-cpp not found; skipped" >&2
    exit 0
fi
mkdir -p "$OUT"
FLAGS="-O3 -std=c++14 -ffast-math -fopenmp -fPIC"
INC="-I $HERE/shim/anchor -I $REF_ROOT/src -I $PYARROW_INC"
g++ $FLAGS $INC -c "$REF_ROOT/src/ncvis.cpp" -o "$OUT/ncvis.o" & P1=$!
g++ $FLAGS $INC -c "$REF_ROOT/src/knntable.cpp" -o "$OUT/knntable.o" & P2=$!
g++ $FLAGS $INC -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o" & P3=$!
wait $P1; wait $P2; wait $P3
g++ -shared -fopenmp "$OUT/ncvis.o" "$OUT/knntable.o" "$OUT/ref_driver.o" -o "$OUT/libncvis_ref.so"
echo "build_ref: $OUT/libncvis_ref.so"
