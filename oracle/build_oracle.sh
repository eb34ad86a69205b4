#!/usr/bin/env bash
# Builds oracle/liboracle.so, the CPU restatement (test infrastructure), with
# plain g++ (no GPU).  ncvis_oracle.cpp uses the reference's own flags
# (setup.py:124-126); ncvis_oracle_sgd.cpp is compiled with strict IEEE
# arithmetic so its explicitly written grouping is what runs on every host.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OBJ="$(mktemp -d)"
trap 'rm -rf "$OBJ"' EXIT
g++ -O3 -std=c++14 -ffast-math -fopenmp -fPIC -c "$HERE/ncvis_oracle.cpp" -o "$OBJ/main.o" & P1=$!
g++ -O3 -std=c++14 -fno-fast-math -ffp-contract=off -fopenmp -fPIC -c "$HERE/ncvis_oracle_sgd.cpp" -o "$OBJ/sgd.o" & P2=$!
wait $P1; wait $P2
g++ -shared -fopenmp "$OBJ/main.o" "$OBJ/sgd.o" -o "$HERE/liboracle.so"
echo "build_oracle: $HERE/liboracle.so"
