#!/usr/bin/env bash
# Test infrastructure: compile the reference SFCI SpMSpV sources, unmodified and
# where they lie in the reference tree, together with oracle/ref_harness.cpp into
# oracle/_ref/libsfci_ref.so.  Only the three translation units of the SpMSpV path
# are built (functions.cpp, bitstr.cpp, introsort.cpp); Eigen is replaced by the
# name-only stub under oracle/ref_stub.  Usage: oracle/build_ref.sh [REF_ROOT]
# REF_ROOT defaults to $SFCI_REFERENCE_ROOT, else a checkout named "reference"
# beside this repository.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${SFCI_REFERENCE_ROOT:-$(dirname "$HERE")/../reference}}"
SRC="$REF/src"
if [ ! -f "$SRC/functions.cpp" ]; then
  echo "reference sources not found under $SRC; oracle/_ref not built" >&2
  exit 3
fi
mkdir -p "$HERE/_ref"
g++ -std=c++11 -O2 -fopenmp -fPIC -shared -w \
    -I"$HERE/ref_stub" -I"$SRC" \
    "$SRC/functions.cpp" "$SRC/bitstr.cpp" "$SRC/introsort.cpp" "$HERE/ref_harness.cpp" \
    -Wl,--no-undefined -o "$HERE/_ref/libsfci_ref.so"
echo "built $HERE/_ref/libsfci_ref.so"
