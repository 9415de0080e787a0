#!/usr/bin/env bash
# Compile the reference project's own CPU rasteriser (cbclib_v2/_src/src/bresenham.cpp,
# pybind11 module `bresenham`) from the read-only reference checkout into oracle/_ref/.
#
# This is test infrastructure: the module is only ever used as a checker that pins the
# C restatement in oracle/cbc_oracle.c and generates the golden fixtures under
# tests/golden/.  Nothing is copied: g++ reads the sources where they lie.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Exits 0 without building when the reference checkout is absent.
set -euo pipefail
REF="${1:-/root/reference}"
SRC="$REF/cbclib_v2/_src/src/bresenham.cpp"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$SRC" ]; then
    echo "build_ref: $SRC not found, skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
EXT="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
TARGET="$OUT/bresenham$EXT"
if [ -f "$TARGET" ] && [ "$TARGET" -nt "$SRC" ] && [ "$TARGET" -nt "$0" ]; then
    exit 0
fi
PYINC="$(python3 -m pybind11 --includes)"
NPINC="$(python3 -c 'import numpy; print(numpy.get_include())')"
# Same flags as the reference's setup.py for this extension: C++17, -O3, OpenMP,
# hidden visibility.  No -march flag, so no FMA contraction on x86-64.
g++ -O3 -std=c++17 -shared -fPIC -fopenmp -fvisibility=hidden -g0 \
    $PYINC -I"$NPINC" "$SRC" -o "$TARGET.tmp" -lgomp
mv "$TARGET.tmp" "$TARGET"
echo "build_ref: built $TARGET"
