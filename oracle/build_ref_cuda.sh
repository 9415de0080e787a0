#!/usr/bin/env bash
# The reference project's own GPU rasteriser (cbclib_v2/_src/src/cuda_draw_lines.cu,
# pybind11 module `cuda_draw_lines`), built unmodified for sm_103a so that it can be
# timed and compared on the GB300 beside this library.  Test infrastructure only: it
# is never imported by the package.
#
#   oracle/build_ref_cuda.sh stage [REFERENCE_ROOT]   (here, where the reference exists)
#       copies the module's five source files and the pybind11 headers into
#       oracle/_ref/cuda_src/ (git-ignored, not committed; it travels with the working
#       copy to the GPU host, which has no reference checkout)
#   oracle/build_ref_cuda.sh build
#       compiles oracle/_ref/cuda_src/ with nvcc into oracle/_ref/cuda_draw_lines*.so
#       with the reference's own flags (setup.py: -O3, C++17, -fPIC, hidden visibility)
#       plus -gencode for sm_103a (its setup.py passes no -arch for this module)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
STAGE="$HERE/_ref/cuda_src"
MODE="${1:-build}"
if [ "$MODE" = stage ]; then
    REF="${2:-/root/reference}"
    SRC="$REF/cbclib_v2/_src/src"
    if [ ! -f "$SRC/cuda_draw_lines.cu" ]; then
        echo "build_ref_cuda: $SRC/cuda_draw_lines.cu not found, skipping" >&2
        exit 0
    fi
    mkdir -p "$STAGE"
    for f in cuda_draw_lines.cu cupy_array.hpp include.hpp array_view.hpp cuda_geometry.hpp; do
        install -m 644 "$SRC/$f" "$STAGE/$f"
    done
    PB="$(python3 -c 'import pybind11; print(pybind11.get_include())')"
    rm -rf "$STAGE/pybind11_include"
    cp -r "$PB" "$STAGE/pybind11_include"
    echo "build_ref_cuda: staged into $STAGE"
    exit 0
fi
if [ ! -f "$STAGE/cuda_draw_lines.cu" ]; then
    echo "build_ref_cuda: nothing staged in $STAGE" >&2
    exit 1
fi
EXT="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
TARGET="$HERE/_ref/cuda_draw_lines$EXT"
if [ -f "$TARGET" ] && [ "$TARGET" -nt "$STAGE/cuda_draw_lines.cu" ]; then
    echo "$TARGET"
    exit 0
fi
PYINC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
NPINC="$(python3 -c 'import numpy; print(numpy.get_include())')"
nvcc -O3 -std=c++17 -shared -gencode arch=compute_103a,code=sm_103a \
    --compiler-options -fPIC,-O3,-fvisibility=hidden,-g0 \
    -I"$STAGE/pybind11_include" -I"$PYINC" -I"$NPINC" \
    "$STAGE/cuda_draw_lines.cu" -o "$TARGET.tmp" -lcudart
mv "$TARGET.tmp" "$TARGET"
echo "$TARGET"
