#!/bin/sh
# Builds oracle/_build/librefharness.so (the reference-replay harness) when the
# reference's device code (oracle/_ref/pdflow_ref.cubin) and layout header are
# present.  Test infrastructure only.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ORACLE=$(dirname "$HERE")
CUDA=${CUDA_HOME:-/usr/local/cuda}
if [ ! -f "$ORACLE/_ref/csf_layout.h" ] || { [ ! -f "$ORACLE/_ref/pdflow_ref.cubin" ] && [ ! -f "$ORACLE/_ref/pdflow_ref.fatbin" ]; }; then
    echo "reference device code not built (run make -C oracle/ref where the reference sources exist)" >&2
    exit 3
fi
mkdir -p "$ORACLE/_build"
${CC:-gcc} -O2 -fPIC -shared -std=c11 -Wall -I"$CUDA/include" -I"$ORACLE/_ref" \
    "$HERE/refharness.c" -o "$ORACLE/_build/librefharness.so" \
    -L"$CUDA/lib64/stubs" -L"$CUDA/lib64" -lcuda
