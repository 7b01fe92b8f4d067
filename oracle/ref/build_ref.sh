#!/usr/bin/env bash
# Builds oracle/_ref/libmipt_ref.so from the reference's own host headers, read
# in place from the reference checkout (default /root/reference), with the
# project-written CUDA-Q stub in oracle/ref/stub. Test infrastructure only: the
# library generates and checks the golden fixtures under tests/golden/.
# Exits 0 without building when the reference checkout is absent.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${MIPT_REFERENCE_ROOT:-/root/reference}"
out="$here/../_ref"
if [ ! -d "$ref/cpp/include/mipt" ]; then
    echo "build_ref: reference checkout not found at $ref; skipping" >&2
    exit 0
fi
mkdir -p "$out"
g++ -std=c++20 -O2 -fPIC -shared -w \
    -I"$here/stub" -I"$ref/cpp/include" \
    "$here/ref_harness.cpp" -o "$out/libmipt_ref.so" -ldl
echo "build_ref: wrote $out/libmipt_ref.so"
