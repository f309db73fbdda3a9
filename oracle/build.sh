#!/usr/bin/env bash
# Build recipe for the test oracle (CPU only).
#   oracle/_build/liboracle.so  -- the FP64 CPU restatement (fw_oracle.cpp)
#   oracle/_ref/libgbref.so     -- the reference project's own CPU functions,
#                                  compiled from its headers where they lie;
#                                  built only when the reference tree exists.
# Both outputs are git-ignored; the first is rebuilt on every machine.
set -euo pipefail
here="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
mkdir -p "$here/_build"
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -pthread \
    -o "$here/_build/liboracle.so" "$here/fw_oracle.cpp"

# the reference tree where it lies (GPUBOSCIA_REFERENCE overrides); its root
# is recorded beside the library so the CPU tests that read the reference's
# data files find them without naming a path of their own
ref="${GPUBOSCIA_REFERENCE:-/root/reference}"
if [ -d "$ref/include/gpuboscia" ]; then
    mkdir -p "$here/_ref"
    nvcc -std=c++17 -O2 -Xcompiler -fPIC -Xcompiler -ffp-contract=off -shared \
        -I "$ref/include" -o "$here/_ref/libgbref.so" "$here/ref_shim.cu"
    printf '%s\n' "$(cd "$ref" && pwd)" > "$here/_ref/reference_root.txt"
fi
