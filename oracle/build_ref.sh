#!/usr/bin/env bash
# Compiles the reference diffvg CPU path (pybind11 module) from the read-only
# reference sources into oracle/_ref/, for use as a test oracle only.
# The reference's own CMake build is not used: its pybind11/ and thrust/
# submodules are empty, so the pip pybind11 headers and the CUDA toolkit's
# CCCL (thrust in CPP mode) stand in for them.
# -ffp-contract=off keeps the arithmetic unfused on every host architecture,
# so that the x86 and aarch64 builds round identically.
set -euo pipefail
REF=${DVG_REFERENCE_DIR:-/root/reference}
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/diffvg.cpp" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref build" >&2
  exit 0
fi
mkdir -p "$OUT"
PYINC=$(python3 -c "import sysconfig; print(sysconfig.get_paths()['include'])")
PBINC=$(python3 -c "import pybind11; print(pybind11.get_include())")
SUFFIX=$(python3 -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
CUDA=${CUDA_HOME:-/usr/local/cuda}
TARGET="$OUT/diffvg$SUFFIX"
if [ -f "$TARGET" ] && [ "$TARGET" -nt "$REF/diffvg.cpp" ] && [ "$TARGET" -nt "$0" ]; then
  exit 0
fi
g++ -O3 -std=c++17 -shared -fPIC -ffp-contract=off -w \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
  -I"$PBINC" -I"$PYINC" -I"$CUDA/include/cccl" -I"$CUDA/include" \
  "$REF/atomic.cpp" "$REF/color.cpp" "$REF/diffvg.cpp" "$REF/parallel.cpp" \
  "$REF/scene.cpp" "$REF/shape.cpp" -lpthread -o "$TARGET.tmp"
mv "$TARGET.tmp" "$TARGET"
echo "built $TARGET"
