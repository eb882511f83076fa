#!/usr/bin/env bash
# Compiles the reference diffvg CPU path (pybind11 module) from the read-only
# reference sources into oracle/_ref/, for use as a test oracle only.
# The reference's own CMake build is not used: its pybind11/ and thrust/
# submodules are empty, so the pip pybind11 headers and the CUDA toolkit's
# CCCL (thrust in CPP mode) stand in for them.
# -ffp-contract=off keeps the arithmetic unfused on every host architecture,
# so that the x86 and aarch64 builds round identically.
#
# The reference checkout is DVG_REFERENCE_DIR (default /root/reference, where
# the build container mounts it).  `build_ref.sh --print-ref-dir` prints it.
#
# DVG_REF_VARIANT=defined builds a second module into oracle/_ref_defined/
# from a scratch copy of the sources (under a temporary directory, removed
# afterwards) in which the one uninitialised read of the reference's closest-
# point / stroke quintic is given a value: the isolator interval array
# (compute_distance.h:200, within_distance.h:195) starts as {-1,-1,-1,-1}, so
# the slot that the reference leaves unset when -B/5 falls outside [0, 1]
# reads -1 (skipped) instead of whatever an earlier evaluation left on the
# stack.  Nothing else changes.  It serves to show which differences between
# the reference and this project come from that read.
set -euo pipefail
REF=${DVG_REFERENCE_DIR:-/root/reference}
if [ "${1:-}" = "--print-ref-dir" ]; then
  echo "$REF"
  exit 0
fi
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
VARIANT=${DVG_REF_VARIANT:-stock}
if [ ! -f "$REF/diffvg.cpp" ]; then
  echo "reference sources not found at $REF; skipping the reference module build" >&2
  exit 0
fi
case "$VARIANT" in
  stock) OUT="$HERE/_ref" ;;
  defined) OUT="$HERE/_ref_defined" ;;
  *) echo "unknown DVG_REF_VARIANT $VARIANT" >&2; exit 1 ;;
esac
mkdir -p "$OUT"
PYINC=$(python3 -c "import sysconfig; print(sysconfig.get_paths()['include'])")
PBINC=$(python3 -c "import pybind11; print(pybind11.get_include())")
SUFFIX=$(python3 -c "import sysconfig; print(sysconfig.get_config_var('EXT_SUFFIX'))")
CUDA=${CUDA_HOME:-/usr/local/cuda}
TARGET="$OUT/diffvg$SUFFIX"
if [ -f "$TARGET" ] && [ "$TARGET" -nt "$REF/diffvg.cpp" ] && [ "$TARGET" -nt "$0" ]; then
  exit 0
fi
SRC="$REF"
if [ "$VARIANT" = "defined" ]; then
  SRC=$(mktemp -d)
  trap 'rm -rf "$SRC"' EXIT
  cp "$REF"/*.h "$REF"/*.cpp "$SRC"/
  for f in compute_distance.h within_distance.h; do
    grep -q 'float intervals\[4\];' "$SRC/$f"
    sed -i 's/float intervals\[4\];/float intervals[4] = {-1.f, -1.f, -1.f, -1.f};/' "$SRC/$f"
  done
fi
g++ -O3 -std=c++17 -shared -fPIC -ffp-contract=off -w \
  -DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_CPP \
  -I"$SRC" -I"$PBINC" -I"$PYINC" -I"$CUDA/include/cccl" -I"$CUDA/include" \
  "$SRC/atomic.cpp" "$SRC/color.cpp" "$SRC/diffvg.cpp" "$SRC/parallel.cpp" \
  "$SRC/scene.cpp" "$SRC/shape.cpp" -lpthread -o "$TARGET.tmp"
mv "$TARGET.tmp" "$TARGET"
echo "built $TARGET"
