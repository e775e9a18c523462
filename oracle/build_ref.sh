#!/usr/bin/env bash
# Builds the reference's own CPU kernel (pybind11 module `kernel`) from its unmodified
# sources under /root/reference, with the stand-in headers in oracle/ref_shim/ placed
# first on the include path, and the reference's scalar fast_norm functions with the harness
# oracle/ref_fast_scalar.cpp. Output goes only to oracle/_ref/ (git-ignored).
# Needs pybind11 and the Python headers; when either is missing the build is skipped.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${HPDEX_REFERENCE_ROOT:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/cpp/mannwhitneyu.cpp" ]; then
  echo "build_ref: reference sources not present; skipped"; exit 0
fi
mkdir -p "$OUT"
# The reference's scalar fast_norm functions (src/cpp/include/common.hpp, from fast_erfc up to
# its first SIMD template), copied unmodified into _ref/ and compiled into a small library with
# oracle/ref_fast_scalar.cpp. Flags as the reference's own build (-O3, no -march).
awk '/force_inline_ double fast_erfc\(double x\)/{f=1} /^template<class D>/{f=0} f' \
  "$REF/src/cpp/include/common.hpp" > "$OUT/ref_fast_scalar_block.hpp"
if grep -q "p_asymptotic_less" "$OUT/ref_fast_scalar_block.hpp"; then
  g++ -O3 -std=c++17 -shared -fPIC -I"$OUT" "$HERE/ref_fast_scalar.cpp" \
    -o "$OUT/libref_fast_scalar.so"
  echo "build_ref: built $OUT/libref_fast_scalar.so"
else
  echo "build_ref: scalar fast_norm block not found in common.hpp; skipped"
fi
PYINC="$(python3 -c 'import sysconfig; print(sysconfig.get_paths()["include"])')"
PB11="$(python3 -c 'import pybind11; print(pybind11.get_include())' 2>/dev/null || true)"
if [ -z "$PB11" ] || [ ! -f "$PYINC/Python.h" ]; then
  echo "build_ref: pybind11 or Python headers missing; skipped"; exit 0
fi
SUFFIX="$(python3 -c 'import sysconfig; print(sysconfig.get_config_var("EXT_SUFFIX"))')"
g++ -O3 -std=c++17 -fopenmp -shared -fPIC \
  -I"$HERE/ref_shim" -I"$REF/src/cpp/include" -I"$PYINC" -I"$PB11" \
  "$REF/src/cpp/module.cpp" "$REF/src/cpp/mannwhitneyu.cpp" \
  -o "$OUT/kernel$SUFFIX"
echo "build_ref: built $OUT/kernel$SUFFIX"
