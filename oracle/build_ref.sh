#!/usr/bin/env bash
# Builds oracle/_ref/liboracle_ref.so: the reference's own sparse-grid headers and
# bonxai_map/src/probabilistic_map.cpp, compiled unmodified from where they lie,
# behind the C API in oracle/oracle_api.h (test infrastructure only).
#
# Only this container has the reference sources; the GPU machine uses the golden
# fixtures under tests/golden/ and the restatement in oracle/bonxai_oracle.cpp.
# Usage: oracle/build_ref.sh [reference_root]   (default /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${BONXAI_REFERENCE:-/root/reference}}"
if [ ! -f "$REF/bonxai_map/src/probabilistic_map.cpp" ]; then
  echo "reference sources not found under $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$HERE/_ref"
g++ -std=c++17 -O3 -ffp-contract=off -fPIC -shared \
  -I"$REF/bonxai_core/include" -I"$REF/bonxai_map/include" \
  -I"$HERE/eigen_shim" -I"$HERE" \
  "$HERE/ref_harness.cpp" "$REF/bonxai_map/src/probabilistic_map.cpp" \
  -o "$HERE/_ref/liboracle_ref.so.tmp"
mv "$HERE/_ref/liboracle_ref.so.tmp" "$HERE/_ref/liboracle_ref.so"
echo "built $HERE/_ref/liboracle_ref.so"
