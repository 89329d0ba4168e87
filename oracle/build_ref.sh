#!/usr/bin/env bash
# Build the unmodified ABIE C library from its own sources into oracle/_ref/.
#
# The output is used only as a checker: tests and the golden-vector generator
# load it through ctypes to pin the C restatement in oracle/abie_oracle.c.
# Sources are compiled where they lie; nothing is copied into this repository.
# Flags follow the reference's setup.py (-O3 -std=c99 -fPIC -shared -fcommon);
# -fcommon is required because several headers hold tentative definitions.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/common.c" ]; then
    echo "build_ref: no reference sources at $REF; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
SRCS=(common.c integrator_gauss_radau15.c integrator_wisdom_holman.c integrator_runge_kutta.c additional_forces.c)
ARGS=()
for s in "${SRCS[@]}"; do ARGS+=("$REF/src/$s"); done
gcc -O3 -std=c99 -fPIC -shared -fcommon -I"$REF/src" "${ARGS[@]}" -lm -o "$OUT/libabie_ref.so"
echo "build_ref: wrote $OUT/libabie_ref.so"
