#!/bin/sh
# Build the checker library oracle/_ref/libassist_ref.so from the UNMODIFIED
# ASSIST sources where they lie, against this project's REBOUND stand-in.
# Flags follow ASSIST's own build (setup.py:107-136: -O3 -std=c99
# -fno-strict-aliasing); -ffp-contract=off keeps x86 and Arm results identical.
# Usage: oracle/build_ref.sh [ASSIST source root]   (default: /root/reference)
set -e
REF="${1:-${ASSIST_REFERENCE:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
if [ ! -f "$REF/src/forces.c" ]; then
    echo "build_ref.sh: ASSIST sources not found under $REF; skipping" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
gcc -O3 -std=c99 -D_GNU_SOURCE -fno-strict-aliasing -ffp-contract=off -fPIC -shared -w \
    -I "$HERE/ref_standin" -I "$REF/src" \
    "$REF/src/assist.c" "$REF/src/forces.c" "$REF/src/spk.c" "$REF/src/ascii_ephem.c" "$REF/src/tools.c" \
    "$HERE/ref_harness.c" -o "$HERE/_ref/libassist_ref.so" -lm
echo "built $HERE/_ref/libassist_ref.so"
