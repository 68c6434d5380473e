#!/bin/sh
# Builds oracle/_ref/libinfernal_ref.so: Infernal's own scanner sources,
# compiled in place from the read-only reference tree against the
# project-written Easel/HMMER shim in oracle/ref_shim, plus the harness
# oracle/ref_harness.c.  Parity checker only; the product never links it.
#
# Usage: oracle/build_ref.sh [reference_root]   (default /root/reference)
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${1:-/root/reference}
SRC="$REF/src"
OUT="$HERE/_ref"
[ -f "$SRC/cm_dpsearch.c" ] || { echo "reference sources not found under $SRC" >&2; exit 2; }
mkdir -p "$OUT/obj"
CFLAGS="-O2 -fPIC -ffp-contract=off -w -I$HERE/ref_shim -I$SRC"
rm -f "$OUT"/obj/*.o "$OUT/libinfernal_ref.so"
export CFLAGS OUT
printf '%s\n' "$SRC/cm_dpsearch.c" "$SRC/cm_dpsearch_trunc.c" "$SRC/logsum.c" "$SRC/cm_mx.c" \
  "$SRC/cm_tophits.c" "$SRC/cm_trunc.c" "$SRC/cm_qdband.c" "$SRC/display.c" "$SRC/cm_modelconfig.c" \
  "$HERE/ref_harness.c" "$HERE/ref_offpath.c" |
  xargs -P 8 -I{} sh -c 'gcc $CFLAGS -c "{}" -o "$OUT/obj/$(basename "{}" .c).o"'
gcc -shared -o "$OUT/libinfernal_ref.so" "$OUT"/obj/*.o -lm
echo "built $OUT/libinfernal_ref.so"
