#!/bin/sh
# Builds oracle/_ref/libinfernal_ref.so: Infernal's own scanner sources,
# compiled in place from the read-only reference tree against the
# project-written Easel/HMMER shim in oracle/ref_shim, plus the harness
# oracle/ref_harness.c.  Parity checker only; the product never links it.
#
# Also compiles, into oracle/_ref/adapter_obj, the Infernal-side adapter
# (infernal_gb300/adapter/infernal_gb300_adapter.c) against the reference's
# own headers, with the harness and the stand-ins of the two scanners the
# adapter does not provide: tests/test_adapter_cpu.py links these objects
# with the reference's non-scanner objects and the host-emulation build of
# the GPU library.
#
# Usage: oracle/build_ref.sh <reference_root>
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ROOT=$(cd "$HERE/.." && pwd)
REF=${1:?usage: build_ref.sh <reference_root>}
SRC="$REF/src"
OUT="$HERE/_ref"
[ -f "$SRC/cm_dpsearch.c" ] || { echo "reference sources not found under $SRC" >&2; exit 2; }
mkdir -p "$OUT/obj" "$OUT/adapter_obj"
CFLAGS="-O2 -fPIC -ffp-contract=off -w -I$HERE/ref_shim -I$SRC"
rm -f "$OUT"/obj/*.o "$OUT"/adapter_obj/*.o "$OUT/libinfernal_ref.so"
export CFLAGS OUT
printf '%s\n' "$SRC/cm_dpsearch.c" "$SRC/cm_dpsearch_trunc.c" "$SRC/logsum.c" "$SRC/cm_mx.c" \
  "$SRC/cm_tophits.c" "$SRC/cm_trunc.c" "$SRC/cm_qdband.c" "$SRC/display.c" "$SRC/cm_modelconfig.c" \
  "$HERE/ref_harness.c" "$HERE/ref_offpath.c" |
  xargs -P 8 -I{} sh -c 'gcc $CFLAGS -c "{}" -o "$OUT/obj/$(basename "{}" .c).o"'
gcc -shared -o "$OUT/libinfernal_ref.so" "$OUT"/obj/*.o -lm
gcc $CFLAGS -I"$ROOT/include" -c "$ROOT/infernal_gb300/adapter/infernal_gb300_adapter.c" -o "$OUT/adapter_obj/adapter.o"
gcc $CFLAGS -c "$HERE/adapter_stubs.c" -o "$OUT/adapter_obj/adapter_stubs.o"
echo "built $OUT/libinfernal_ref.so"
