#!/bin/sh
# Builds the reference's own CPU implementation of the frame-development path
# (lib/ref plus the host colour, noise and AWB files it calls) from the
# sources where they lie in the reference tree, into oracle/_ref/. Nothing is
# copied out of the reference. The result is test infrastructure: the tests
# and the golden-fixture script use it to pin the oracle restatement in
# oracle/craw_oracle.c; it never ships and never runs in the product path.
#
# Also builds and runs the reference's own CPU unit tests (test_ref_debayer,
# test_awb) against it, which is the check that the build is the reference.
#
#   usage: oracle/build_ref.sh [REFERENCE_DIR]
#   (default: $CRAW_REFERENCE_DIR, else /root/reference)
set -eu
REF=${1:-${CRAW_REFERENCE_DIR:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -d "$REF/lib/ref" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
mkdir -p "$OUT/obj"
CC=${CC:-gcc}
CFLAGS="-std=c2x -O2 -fPIC -ffp-contract=off -w -I$HERE/shim -I$REF/include -I$REF/lib"
SRCS="$REF/lib/ref/ref_chroma.c $REF/lib/ref/ref_color.c $REF/lib/ref/ref_debayer.c
      $REF/lib/ref/ref_defringe.c $REF/lib/ref/ref_denoise.c $REF/lib/ref/ref_false_color.c
      $REF/lib/ref/ref_highlight.c $REF/lib/ref/ref_lens.c $REF/lib/ref/ref_sharpen.c
      $REF/lib/profile.c $REF/lib/colorspace.c $REF/lib/gamut.c $REF/lib/awb.c
      $REF/lib/awb_smoother.c $REF/lib/noise.c $REF/lib/lens.c"
OBJS=""
for s in $SRCS; do
    o="$OUT/obj/$(basename "$s" .c).o"
    $CC $CFLAGS -c "$s" -o "$o" &
    OBJS="$OBJS $o"
done
wait
# gamut.h is not public in the reference; export its two functions anyway
# (they are plain global symbols) so the tests can reach them.
$CC -shared -o "$OUT/libcraw_ref.so" $OBJS -lm
for t in test_ref_debayer test_awb; do
    $CC $CFLAGS "$REF/tests/$t.c" $OBJS -lm -o "$OUT/$t"
    "$OUT/$t" > "$OUT/$t.log" 2>&1 || { cat "$OUT/$t.log"; exit 1; }
    tail -1 "$OUT/$t.log"
done
echo "built $OUT/libcraw_ref.so"
