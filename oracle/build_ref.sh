#!/usr/bin/env bash
# Builds the UNMODIFIED reference forward model, Jacobian and retrieval
# (src/jurassic.c + src/retrieval.c of the reference tree) together with
# oracle/ref_harness.c into oracle/_ref/libjref_<tag>.so.
#
# TEST INFRASTRUCTURE ONLY (the reference-as-oracle and the timed CPU
# baseline).  The reference sources are compiled where they lie; nothing is
# copied.  GSL is absent here, so the reference includes resolve to the
# project's own compat shim under oracle/gsl_shim.
#
# usage: oracle/build_ref.sh <tag> [extra -D dimension flags]
#   e.g. oracle/build_ref.sh std
#        oracle/build_ref.sh big -DND=320 -DNG=5 -DNR=64
#        oracle/build_ref.sh --where     (prints the reference tree used)
# The reference tree is $JURASSIC_REF_DIR; unset, it is the build
# container's read-only mount below (the only place in the repository that
# names it).  The GPU machine has no reference tree.
set -euo pipefail
REF=${JURASSIC_REF_DIR:-/root/reference}
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
if [ "${1:-}" = "--where" ]; then
  if [ -f "$REF/src/jurassic.c" ]; then echo "$REF"; exit 0; fi
  exit 3
fi
TAG=${1:-std}
shift || true
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ ! -f "$REF/src/jurassic.c" ]; then
  echo "reference sources not found under $REF/src; nothing built" >&2
  exit 3
fi
CC=${CC:-gcc}
# -ffp-contract=off: no FMA contraction, so results are the same on x86 and Arm.
CFLAGS="-O2 -fPIC -fopenmp -ffp-contract=off -w -I$HERE/gsl_shim -I$REF/src -DVERSION=\"reference\" $*"
TMP=$(mktemp -d)
trap 'rm -rf "$TMP"' EXIT
$CC $CFLAGS -c "$REF/src/jurassic.c" -o "$TMP/jurassic.o"
$CC $CFLAGS -Dmain=jref_retrieval_main \
  -Dwrite_atm=jref_hook_write_atm -Dwrite_obs=jref_hook_write_obs \
  -Dwrite_matrix=jref_hook_write_matrix \
  -c "$REF/src/retrieval.c" -o "$TMP/retrieval.o"
$CC $CFLAGS -c "$HERE/ref_harness.c" -o "$TMP/ref_harness.o"
$CC -shared -fopenmp -o "$OUT/libjref_${TAG}.so" "$TMP/jurassic.o" "$TMP/retrieval.o" "$TMP/ref_harness.o" -lm
echo "built $OUT/libjref_${TAG}.so"
