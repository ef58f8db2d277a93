#!/bin/sh
# Compile the reference's serial CPU solvers, unmodified, from their sources
# where they lie (read-only) into oracle/_ref/bin.  Test infrastructure: used
# to cross-check the oracle's restatement; never part of the product.
#   oracle/ref_build.sh [--optional] [REFERENCE_ROOT]
# REFERENCE_ROOT defaults to $SLIDE_REFERENCE_DIR, else to the location of
# the reference checkout in the build container (/root/reference).  With
# --optional a missing checkout (as on the GPU machine) is not an error.
set -e
OPTIONAL=0
if [ "$1" = "--optional" ]; then OPTIONAL=1; shift; fi
REF=${1:-${SLIDE_REFERENCE_DIR:-/root/reference}}
OUT="$(cd "$(dirname "$0")" && pwd)/_ref/bin"
if [ ! -d "$REF/src" ]; then
  [ "$OPTIONAL" = 1 ] && { echo "reference sources not present: oracle/_ref not built"; exit 0; }
  echo "reference sources not found at $REF" >&2; exit 1
fi
mkdir -p "$OUT"
for f in 24puzzle_expand.cc 24puzzle_expand_with_pdb.cpp 24puzzle.cc 15puzzle_expand.cc; do
  g++ -std=c++11 -O2 -w -o "$OUT/${f%.*}" "$REF/src/$f"
done
echo "built into $OUT"
