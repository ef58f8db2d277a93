#!/bin/sh
# Compile the reference's serial CPU solvers, unmodified, from their sources
# where they lie (read-only) into oracle/_ref/bin.  Test infrastructure: used
# to cross-check the oracle's restatement; never part of the product.
#   oracle/ref_build.sh [REFERENCE_ROOT]
set -e
REF=${1:-/root/reference}
OUT="$(cd "$(dirname "$0")" && pwd)/_ref/bin"
[ -d "$REF/src" ] || { echo "reference sources not found at $REF" >&2; exit 1; }
mkdir -p "$OUT"
for f in 24puzzle_expand.cc 24puzzle_expand_with_pdb.cpp 24puzzle.cc 15puzzle_expand.cc; do
  g++ -std=c++11 -O2 -w -o "$OUT/${f%.*}" "$REF/src/$f"
done
echo "built into $OUT"
