#!/usr/bin/env bash
# Builds the reference's own CPU recurrences (LCS.cpp, ED.cpp, SW.cpp) from their
# sources where they lie in the read-only reference checkout, unmodified, into
# oracle/_ref/.  Test infrastructure only: the binaries are the checker that pins
# the C restatement in oracle/oracle.c, never part of the product path.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
# The checkout is REFERENCE_ROOT, else $GME_REFERENCE_ROOT, else a directory named
# `reference` beside this repository's own directory.  Exits 0 without building
# when none of them holds the sources (the GPU host has no checkout).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REPO="$(dirname "$HERE")"
REF="${1:-${GME_REFERENCE_ROOT:-$(dirname "$REPO")/reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/LCS/LCS.cpp" ]; then
  echo "build_ref: reference sources not present at $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -O2 -w -o "$OUT/LCS" "$REF/LCS/LCS.cpp"
g++ -O2 -w -o "$OUT/ED"  "$REF/EditDistance/ED.cpp"
g++ -O2 -w -o "$OUT/SW"  "$REF/SmithWaterman/SW.cpp"
echo "build_ref: built $OUT/{LCS,ED,SW}"
