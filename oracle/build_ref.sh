#!/usr/bin/env bash
# Builds the reference's own CPU recurrences (LCS.cpp, ED.cpp, SW.cpp) from their
# sources where they lie in the read-only reference checkout, unmodified, into
# oracle/_ref/.  Test infrastructure only: the binaries are the checker that pins
# the C restatement in oracle/oracle.c, never part of the product path.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default /root/reference)
# Exits 0 without building when the reference checkout is absent (the GPU host).
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "$0")" && pwd)"
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
