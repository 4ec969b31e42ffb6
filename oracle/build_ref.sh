#!/usr/bin/env bash
# Compile the reference ChIMES-lsq sources (serial, no MPI) into oracle/_ref/.
#
# Test infrastructure only: the binaries are the parity oracle and the CPU
# baseline.  Sources are compiled where they lie under the reference checkout
# (default /root/reference, override with CHIMES_REF_DIR); nothing is copied.
# The one missing external header is replaced by oracle/refstub (aborting stub).
#
# -ffp-contract=off keeps the reference's FP64 rounding sequence identical on
# x86_64 and aarch64 (GCC contracts a*b+c into FMA by default on aarch64).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${CHIMES_REF_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "build_ref.sh: reference sources not found at $REF/src" >&2
  exit 2
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-O3 -std=c++11 -ffp-contract=off -w -I"$HERE/refstub/src" -I"$REF/src")
COMMON=(functions.C Ewald.C ClassDefs.C Fcut.C Cluster.C util.C Cheby.C io_styles.C feexcept.C input.C)
cd "$REF/src"
"$CXX" "${FLAGS[@]}" chimes_lsq.C A_Matrix.C "${COMMON[@]}" -o "$OUT/chimes_lsq" &
"$CXX" "${FLAGS[@]}" chimes_md.C "${COMMON[@]}" -o "$OUT/chimes_md" &
wait %1 && wait %2
echo "built $OUT/chimes_lsq $OUT/chimes_md"
