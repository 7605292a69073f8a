#!/bin/sh
# Builds reference-derived golden-vector tools into oracle/_ref/ (git-ignored).
#   ref_tables: the reference's own FunctionData/PPolynomial host code
#               (FunctionData.inl:112-205) driven by oracle/ref_tables_driver.cu.
# The reference sources are read in place from $PRGPU_REFERENCE (default
# /root/reference); nothing is copied into the repository.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
REF=${PRGPU_REFERENCE:-/root/reference}
OUT="$HERE/_ref"
mkdir -p "$OUT"
if [ ! -f "$REF/FunctionData.inl" ]; then
  echo "reference tree not found at $REF" >&2
  exit 3
fi
/usr/local/cuda/bin/nvcc -std=c++17 -x cu -Xcompiler -ffp-contract=off -I"$REF" \
  "$HERE/ref_tables_driver.cu" -o "$OUT/ref_tables" 2>"$OUT/ref_tables.build.log"
echo "$OUT/ref_tables"
