#!/bin/sh
# Builds the CPU oracle (test infrastructure) into oracle/liboracle.so.
# -ffp-contract=off keeps host arithmetic unfused, as on the reference's x86 host;
# the oracle's explicit fmaf()/fma() calls mark the reference's device-side FMAs.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
ARCHFLAGS=""
case "$(uname -m)" in
  x86_64) ARCHFLAGS="-mfma" ;;
esac
${CXX:-g++} -O2 -std=c++17 -fopenmp -ffp-contract=off $ARCHFLAGS -fPIC -shared \
  -o "$HERE/liboracle.so" "$HERE/oracle.cpp"
