#!/bin/sh
# Builds the reference's own CUDA program (DavidXu-JJ/PoissonRecon_GPU; maxDepth
# 8, fixed by its main.cu:69) into oracle/_ref/ref_cuda: test infrastructure and
# the GPU baseline, never part of the library.
#
#   sh oracle/ref_cuda.sh stage   copy the reference's source files, unchanged,
#                                 from the reference tree ($PRGPU_REFERENCE,
#                                 default /root/reference) into oracle/_ref/src
#                                 (git-ignored), so that a machine without the
#                                 tree (the Arm GPU machine) can build them
#   sh oracle/ref_cuda.sh build   compile oracle/_ref/ref_cuda for sm_103a from
#                                 oracle/_ref/src (or from the tree when present)
#
# The reference files are compiled as they are, with what the reference's
# CMakeLists.txt builds (main.cu CmdLineParser.cu Geometry.cu plyfile.cu
# Factor.cu, separable compilation).  Three things around them stand in for what
# the reference hard-codes or no longer finds:
#   * oracle/ref_shim comes first on the include path; its
#     thrust/async/reduce.h replaces the header CCCL 3 removed (main.cu:15);
#   * main.cu is compiled with -Dmain=prgpu_reference_main, so that the driver
#     (oracle/ref_cuda_driver.cu) calls either the stock main() or
#     pipelineBuildNodeArray;
#   * the program is linked with -Wl,--wrap=fopen (oracle/ref_shim/ref_io.cpp),
#     which opens the fixed /home/davidxu/ paths of main.cu:3251-3252 inside
#     $PRGPU_REF_IO_DIR.
# The reference's CMake build targets sm_80 with default optimisation; here the
# device code is built for sm_103a and the host code with -O3.  main.cu is
# compiled with -maxrregcount=64: for sm_103a nvcc 13 gives computeVectorField
# 72 registers, and its launch with 32x32 = 1024 threads (main.cu:3369-3372) then
# cannot start (72 x 1024 exceeds the 65536 registers of an SM); the reference
# never checks launches (Debug.cuh:10-24), so without the cap its vector field
# stays zero and a later Thrust call aborts on the pending error.  Host code is
# compiled with -ffp-contract=off: the reference was written on x86-64, where the
# host compiler does not fuse a*b+c; GCC on the Arm GPU machine does by default, and
# then 11% of the normalised normals' components (main.cu:561-568) differ by 1-2
# ulp from the x86 results.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
SRC="$OUT/src"
REF=${PRGPU_REFERENCE:-/root/reference}
FILES="main.cu CmdLineParser.cu CmdLineParser.cuh CmdLineParser.inl Geometry.cu Geometry.cuh Geometry.inl
 plyfile.cu PlyFile.cuh PointStream.cuh PointStream.inl Debug.cuh OctNode.cuh Hash.cuh BinaryNode.cuh
 Factor.cu Factor.cuh Polynomial.cuh Polynomial.inl PPolynomial.cuh PPolynomial.inl FunctionData.cuh
 FunctionData.inl ConfirmedPPolynomial.cuh Allocator.cuh Vector.cuh Vector.inl SparseMatrix.cuh
 SparseMatrix.inl ConfirmedSparseMatrix.cuh ConfirmedVector.cuh CG_CUDA.cuh exception.h helper_cuda.h
 helper_image.h helper_timer.h helper_string.h helper_functions.h MarchingCubes.cuh"

case "$1" in
stage)
  if [ ! -f "$REF/main.cu" ]; then
    echo "reference tree not found at $REF" >&2
    exit 3
  fi
  mkdir -p "$SRC"
  for f in $FILES; do cp "$REF/$f" "$SRC/$f"; done
  echo "$SRC"
  ;;
build)
  if [ -f "$REF/main.cu" ]; then IN="$REF"; else IN="$SRC"; fi
  if [ ! -f "$IN/main.cu" ]; then
    echo "no reference sources (run 'sh oracle/ref_cuda.sh stage' where the reference tree is)" >&2
    exit 3
  fi
  NVCC=${NVCC:-/usr/local/cuda/bin/nvcc}
  OBJ="$OUT/obj"
  mkdir -p "$OBJ"
  FLAGS="-std=c++17 -O3 -rdc=true -gencode arch=compute_103a,code=sm_103a -Xcompiler -O3,-ffp-contract=off -w"
  INC="-I$HERE/ref_shim -I$IN"
  pids=""
  "$NVCC" $FLAGS $INC -maxrregcount=64 -Dmain=prgpu_reference_main -c "$IN/main.cu" -o "$OBJ/main.o" \
    > "$OBJ/main.log" 2>&1 & pids="$pids $!"
  for u in CmdLineParser Geometry plyfile Factor; do
    "$NVCC" $FLAGS $INC -c "$IN/$u.cu" -o "$OBJ/$u.o" > "$OBJ/$u.log" 2>&1 & pids="$pids $!"
  done
  "$NVCC" $FLAGS $INC -c "$HERE/ref_cuda_driver.cu" -o "$OBJ/driver.o" > "$OBJ/driver.log" 2>&1 & pids="$pids $!"
  ${CXX:-g++} -O2 -c "$HERE/ref_shim/ref_io.cpp" -o "$OBJ/ref_io.o"
  fail=0
  for p in $pids; do wait $p || fail=1; done
  if [ $fail -ne 0 ]; then cat "$OBJ"/*.log >&2; exit 1; fi
  "$NVCC" -rdc=true -gencode arch=compute_103a,code=sm_103a "$OBJ/main.o" "$OBJ/CmdLineParser.o" "$OBJ/Geometry.o" \
    "$OBJ/plyfile.o" "$OBJ/Factor.o" "$OBJ/driver.o" "$OBJ/ref_io.o" -Xlinker --wrap=fopen -o "$OUT/ref_cuda"
  echo "$OUT/ref_cuda"
  ;;
*)
  echo "usage: sh oracle/ref_cuda.sh stage|build" >&2
  exit 2
  ;;
esac
