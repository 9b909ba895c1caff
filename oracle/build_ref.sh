#!/usr/bin/env bash
# Builds the reference's own code for use as a checker, from the reference
# sources where they lie (never copied into the repository):
#   oracle/_ref/ref_rotations          rotations.c + a KAT driver (host, any CPU)
#   oracle/_ref/libemc_ref_kernels.so  emc_cuda.cu + emc_atomic.cu for sm_103a,
#                                      behind the C wrappers of ref_harness.cu
#                                      (only with --kernels; needs nvcc)
#   oracle/_ref/libemc_ref_helper.so   emc_helper.cpp + rotations.c (host) behind
#                                      the C wrappers of ref_helper_harness.cpp
#                                      (only with --helper)
# The reference tree is $EMC_REF_DIR, else the staged copy baseline/_ref/src
# (git-ignored; see --stage).  Outputs go to oracle/_ref/ only.
#   --stage   copy the reference files the checkers need from $EMC_REF_DIR into
#             baseline/_ref/src (git-ignored) so that a machine without the
#             reference tree (the GPU host) can build them too.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
repo="$(cd "$here/.." && pwd)"
out="$here/_ref"
ref="${EMC_REF_DIR:-$repo/baseline/_ref/src}"
want_kernels=0
want_helper=0
for a in "$@"; do
  case "$a" in
    --kernels) want_kernels=1 ;;
    --helper) want_helper=1 ;;
    --stage)
      mkdir -p "$repo/baseline/_ref/src"
      if [[ "$ref" == "$repo/baseline/_ref/src" ]]; then echo "--stage needs EMC_REF_DIR" >&2; exit 1; fi
      for f in rotations.c rotations.h emc_cuda.cu emc_atomic.cu emc_cuda_help.h emc_helper.h \
               emc_helper.cpp configs.h emc.conf; do
        cp "$ref/$f" "$repo/baseline/_ref/src/$f"
      done
      echo "staged reference sources in baseline/_ref/src"
      exit 0 ;;
  esac
done
if [[ ! -f "$ref/rotations.c" ]]; then
  echo "reference tree not found ($ref)" >&2
  exit 1
fi
mkdir -p "$out"
gcc -O2 -std=gnu99 -w -I"$here/shim" -I"$ref" -include stdio.h -include stdlib.h \
    -include string.h -include math.h \
    "$ref/rotations.c" "$here/ref_rotations_main.c" "$here/shim/spimage_stubs.c" -lm \
    -o "$out/ref_rotations"
if [[ $want_helper == 1 ]]; then
  # float arithmetic without contraction, as the reference's x86-64 build
  # (no FMA in its default target) evaluates it, on every host
  gcc -O2 -std=gnu99 -fPIC -w -ffp-contract=off -I"$here/shim" -I"$ref" -include stdio.h \
      -include stdlib.h -include string.h -include math.h -c "$ref/rotations.c" \
      -o "$out/rotations_helper.o"
  g++ -O2 -std=c++17 -fPIC -w -ffp-contract=off -I"$here/shim" -I"$ref" -include cstdio \
      -include cstring -shared "$ref/emc_helper.cpp" "$here/ref_helper_harness.cpp" \
      "$out/rotations_helper.o" -o "$out/libemc_ref_helper.so"
fi
if [[ $want_kernels == 1 ]]; then
  # emc_cuda.cu and emc_atomic.cu each define inblock_reduce, so they are
  # separate translation units, as in the reference's own build.
  flags=(-std=c++17 -O3 -gencode arch=compute_103a,code=sm_103a -Xcompiler -fPIC -w
         -I"$here/shim" -I"$ref" -DcudaThreadSynchronize=cudaDeviceSynchronize
         -include thrust/transform_reduce.h)
  nvcc "${flags[@]}" -c "$ref/emc_cuda.cu" -o "$out/emc_cuda.o" &
  nvcc "${flags[@]}" -c "$ref/emc_atomic.cu" -o "$out/emc_atomic.o" &
  nvcc "${flags[@]}" -c "$here/ref_harness.cu" -o "$out/ref_harness.o" &
  wait
  gcc -O2 -fPIC -c -I"$here/shim" "$here/shim/spimage_stubs.c" -o "$out/spimage_stubs.o"
  nvcc -shared -gencode arch=compute_103a,code=sm_103a "$out/emc_cuda.o" "$out/emc_atomic.o" \
      "$out/ref_harness.o" "$out/spimage_stubs.o" -lcufft -o "$out/libemc_ref_kernels.so"
fi
echo "built reference checker in $out"
