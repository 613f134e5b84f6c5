#!/usr/bin/env bash
# Build oracle/_ref/libvpmc_ref.so from the reference's own CPU sources, read
# in place from the reference tree named by VPMC_REFERENCE_DIR, plus
# oracle/ref_shim.cpp.  Test infrastructure only: the output is git-ignored
# and used to pin the oracle and make golden vectors.  Exits 0 without
# building when VPMC_REFERENCE_DIR is unset or holds no reference tree.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${VPMC_REFERENCE_DIR:-}"
out="$here/_ref"
if [ -z "$ref" ] || [ ! -d "$ref/src/cpu" ]; then
    echo "build_ref: no reference tree (set VPMC_REFERENCE_DIR); skipping" >&2
    exit 0
fi
mkdir -p "$out/stub/thrust"
# src/utilities.cu includes <thrust/host_vector.h> unconditionally although its
# CPU branch does not use it; an empty stub lets it compile as C++.
: > "$out/stub/thrust/host_vector.h"
CXX="${CXX:-g++}"
flags=(-std=c++20 -O2 -fPIC -fopenmp -ffp-contract=off -w
       -I"$ref/include" -I"$out/stub")
srcs=("$ref/src/cpu/hash.cpp" "$ref/src/omp/hash_omp.cpp"
      "$ref/src/cpu/evaluate_vorticity.cpp" "$ref/src/cpu/monte_carlo_bs.cpp"
      "$ref/src/cpu/monte_carlo_sampling.cpp" "$ref/src/cpu/build_particle_sets.cpp")
"$CXX" "${flags[@]}" -shared -o "$out/libvpmc_ref.so" \
    "$here/ref_shim.cpp" "${srcs[@]}" -x c++ "$ref/src/utilities.cu" -x none
echo "build_ref: wrote $out/libvpmc_ref.so"
