#!/usr/bin/env bash
# Builds the reference runner (oracle/ref_driver.cu) against the reference's
# own sources -- TEST INFRASTRUCTURE ONLY; nothing here is committed or
# shipped.  Everything it writes goes to oracle/_ref/ (git-ignored).
#
#   bash oracle/ref_build.sh stage   # where the reference checkout exists:
#                                    # copy its six source files into
#                                    # oracle/_ref/src/ (never committed)
#   bash oracle/ref_build.sh build   # on the GPU machine: compile with nvcc
#
# The reference is header-only plus turtle-sort.cu and is built the way its
# README builds it (nvcc, relocatable device code for dynamic parallelism,
# -lcuda -lcudadevrt).  One change is needed for GCC: the MultiSort member
# template re-declares the class's template parameter `Type`
# (turtle-sort.cuh:265,266,272), which MSVC accepts and GCC rejects; the
# staged copy renames it to MType on those three lines only.  The reference's
# 8-bit signed key type is `char` (turtle-sort.cu:999-1019), which is signed
# on x86 and unsigned on Arm; nvcc's device code follows the host ABI, so on
# an Arm host the reference sorts `char` keys in unsigned order.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
REF="${TURTLE_REFERENCE:-/root/reference}"
FILES="turtle-sort.cu turtle-sort.cuh turtle-buffer.cuh turtle-multi-sort.cuh quick-helper.cuh turtle-globals.cuh"

case "${1:-build}" in
  stage)
    mkdir -p "$SRC"
    for f in $FILES; do cp "$REF/$f" "$SRC/$f"; chmod u+w "$SRC/$f"; done
    sed -i -e '265s/typename Type/typename MType/' \
           -e '266s/Type\* hostDataToSort/MType* hostDataToSort/' \
           -e '272s/MultiSorter<Type,/MultiSorter<MType,/' "$SRC/turtle-sort.cuh"
    grep -n "MType" "$SRC/turtle-sort.cuh"
    ;;
  build)
    test -f "$SRC/turtle-sort.cu" || { echo "no staged reference sources in $SRC" >&2; exit 1; }
    NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
    "$NVCC" -std=c++17 -O3 -rdc=true -gencode arch=compute_103a,code=sm_103a \
        -w -I "$SRC" \
        "$HERE/ref_driver.cu" "$SRC/turtle-sort.cu" \
        -o "$OUT/turtle_ref" -lcuda -lcudadevrt
    echo "built $OUT/turtle_ref"
    ;;
  *)
    echo "usage: $0 stage|build" >&2; exit 2 ;;
esac
