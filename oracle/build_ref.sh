#!/usr/bin/env bash
# Build the reference's own CPU code into oracle/_ref/ (TEST INFRASTRUCTURE ONLY).
#
# Runs only where the reference checkout exists (default /root/reference, or
# $TSG_REFERENCE_DIR).  Sources are compiled where they lie, unmodified; the
# outputs go to oracle/_ref/ (git-ignored).  Two libraries:
#   libthmkl_ref.so  thmkl_dcsrmultcsr.c (OpenMP CSR SpGEMM + mmio loader),
#                    its main() renamed so the routine can be called by ctypes
#   libstir_ref.so   main_spgemm-col.cu host routines through ref_shim_stir.cu;
#                    two shims let the 2021 source build with CUDA 13:
#                    cudaThreadSynchronize (removed API) -> cudaDeviceSynchronize,
#                    cudaDeviceProp::clockRate (removed field) -> .major
set -euo pipefail
REF="${TSG_REFERENCE_DIR:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/thmkl_dcsrmultcsr.c" ]; then
  echo "reference checkout not found at $REF; nothing to build" >&2
  exit 0
fi
mkdir -p "$OUT"
gcc -O3 -fopenmp -fPIC -shared -w -Dmain=thmkl_ref_main -I"$REF" \
    "$REF/thmkl_dcsrmultcsr.c" -o "$OUT/libthmkl_ref.so"
nvcc -O2 -w -Xcompiler -fPIC -shared -gencode arch=compute_103a,code=sm_103a \
    -Dmain=stir_ref_main -DcudaThreadSynchronize=cudaDeviceSynchronize -DclockRate=major \
    -I"$REF" "$HERE/ref_shim_stir.cu" -o "$OUT/libstir_ref.so"
echo "built $OUT/libthmkl_ref.so $OUT/libstir_ref.so"
