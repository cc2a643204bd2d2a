#!/bin/bash
# Builds the reference's own CPU path (its OpenMP branch, no -DGPU) straight from
# the reference sources, plus oracle/ref_harness.cu, into oracle/_ref/libg3lref.so.
#
# The sources are compiled where they lie (G3L_REF_SRC, default
# /root/reference/src); nothing is copied.  -ffp-contract=off keeps the host
# arithmetic free of fused multiply-adds on every platform, so the build and the
# oracle restatement evaluate the same IEEE operations.
#
# This script is the one place that names the reference's mount point; the Python
# side asks it (`build_ref.sh --where`) instead of repeating the path.
set -euo pipefail
REF=${G3L_REF_SRC:-/root/reference/src}
if [ "${1:-}" = "--where" ]; then
    echo "$REF"
    exit 0
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/NNMap_Model.cu" ]; then
    echo "reference sources not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT/obj"
CXXF="-std=c++17 -O2 -fopenmp -fPIC -ffp-contract=off -I$REF"
NVF="-std=c++17 -O3 -rdc=true -Xcompiler -fopenmp,-fPIC,-ffp-contract=off -I$REF"
pids=()
for f in hcubature Cosmology Params Function Function2D; do
    g++ $CXXF -c "$REF/$f.cpp" -o "$OUT/obj/$f.o" & pids+=($!)
done
# the table precomputation (doPrecomputations.x); it needs C++20 for <numbers>, and
# Powerspectrum.cpp uses std::min_element without including <algorithm>
for f in Powerspectrum HMF; do
    g++ ${CXXF/-std=c++17/-std=c++20} -include algorithm -c "$REF/$f.cpp" -o "$OUT/obj/$f.o" &
    pids+=($!)
done
for f in HOD generalFunctions NNMap_Model NMapMap_Model; do
    nvcc $NVF -c "$REF/$f.cu" -o "$OUT/obj/$f.o" 2> "$OUT/obj/$f.log" & pids+=($!)
done
nvcc $NVF -c "$HERE/ref_harness.cu" -o "$OUT/obj/ref_harness.o" & pids+=($!)
# the SCALING build (satellite-variance rescaling, src/Makefile:17-21): NNMap model only
mkdir -p "$OUT/obj_scaling"
nvcc $NVF -DSCALING=1 -c "$REF/NNMap_Model.cu" -o "$OUT/obj_scaling/NNMap_Model.o" \
    2> "$OUT/obj_scaling/NNMap_Model.log" & pids+=($!)
nvcc $NVF -DSCALING=1 -c "$HERE/ref_harness.cu" -o "$OUT/obj_scaling/ref_harness.o" & pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
nvcc -shared -rdc=true -Xcompiler -fopenmp "$OUT"/obj/*.o -o "$OUT/libg3lref.so"
echo "built $OUT/libg3lref.so"
common=()
for f in hcubature Cosmology Params Function Function2D HOD generalFunctions; do
    common+=("$OUT/obj/$f.o")
done
nvcc -shared -rdc=true -Xcompiler -fopenmp "${common[@]}" "$OUT"/obj_scaling/*.o \
    -o "$OUT/libg3lref_scaling.so"
echo "built $OUT/libg3lref_scaling.so"
