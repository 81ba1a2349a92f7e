#!/bin/bash
# Builds oracle/_ref/libmgref.so: the reference MGmol's own hot-path
# translation units, compiled unmodified from the read-only source tree,
# against the single-task shims in oracle/shim/, plus oracle/ref_driver.cpp.
# Test infrastructure only (pins the oracle restatement; records fixtures).
# Usage: oracle/build_ref.sh [path-to-mgmol-source]
#   (default: $MGMOL_SRC, else /root/reference)
set -e
REF=${1:-${MGMOL_SRC:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
SRC=$REF/src
if [ ! -d "$SRC/pb" ]; then
    echo "build_ref: reference source not found at $REF; skipped" >&2
    exit 0
fi
OUT=$HERE/_ref
mkdir -p "$OUT/obj"
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O2 -fopenmp -ffp-contract=off -fPIC -w"
INC="-I$HERE/shim -I$SRC -I$SRC/pb -I$SRC/tools -I$SRC/linear_algebra -I$SRC/local_matrices -I$SRC/DistMatrix -I$SRC/sparse_linear_algebra -I$SRC/radial"
TUS="pb/Laph2.cc pb/Laph4.cc pb/Laph4M.cc pb/Laph6.cc pb/Laph8.cc tools/MPIdata.cc tools/MGmol_MPI.cc tools/mgmol_mpi_tools.cc Mesh.cc pb/FDkernels.cc pb/MGkernels.cc pb/Grid.cc pb/PEenv.cc pb/GridFunc.cc pb/GridFuncVector.cc pb/FDoper.cc pb/Lap.cc tools/Timer.cc tools/Vector3D.cc linear_algebra/mputils.cc GridMask.cc GridMaskMax.cc GridMaskMult.cc Map2Masks.cc SubCell.cc tools/coloring.cc tools/SymmetricMatrix.cc"
OBJS=""
pids=""
for tu in $TUS; do
    o=$OUT/obj/$(echo "$tu" | tr '/' '_' | sed 's/\.cc$/.o/')
    $CXX $FLAGS $INC -c "$SRC/$tu" -o "$o" &
    pids="$pids $!"
    OBJS="$OBJS $o"
done
$CXX $FLAGS $INC -c "$HERE/ref_driver.cpp" -o "$OUT/obj/ref_driver.o" &
pids="$pids $!"
# FunctionsPacking's colourings (tools/coloring.cc, tools/SymmetricMatrix.cc)
$CXX $FLAGS $INC -c "$HERE/ref_pack.cpp" -o "$OUT/obj/ref_pack.o" &
pids="$pids $!"
# S and H through the reference's local matrices and LocalMatrices2DistMatrix
# (its 1e-14 filter), with single-task stand-ins for the ScaLAPACK-backed
# DistMatrix / SparseDistMatrix headers (oracle/shim_dist/, searched first)
MINC="-I$HERE/shim_dist $INC"
for tu in local_matrices/LocalMatrices.cc local_matrices/SquareLocalMatrices.cc LocalMatrices2DistMatrix.cc; do
    o=$OUT/obj/$(echo "$tu" | tr '/' '_' | sed 's/\.cc$/.o/')
    $CXX $FLAGS $MINC -c "$SRC/$tu" -o "$o" &
    pids="$pids $!"
    OBJS="$OBJS $o"
done
$CXX $FLAGS $MINC -c "$HERE/ref_matrices.cpp" -o "$OUT/obj/ref_matrices.o" &
pids="$pids $!"
# AndersonMix<T>::update, TESTING build, one instantiation per storage type
# over the block type of shim_anderson/Solution.h
# The include guards of the reference's orbital headers are predefined: the
# TESTING build instantiates AndersonMix only for the shim's block type and
# needs none of their (ScaLAPACK / HDF5) dependencies.
AINC="-DMGMOL_EXTENDEDGRIDORBITALS_H -DLOCALGRIDORBITALS_H -I$HERE/shim_anderson $INC"
$CXX $FLAGS -DTESTING -DSolution=SolutionF $AINC -c "$SRC/AndersonMix.cc" -o "$OUT/obj/AndersonMix_f.o" &
pids="$pids $!"
$CXX $FLAGS -DTESTING -DSolution=SolutionD $AINC -c "$SRC/AndersonMix.cc" -o "$OUT/obj/AndersonMix_d.o" &
pids="$pids $!"
$CXX $FLAGS $AINC -c "$HERE/ref_anderson.cpp" -o "$OUT/obj/ref_anderson.o" &
pids="$pids $!"
$CXX $FLAGS -c "$HERE/shim/blas_shim.cpp" -o "$OUT/obj/blas_shim.o" &
pids="$pids $!"
for p in $pids; do wait $p; done
$CXX $FLAGS -shared -o "$OUT/libmgref.so" $OBJS "$OUT/obj/ref_driver.o" "$OUT/obj/ref_pack.o" "$OUT/obj/ref_matrices.o" "$OUT/obj/blas_shim.o" \
    "$OUT/obj/AndersonMix_f.o" "$OUT/obj/AndersonMix_d.o" "$OUT/obj/ref_anderson.o"
echo "build_ref: $OUT/libmgref.so"
