#!/usr/bin/env bash
# Compile the reference solver's serial path, straight from its sources, into
# an oracle binary under oracle/_ref/ (git-ignored).  Test infrastructure only.
#   usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   (default: $REFERENCE_ROOT, else /root/reference)
# Needs only g++: MPI, HDF5 and SAMRAI are replaced by the stand-in headers in
# oracle/shims/.  -ffp-contract=off keeps every a*b+c as two rounded operations
# on both x86-64 and aarch64, so the oracle's results do not depend on the host.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${REFERENCE_ROOT:-/root/reference}}"
SRC="$REF/src"
OUT="$HERE/_ref"
if [ ! -d "$SRC/UnstructSolver" ]; then
  echo "reference sources not found under $SRC" >&2; exit 1
fi
mkdir -p "$OUT/obj"
CXX="${CXX:-g++}"
FLAGS=(-O2 -std=c++17 -ffp-contract=off -fno-fast-math -w -fPIC
       -include "$HERE/shims/compat.h" -I"$HERE/shims"
       -I"$SRC" -I"$SRC/UnstructSolver" -I"$SRC/toolBox" -I"$SRC/mathTools" -I"$SRC/UniTioga" -I"$SRC/reader")
UNITS=(UnstructSolver/UnstructIntegrator UnstructSolver/TopologyHolderStrategy
       UnstructSolver/TopologyHolderStrategyOutput UnstructSolver/Euler2D UnstructSolver/ViscousFlow2D
       UnstructSolver/FluxStrategy UnstructSolver/LimiterStrategy UnstructSolver/TimeIntegrator
       UnstructSolver/LUSGS_Integrator UnstructSolver/HLLCFluxStrategy UnstructSolver/UnstructFeeder
       UnstructSolver/commCell reader/Reader UniTioga/CellBrick mathTools/cellVolume mathTools/vector3d)
OBJS=()
pids=()
for u in "${UNITS[@]}"; do
  o="$OUT/obj/$(echo "$u" | tr '/' '_').o"
  OBJS+=("$o")
  if [ ! -f "$o" ] || [ "$SRC/$u.cpp" -nt "$o" ]; then
    "$CXX" "${FLAGS[@]}" -c "$SRC/$u.cpp" -o "$o" & pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" "${FLAGS[@]}" "$HERE/ref_driver.cpp" "${OBJS[@]}" -o "$OUT/ref_driver"
# the overset search, weights and data update (UniTioga + mathTools) in a second driver
# (MeshBlock.cpp reaches MPI types only through its HDF5 writer: the MPI stand-in is force-included)
OVS=(UniTioga/search UniTioga/utils UniTioga/ADT UniTioga/recursiveADT UniTioga/checkContainment
     UniTioga/dataUpdate UniTioga/MeshBlock UniTioga/write UniTioga/linkList UniTioga/holeMap UniTioga/bookkeeping
     mathTools/math mathTools/median mathTools/kaiser)
OOBJS=()
pids=()
for u in "${OVS[@]}"; do
  o="$OUT/obj/$(echo "$u" | tr '/' '_').o"
  OOBJS+=("$o")
  if [ ! -f "$o" ] || [ "$SRC/$u.cpp" -nt "$o" ]; then
    "$CXX" "${FLAGS[@]}" -include "$HERE/shims/mpi.h" -c "$SRC/$u.cpp" -o "$o" & pids+=($!)
  fi
done
for p in "${pids[@]}"; do wait "$p"; done
"$CXX" "${FLAGS[@]}" "$HERE/ref_overset.cpp" "${OOBJS[@]}" "$OUT/obj/mathTools_vector3d.o" \
  "$OUT/obj/mathTools_cellVolume.o" -o "$OUT/ref_overset"
echo "built $OUT/ref_driver $OUT/ref_overset"
