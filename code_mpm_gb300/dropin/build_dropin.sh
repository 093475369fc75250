#!/usr/bin/env bash
# Links code_MPM with the GB300 drop-in: the reference's own physics sources,
# minus the two translation units the drop-in replaces
# (PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks{,_Contact}.cpp),
# plus PhysicsEngine_runSimulation_GB300.cpp and libmpm_gb300.so, with the
# headless driver oracle/ref_driver.cpp as main().  Output: oracle/_ref/ref_gb300.
#
# The reference needs the same two mechanical edits as oracle/build_ref.sh:
# the header members the contact path uses are uncommented (force-included,
# streamed through sed, no copy written), and glm comes from oracle/glmshim.
#
# usage: code_mpm_gb300/dropin/build_dropin.sh [reference_dir]
#   reference_dir: default $MPM_REFERENCE_DIR, else a checkout named `reference` beside this repository
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
ROOT="$(cd "$HERE/../.." && pwd)"
REF="${1:-${MPM_REFERENCE_DIR:-$ROOT/../reference}}"
OUT="$ROOT/oracle/_ref"
LIBDIR="$ROOT/code_mpm_gb300/_lib"
if [ ! -f "$REF/PhysicsEngine.h" ]; then
    echo "reference sources not found under $REF" >&2
    exit 2
fi
[ -f "$LIBDIR/libmpm_gb300.so" ] || python -m code_mpm_gb300.build
mkdir -p "$OUT/obj_gb300"
CXX="${CXX:-g++}"
BASE=(-std=c++17 -O2 -ffp-contract=off -w -I "$ROOT/oracle/glmshim" -I "$REF" -I "$ROOT/oracle" -I "$ROOT/include" -I "$HERE"
      -include vector -include iostream)
patch_gridpoint() { sed -e '26s|^//||' "$REF/GridPoint.h"; }
patch_mp() { sed -e '33s|^//||' -e '51s|^//||' -e '71s|^//||' "$REF/MaterialPoint_BC.h"; }
SRCS=("$REF/PhysicsEngine.cpp"
      "$REF/ConstitutiveRelation_calculateIncrement_Elastic.cpp"
      "$REF/ConstitutiveRelation_calculateIncrement_PerfectlyPlastic.cpp"
      "$REF/ConstitutiveRelation_calculateIncrement_VonMisesHardening.cpp"
      "$REF/ConstitutiveRelation_calculateState.cpp"
      "$REF/ConstitutiveRelation_MatrixAlgebra.cpp"
      "$REF/GridPoint_Mediator.cpp"
      "$HERE/PhysicsEngine_runSimulation_GB300.cpp"
      "$ROOT/oracle/ref_driver.cpp")
objs=()
for src in "${SRCS[@]}"; do
    obj="$OUT/obj_gb300/$(basename "${src%.cpp}").o"
    "$CXX" "${BASE[@]}" -fopenmp -include <(patch_gridpoint) -include <(patch_mp) -x c++ - -c -o "$obj" < "$src"
    objs+=("$obj")
done
"$CXX" -fopenmp -o "$OUT/ref_gb300" "${objs[@]}" -L "$LIBDIR" -lmpm_gb300 -Wl,-rpath,"$LIBDIR" -lgomp
rm -rf "$OUT/obj_gb300"
echo "$OUT/ref_gb300"
