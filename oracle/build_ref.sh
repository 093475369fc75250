#!/usr/bin/env bash
# Builds the reference solver's own physics sources, where they lie under the
# reference checkout, into headless binaries under oracle/_ref/.  Test
# infrastructure: the binaries produce golden states that pin the CPU
# restatement (oracle/mpm_oracle.c); nothing in the product links them.
#
# The reference ships no build files and does not compile as shipped, so two
# mechanical edits are applied as the sources stream into the compiler (no
# patched copy of any source is written to disk):
#   1. `return 0;` before every column-0 closing brace of
#      PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp: the six int
#      phase functions (:4,:23,:48,:90,:143,:175) and the large-strain pass
#      (:281) fall off their end, which GCC 13 turns into a trap (-O0) or a
#      jump into the next function (-O2).  Arithmetic is untouched.
#   2. The four members that ..._MPLocks_Contact.cpp uses but the headers
#      comment out are uncommented: GridPoint.h:26 (d3_MassGradient) and
#      MaterialPoint_BC.h:33,51,71 (b_DisplacementControl, d3_MassGradient,
#      d6_Strain_Rate).  The patched headers are force-included first, so
#      their include guards make the originals no-ops.
# glm is not vendored by the reference; oracle/glmshim provides the subset it
# uses.
#
# Variants:
#   ref_seq   OpenMP pragmas off: one thread, particles visited in index
#             order.  This is the deterministic golden reference.
#   ref_seq_ls  as ref_seq with the non-contact loop's pass 2 switched to the
#             large-strain pass the reference ships disabled: a third
#             mechanical edit, applied as the source streams in, comments out
#             the SmallStrain call (…MPLocks.cpp:604) and uncomments the
#             LargeStrain call (:605).
#   ref_omp   -fopenmp as shipped (_MAX_N_THREADS = 8, PhysicsEngine.h:27).
#   ref_ompN  -fopenmp with _MAX_N_THREADS set to N (default: nproc).
#
# usage: oracle/build_ref.sh [reference_dir] [N]
#   reference_dir: default $MPM_REFERENCE_DIR, else a checkout named `reference` beside this repository
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${MPM_REFERENCE_DIR:-$HERE/../../reference}}"
NTH="${2:-$(nproc)}"
OUT="$HERE/_ref"
if [ ! -f "$REF/PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp" ]; then
    echo "reference sources not found under $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
# MaterialPoint_BC.h relies on its includer for <vector>; force it in ahead of the patched headers.
BASE=(-std=c++17 -O2 -ffp-contract=off -w -I "$HERE/glmshim" -I "$REF" -I "$HERE" -include vector -include iostream)

patch_gridpoint() { sed -e '26s|^//||' "$REF/GridPoint.h"; }
patch_mp() { sed -e '33s|^//||' -e '51s|^//||' -e '71s|^//||' "$REF/MaterialPoint_BC.h"; }
patch_engine() { sed -e "s|^#define _MAX_N_THREADS\t8|#define _MAX_N_THREADS $1|" "$REF/PhysicsEngine.h"; }

TUS=(PhysicsEngine.cpp
     PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp
     PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks_Contact.cpp
     ConstitutiveRelation_calculateIncrement_Elastic.cpp
     ConstitutiveRelation_calculateIncrement_PerfectlyPlastic.cpp
     ConstitutiveRelation_calculateIncrement_VonMisesHardening.cpp
     ConstitutiveRelation_calculateState.cpp
     ConstitutiveRelation_MatrixAlgebra.cpp
     GridPoint_Mediator.cpp)

# build <name> <threads-or-empty> <extra flags...>
build() {
    local name="$1" nth="$2"
    shift 2
    local objdir="$OUT/obj_$name"
    mkdir -p "$objdir"
    local objs=()
    for tu in "${TUS[@]}" ref_driver.cpp; do
        local src obj="$objdir/${tu%.cpp}.o"
        if [ "$tu" = ref_driver.cpp ]; then src="$HERE/ref_driver.cpp"; else src="$REF/$tu"; fi
        local filt=(cat "$src")
        if [ "$tu" = PhysicsEngine_runSimulation_Classic_DoublePass_MPLocks.cpp ]; then
            if [ "$name" = ref_seq_ls ]; then
                filt=(sed -e 's|^}$|return 0;}|' \
                      -e '604s|^\t\t\tthis->runSimulation_G2P_P2_SmallStrain|\t\t\t//this->runSimulation_G2P_P2_SmallStrain|' \
                      -e '605s|^\t\t\t//this->runSimulation_G2P_P2_LargeStrain|\t\t\tthis->runSimulation_G2P_P2_LargeStrain|' \
                      "$src")
            else
                filt=(sed -e 's|^}$|return 0;}|' "$src")
            fi
        fi
        if [ -n "$nth" ]; then
            "${filt[@]}" | "$CXX" "${BASE[@]}" "$@" -include <(patch_gridpoint) -include <(patch_mp) \
                -include <(patch_engine "$nth") -x c++ - -c -o "$obj"
        else
            "${filt[@]}" | "$CXX" "${BASE[@]}" "$@" -include <(patch_gridpoint) -include <(patch_mp) \
                -x c++ - -c -o "$obj"
        fi
        objs+=("$obj")
    done
    "$CXX" "$@" -o "$OUT/$name" "${objs[@]}" -lgomp
    rm -rf "$objdir"
}

build ref_seq ""
build ref_seq_ls "" -DMPM_REF_LARGE_STRAIN
# the reference's 2D voxel canvas (Canvas2D_CC.cpp, as shipped) with its driver
"$CXX" "${BASE[@]}" "$REF/Canvas2D_CC.cpp" "$HERE/canvas_driver.cpp" -o "$OUT/ref_canvas"
build ref_omp "" -fopenmp
build "ref_omp$NTH" "$NTH" -fopenmp
echo "built: $(ls "$OUT")"
