#!/usr/bin/env bash
# Builds the parity pin: the reference's own kernel sources (U_Q.cl,
# Viscous.cl, Weno.cl), compiled where they lie as host C++ through
# oracle/ref_shim.h, and its boundary routine (Flow_Initialisation.cpp)
# through oracle/bc_ref_shim.h, into oracle/_ref/libcfd_ref.so (geometry:
# oracle/_ref/libcfd_ref_geom.so).  Outputs go only to
# oracle/_ref/ (git-ignored).  Generated files: a copy of Viscous.cl whose
# four hard-coded constants (Mach, Reyl, Pr, Free_t) read globals, so the pin
# also covers other flow parameters, and a copy of Flow_Initialisation.cpp
# with its include lines pointed at the shim; and the geometry producer
# (Grid_Transformation.cpp's metric_term() and the half-point block of
# Main.cpp) through oracle/metric_ref_shim.h.  Needs the reference checkout;
# exits 0 without building when it is absent.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
# the reference checkout: CFD_REFERENCE_DIR, else "reference" beside this repository
REF_DIR="${CFD_REFERENCE_DIR:-$HERE/../../reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/Weno.cl" ]; then
    echo "build_ref: reference sources not found at $REF_DIR; skipping" >&2
    exit 0
fi
mkdir -p "$OUT"
sed -e 's/const double Mach = 1\.5;/const double Mach = ::ref_visc_mach;/' \
    -e 's/const double Reyl = 500\.0;/const double Reyl = ::ref_visc_reyl;/' \
    -e 's/const double Pr = 0\.72;/const double Pr = ::ref_visc_pr;/' \
    -e 's/const double Free_t = 273\.0;/const double Free_t = ::ref_visc_tinf;/' \
    "$REF_DIR/Viscous.cl" > "$OUT/Viscous_param.cl"
for c in ref_visc_mach ref_visc_reyl ref_visc_pr ref_visc_tinf; do
    grep -q "= ::$c;" "$OUT/Viscous_param.cl" || { echo "build_ref: substitution of $c failed" >&2; exit 1; }
done
# The boundary routine: a copy whose two include lines name the shim instead
# of functions.h (MPI + OpenCL) and the MPI header.
sed -e 's|#include "functions.h"|#include "bc_ref_shim.h"|' \
    -e 's|#include <openmpi-x86_64/mpi.h>||' \
    "$REF_DIR/Flow_Initialisation.cpp" > "$OUT/Flow_Initialisation_ref.cpp"
grep -q '#include "bc_ref_shim.h"' "$OUT/Flow_Initialisation_ref.cpp" || { echo "build_ref: include substitution failed" >&2; exit 1; }
# The geometry producer: metric_term() from a copy of Grid_Transformation.cpp
# with its includes pointed at the shim, and the half-point block of
# Main.cpp (between its "evaluating metrics at half points" comment and the
# ghost-point repetition) cut out and wrapped in a function.
sed -e 's|#include "functions.h"|#include "metric_ref_shim.h"|' \
    -e 's|#include <mpi.h>||' \
    "$REF_DIR/Grid_Transformation.cpp" > "$OUT/Grid_Transformation_ref.cpp"
grep -q '#include "metric_ref_shim.h"' "$OUT/Grid_Transformation_ref.cpp" || { echo "build_ref: include substitution failed" >&2; exit 1; }
{
    echo '#include "metric_ref_shim.h"'
    echo 'void ref_half_points_body()'
    echo '{'
    awk '/Repeating for evaluating metrics at half points for ghost points/ {on = 0}
         on {print}
         /evaluating metrics at half points\*/ && !/Repeating/ {on = 1}' "$REF_DIR/Main.cpp"
    echo '}'
} > "$OUT/half_points_ref.cpp"
grep -q 'deter\[i\].km' "$OUT/half_points_ref.cpp" || { echo "build_ref: half-point block not found" >&2; exit 1; }
g++ -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w \
    -I"$HERE" -I"$OUT" -I"$REF_DIR" \
    "$HERE/ref_kernels.cpp" "$HERE/ref_bc.cpp" "$OUT/Flow_Initialisation_ref.cpp" -o "$OUT/libcfd_ref.so"
# separate library: the geometry routines use the same global names
g++ -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w \
    -I"$HERE" -I"$OUT" \
    "$HERE/ref_metrics.cpp" "$OUT/Grid_Transformation_ref.cpp" "$OUT/half_points_ref.cpp" -o "$OUT/libcfd_ref_geom.so"
echo "build_ref: built $OUT/libcfd_ref.so and $OUT/libcfd_ref_geom.so"
