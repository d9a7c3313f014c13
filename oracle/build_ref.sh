#!/usr/bin/env bash
# Builds oracle/_ref/libfia_ref_float.so and libfia_ref_double.so from the reference's
# own hot-path sources, compiled where they lie in the reference checkout (FIA_REFERENCE_DIR;
# default: a directory named "reference" beside this repository), plus the self-written Eigen subset
# (oracle/ref_shim) and the C entry points of oracle/ref_harness.cpp.
#   float  : the reference as shipped (define_float_type.h selects float)
#   double : the same sources seen through an include directory of symbolic links to the
#            reference headers, in which define_float_type.h points at
#            oracle/ref_shim_double/define_float_type.h (the reference's double aliases)
# Test infrastructure only; outputs go to oracle/_ref/ (git-ignored).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${FIA_REFERENCE_DIR:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then echo "reference checkout not found at $REF" >&2; exit 2; fi
TUS="grid_3d grid utils physical_const cell_face cell_face_3D cell_vertex cell_vertex_3D triangle_3D
polygon_3D polygon_vector gauss_quadrature_points split_face_3D calc_backtraced_face_3D
backtrace_and_calc_all_quadrature_point_list backtrace_and_calc_all_quadrature_point_list_for_integrate_density
calc_density_in_cell_from_quadrature_point_list calc_density_in_cell_from_quadrature_point_list_for_integrate_density
calc_velocity_from_quadrature_point_list calc_velocity_from_quadrature_point_list_use_integral
calc_psi_3D calc_psi WENO6_interpolation_1d WENO6_interpolation_2d WENO6_interpolation_3d
WENO4_interpolation_3d linear_interpolation_1d linear_interpolation_2d linear_interpolation_3d sginterp3 sginterp2"
CXXFLAGS="-O2 -ffp-contract=off -fPIC -std=c++17 -w"
mkdir -p "$OUT"
for prec in float double; do
  OBJ="$OUT/obj_$prec"; mkdir -p "$OBJ"
  if [ "$prec" = float ]; then
    INC="-I$HERE/ref_shim -I$REF/include -I$REF/src"
  else
    LNK="$OUT/include_double"; rm -rf "$LNK"; mkdir -p "$LNK"
    for hdr in "$REF"/include/*.h "$REF"/include/*.hpp; do ln -s "$hdr" "$LNK/$(basename "$hdr")"; done
    rm -f "$LNK/define_float_type.h"; ln -s "$HERE/ref_shim_double/define_float_type.h" "$LNK/define_float_type.h"
    INC="-I$HERE/ref_shim -I$LNK -I$REF/src"
  fi
  pids=()
  for t in $TUS; do
    g++ $CXXFLAGS $INC -c "$REF/src/$t.cpp" -o "$OBJ/$t.o" 2>"$OBJ/$t.log" & pids+=($!)
  done
  g++ $CXXFLAGS $INC -c "$HERE/ref_harness.cpp" -o "$OBJ/ref_harness.o" 2>"$OBJ/ref_harness.log" & pids+=($!)
  gcc -O2 -fPIC -c "$HERE/ref_stubs.c" -o "$OBJ/ref_stubs.o" & pids+=($!)
  for p in "${pids[@]}"; do wait "$p" || { cat "$OBJ"/*.log >&2; exit 1; }; done
  g++ -shared -o "$OUT/libfia_ref_$prec.so" "$OBJ"/*.o -lpthread -Wl,--no-undefined
done
echo "built $OUT/libfia_ref_float.so $OUT/libfia_ref_double.so"
