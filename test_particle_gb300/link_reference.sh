#!/usr/bin/env bash
# Links the reference's own program (main.c and every module that is not on
# the tracking hot path) against libtpgpu.so instead of tracking.o,
# emfields.o, interpolation.o, force_free.o, wlcs.o, poincare_map.o and
# data_io.o (the field-file readers, HDF5 included, come from the library).
#
#   REF      reference tree (default: $TP_REFERENCE_DIR)
#   CC       the reference's compiler (mpicc on a cluster)
#   CFLAGS   extra compile flags (the HDF5 include directory)
#   LIBS     extra link flags (-lhdf5_hl -lhdf5 ...)
#   OUT      output directory (default: ./tp_dropin)
#
# The field modules (magnetic_field.c, electric_field.c, velocity_field.c)
# stay: they read the field files into the arrays the library uploads.  Their
# set-up functions and the reference's globals, defined in the executable,
# take precedence over the library's definitions of the same names (ELF
# symbol interposition), so both sides share one set of globals.
# create_fields_ctype (include/emfields.h:30) builds HDF5 compound types and
# is kept from emfields.c with every other symbol of that object made local.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${REF:-${TP_REFERENCE_DIR:-}}"
[ -d "$REF/src" ] || { echo "set REF to the reference tree" >&2; exit 2; }
CC="${CC:-cc}"
OUT="${OUT:-$PWD/tp_dropin}"
LIBDIR="$HERE/_build"
[ -f "$LIBDIR/libtpgpu.so" ] || { echo "build libtpgpu.so first" >&2; exit 2; }
mkdir -p "$OUT/obj"
FLAGS=(-O2 -fopenmp -fcommon -std=gnu99 -w -include stdbool.h -I"$REF/include" ${CFLAGS:-})
KEEP=(main test_particle domain diagnostics particle_info quick_sort bessel
      magnetic_field electric_field velocity_field)
for s in "${KEEP[@]}"; do
  "$CC" "${FLAGS[@]}" -c "$REF/src/$s.c" -o "$OUT/obj/$s.o"
done
"$CC" "${FLAGS[@]}" -c "$REF/src/emfields.c" -o "$OUT/obj/emfields_full.o"
objcopy --keep-global-symbol=create_fields_ctype "$OUT/obj/emfields_full.o" "$OUT/obj/emfields_h5.o"
rm -f "$OUT/obj/emfields_full.o"
"$CC" -fopenmp -o "$OUT/test_particle" "$OUT"/obj/*.o -L"$LIBDIR" -ltpgpu \
  -Wl,-rpath,"$LIBDIR" ${LIBS:-} -lm
echo "linked $OUT/test_particle"
