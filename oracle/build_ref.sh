#!/usr/bin/env bash
# Builds oracle/_ref/libtpref.so: the reference's own C sources for the hot
# path, compiled where they lie (never copied), plus the pinning harness
# oracle/ref_harness.c, against the single-rank MPI / no-op HDF5 stand-ins in
# oracle/stubs.  Test infrastructure only: used to pin the oracle restatement
# and to generate the golden fixtures under tests/golden.  Needs the reference
# tree (default /root/reference, override with TP_REFERENCE_DIR); exits 0
# without building when it is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${TP_REFERENCE_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src" ]; then
  echo "reference tree not found at $REF; oracle/_ref not built"
  exit 0
fi
mkdir -p "$OUT/obj"
CC="${CC:-gcc}"
# -fcommon: the reference shares globals by tentative definition across files.
# -ffp-contract=off: no FMA contraction, so x86 and aarch64 round alike.
COMMON=(-O2 -fPIC -fopenmp -fcommon -std=gnu99 -ffp-contract=off -w
        -I"$HERE/stubs" -I"$REF/include")
SRCS=(tracking emfields force_free wlcs interpolation magnetic_field
      electric_field velocity_field diagnostics quick_sort particle_info
      data_io bessel domain poincare_map)
pids=()
for s in "${SRCS[@]}"; do
  extra=(-include stdbool.h)
  case "$s" in
    # ABC coefficients become settable globals so one build covers every A,B,C.
    force_free) extra+=(-DABC_FIELD_H -DffA=refh_ffA -DffB=refh_ffB -DffC=refh_ffC
                        -include "$HERE/ref_abc_globals.h") ;;
    # The harness captures the raw diffusion sums before they are formatted.
    diagnostics) extra+=(-Dcollect_diff_coeffs=refh_orig_collect_diff_coeffs) ;;
  esac
  "$CC" "${COMMON[@]}" "${extra[@]}" -c "$REF/src/$s.c" -o "$OUT/obj/$s.o" &
  pids+=($!)
done
# The unused Bulirsch-Stoer stepper: legacy headers, no stdbool (Global.h has its own bool).
"$CC" "${COMMON[@]}" -include "$REF/include/constants.h" -include "$REF/include/particle_info.h" \
  -c "$REF/src/unused/StepperBS.c" -o "$OUT/obj/StepperBS.o" &
pids+=($!)
"$CC" "${COMMON[@]}" -include stdbool.h -c "$HERE/ref_harness.c" -o "$OUT/obj/ref_harness.o" &
pids+=($!)
for p in "${pids[@]}"; do wait "$p"; done
# -Bsymbolic: the stepper's step() must not bind to glibc's legacy regexp step()
"$CC" -shared -fopenmp -Wl,-Bsymbolic -o "$OUT/libtpref.so" "$OUT"/obj/*.o -lm
# where the sources were: the fixture generator and the drop-in link test read it
(cd "$REF" && pwd) > "$OUT/source_dir"
echo "built $OUT/libtpref.so"
