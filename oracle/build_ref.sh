#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.
# Compiles the reference's own poisson.c, metrics.c, implicitsolver.c, rhs.c,
# bcs.c, ibm.c, compgeom.c, variables.c, init.c and (for Divergence) main.c,
# where they lie under the reference
# checkout, unmodified, against the
# single-process PETSc API shim in oracle/petsc_shim/, into
# oracle/_ref/libcvbref.so.  In the objects of rhs.c and bcs.c, Contra2Cart and
# GhostNodeVelocity are renamed cvbref_Contra2Cart / cvbref_GhostNodeVelocity
# (objcopy), so that Projection's own calls still reach the harness's inert
# versions (its parity is checked before those two run) while the harness can
# call the real ones directly.  Nothing
# from the reference is copied into this repository; outputs go to oracle/_ref/
# only.  Entry points the reference calls but the parity path never reaches
# (SNES, KSP, other CURVIB files) become stubs that return a PETSc error code.
#
# usage: oracle/build_ref.sh REFERENCE_DIR
set -euo pipefail
if [ $# -lt 1 ]; then
  echo "usage: $0 REFERENCE_DIR" >&2
  exit 2
fi
REF="$1"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -f "$REF/poisson.c" ]; then
  echo "build_ref: no reference sources at $REF" >&2
  exit 2
fi
mkdir -p "$OUT"
CC="${CC:-gcc}"
CFLAGS="-std=gnu99 -O2 -fPIC -w -I$HERE/petsc_shim/include -I$REF"
objs=()
for f in poisson metrics implicitsolver rhs bcs compgeom variables init; do
  $CC $CFLAGS -c "$REF/$f.c" -o "$OUT/ref_$f.o"
  objs+=("$OUT/ref_$f.o")
done
# main.c holds Divergence (main.c:469) and the restart routines
# Ucont_P_Binary_Output / _Input (main.c:75-467) beside main() and the globals
# the harness defines itself: every symbol of its object but those three and
# the time step ti they name files by is made local, so only they join the
# library.
$CC $CFLAGS -c "$REF/main.c" -o "$OUT/ref_main.o"
objcopy --keep-global-symbol=Divergence --keep-global-symbol=Ucont_P_Binary_Output \
        --keep-global-symbol=Ucont_P_Binary_Input --keep-global-symbol=ti "$OUT/ref_main.o"
objs+=("$OUT/ref_main.o")
# ibm.c declares point_cell_thin with 19 parameters and defines it with 13;
# ibm_compile_fix.h names the two forms apart so the file compiles unmodified.
$CC $CFLAGS -include ibm_compile_fix.h -c "$REF/ibm.c" -o "$OUT/ref_ibm.o"
objs+=("$OUT/ref_ibm.o")
for f in rhs bcs; do
  objcopy --redefine-sym Contra2Cart=cvbref_Contra2Cart \
          --redefine-sym GhostNodeVelocity=cvbref_GhostNodeVelocity "$OUT/ref_$f.o"
done
$CC $CFLAGS -c "$HERE/petsc_shim/petsc_shim.c" -o "$OUT/petsc_shim.o"
$CC $CFLAGS -c "$HERE/petsc_shim/ref_harness.c" -o "$OUT/ref_harness.o"
objs+=("$OUT/petsc_shim.o" "$OUT/ref_harness.o")

# Find what is still unresolved and give each an inert stub.
: > "$OUT/ref_stubs.c"
set +e
missing=$($CC -shared -o "$OUT/libcvbref.so" "${objs[@]}" -lm -Wl,--no-undefined 2>&1 |
  sed -n "s/.*undefined reference to \`\([A-Za-z_][A-Za-z0-9_]*\)'.*/\1/p" | sort -u)
set -e
# A symbol the reference declares as an extern variable (main.c's globals)
# becomes zero-filled data, as main.c's defaults are; the rest become
# functions that report themselves and return a PETSc error code.
is_data() {
  grep -qE "^[[:space:]]*extern[^;(]*[^A-Za-z0-9_]$1[^A-Za-z0-9_(][^(]*;|^[[:space:]]*extern[^;(]*[^A-Za-z0-9_]$1;" \
    "$REF"/*.c "$REF"/*.h 2>/dev/null
}
{
  echo '#include <stdio.h>'
  for s in $missing; do
    if is_data "$s"; then
      echo "__attribute__((aligned(64))) char $s[4096];"
    else
      echo "int $s(void) { fprintf(stderr, \"cvbref: $s is outside the parity path\\n\"); return 1; }"
    fi
  done
} > "$OUT/ref_stubs.c"
$CC $CFLAGS -c "$OUT/ref_stubs.c" -o "$OUT/ref_stubs.o"
$CC -shared -o "$OUT/libcvbref.so" "${objs[@]}" "$OUT/ref_stubs.o" -lm -Wl,--no-undefined
echo "build_ref: $OUT/libcvbref.so ($(echo $missing | wc -w) stubbed entry points)"
