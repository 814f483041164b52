#!/usr/bin/env bash
# TEST INFRASTRUCTURE ONLY.
# Compiles the reference's own poisson.c, metrics.c, implicitsolver.c, rhs.c,
# bcs.c, ibm.c, compgeom.c, variables.c, init.c and (for Divergence and the
# restart routines) main.c, where they lie under the reference checkout,
# unmodified, against the single-process PETSc API shim in oracle/petsc_shim/,
# into oracle/_ref/libcvbref.so.  In the objects of rhs.c and bcs.c,
# Contra2Cart and GhostNodeVelocity are renamed cvbref_Contra2Cart /
# cvbref_GhostNodeVelocity (objcopy), so that Projection's own calls still
# reach the harness's inert versions (its parity is checked before those two
# run) while the harness can call the real ones directly.  Entry points the
# reference calls but the parity path never reaches (SNES, KSP, other CURVIB
# files) become stubs that return a PETSc error code.
#
# Every translation unit is first preprocessed into oracle/_ref/src/*.i (with
# the generated stubs beside them), and the library is compiled from those.
# The preprocessed units need neither the reference checkout nor its headers,
# so a machine without the checkout (the GPU machine, where oracle/_ref/ travels
# with the repository) rebuilds the library for its own architecture from
# them with --preprocessed.  Nothing from the reference is copied into the
# repository: oracle/_ref/ is not committed.  The source-level binding
# (curvib_old_gb300/compat/poisson_gb300.c) and the GPU driver of the binding
# test (tests/compat/glue_real.c), which include the reference's variables.h,
# are preprocessed the same way.
#
# usage: oracle/build_ref.sh REFERENCE_DIR
#        oracle/build_ref.sh --preprocessed
set -euo pipefail
if [ $# -lt 1 ]; then
  echo "usage: $0 REFERENCE_DIR | --preprocessed" >&2
  exit 2
fi
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/.." && pwd)"
OUT="$HERE/_ref"
SRC="$OUT/src"
CC="${CC:-gcc}"
UNITS="poisson metrics implicitsolver rhs bcs compgeom variables init main ibm petsc_shim ref_harness"

if [ "$1" != "--preprocessed" ]; then
  REF="$1"
  if [ ! -f "$REF/poisson.c" ]; then
    echo "build_ref: no reference sources at $REF" >&2
    exit 2
  fi
  mkdir -p "$SRC"
  rm -f "$OUT"/ref_*.o
  PP="-std=gnu99 -E -P -I$HERE/petsc_shim/include -I$REF"
  for f in poisson metrics implicitsolver rhs bcs compgeom variables init main; do
    $CC $PP "$REF/$f.c" -o "$SRC/$f.i"
  done
  # ibm.c declares point_cell_thin with 19 parameters and defines it with 13;
  # ibm_compile_fix.h names the two forms apart so the file compiles unmodified.
  $CC $PP -include ibm_compile_fix.h "$REF/ibm.c" -o "$SRC/ibm.i"
  $CC $PP "$HERE/petsc_shim/petsc_shim.c" -o "$SRC/petsc_shim.i"
  $CC $PP "$HERE/petsc_shim/ref_harness.c" -o "$SRC/ref_harness.i"
  # the binding and the binding test's GPU driver (variables.h, cvb.h)
  $CC $PP -I"$ROOT/include" -I"$ROOT/curvib_old_gb300/compat" "$ROOT/curvib_old_gb300/compat/poisson_gb300.c" \
    -o "$SRC/poisson_gb300.i"
  if [ -f "$ROOT/tests/compat/glue_real.c" ]; then
    $CC $PP -I"$ROOT/include" -I"$ROOT/curvib_old_gb300/compat" -I"$ROOT/tests/compat" \
      "$ROOT/tests/compat/glue_real.c" -o "$SRC/glue_real.i"
  fi
  # the stubs: what the linked units leave unresolved
  for u in $UNITS; do
    $CC -std=gnu99 -O2 -ffp-contract=off -fPIC -w -c "$SRC/$u.i" -o "$OUT/ref_$u.o"
  done
  objcopy --keep-global-symbol=Divergence --keep-global-symbol=Ucont_P_Binary_Output \
          --keep-global-symbol=Ucont_P_Binary_Input --keep-global-symbol=ti "$OUT/ref_main.o"
  for f in rhs bcs; do
    objcopy --redefine-sym Contra2Cart=cvbref_Contra2Cart \
            --redefine-sym GhostNodeVelocity=cvbref_GhostNodeVelocity "$OUT/ref_$f.o"
  done
  set +e
  missing=$($CC -shared -o "$OUT/libcvbref.so" "$OUT"/ref_*.o -lm -Wl,--no-undefined 2>&1 |
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
  } > "$SRC/ref_stubs.c"
  rm -f "$OUT"/ref_*.o
fi

if [ ! -f "$SRC/poisson.i" ] || [ ! -f "$SRC/ref_stubs.c" ]; then
  echo "build_ref: no preprocessed reference units in $SRC" >&2
  exit 2
fi
# -ffp-contract=off: every product and sum rounds on its own, in the C order
# of the source, on every architecture (gcc fuses a*b+c into one multiply-add
# by default where the target has one, as aarch64 does)
CFLAGS="-std=gnu99 -O2 -ffp-contract=off -fPIC -w"
objs=()
for u in $UNITS; do
  $CC $CFLAGS -c "$SRC/$u.i" -o "$OUT/ref_$u.o"
  objs+=("$OUT/ref_$u.o")
done
# main.c holds Divergence (main.c:469) and the restart routines
# Ucont_P_Binary_Output / _Input (main.c:75-467) beside main() and the globals
# the harness defines itself: every symbol of its object but those three and
# the time step ti they name files by is made local, so only they join the
# library.
objcopy --keep-global-symbol=Divergence --keep-global-symbol=Ucont_P_Binary_Output \
        --keep-global-symbol=Ucont_P_Binary_Input --keep-global-symbol=ti "$OUT/ref_main.o"
for f in rhs bcs; do
  objcopy --redefine-sym Contra2Cart=cvbref_Contra2Cart \
          --redefine-sym GhostNodeVelocity=cvbref_GhostNodeVelocity "$OUT/ref_$f.o"
done
$CC $CFLAGS -c "$SRC/ref_stubs.c" -o "$OUT/ref_stubs.o"
$CC -shared -o "$OUT/libcvbref.so" "${objs[@]}" "$OUT/ref_stubs.o" -lm -Wl,--no-undefined
echo "build_ref: $OUT/libcvbref.so ($(grep -c '^int \|^__attr' "$SRC/ref_stubs.c") stubbed entry points)"
