#!/bin/sh
# Build recipe for the CPU checkers (test infrastructure only):
#
#  1. oracle/_ref/liboracle.so -- the C restatement oracle/v2c_oracle.c.
#  2. oracle/_ref/v2c_ref      -- the reference's own hot-path routines,
#     compiled from its sources with oracle/ref_harness.c.
#
# For (2) the reference sources are copied from $V2C_REFERENCE/src (set
# V2C_REFERENCE to the reference checkout, the directory that holds src/)
# into oracle/_ref/src, raising only the array-size macros of headevps.c so
# larger grids and marker sets fit.  That staging directory is git-ignored;
# it exists so the same recipe can rebuild the binary on a machine without
# the reference tree.  With V2C_REFERENCE unset the staged copy is used;
# when neither is present only (1) is built.
#
# Both are compiled with -ffp-contract=off so FP64 arithmetic is evaluated
# exactly as written on every host architecture.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
REF="${V2C_REFERENCE:-}"
CC="${CC:-gcc}"
mkdir -p "$OUT"

$CC -std=gnu99 -O2 -ffp-contract=off -fPIC -shared -Wall \
    -o "$OUT/liboracle.so" "$HERE/v2c_oracle.c" -lm

FILES="headevps.c input_RSF.c calc_RSF.c gausevps.c interpolation.c \
density_ductilevisc_calc.c moveandrotatemarkers.c \
momentum_continuity_addmatrix_checkerror.c momentum_continuity_iterate.c \
temperature_iterate.c plastic.c recalc_marker_properties.c load_save.c"

if [ -n "$REF" ] && [ -d "$REF/src" ]; then
  mkdir -p "$OUT/src"
  for f in $FILES; do cp "$REF/src/$f" "$OUT/src/$f"; done
  # grid up to 1100 x 420 lines, 8.2 M markers (a 1001 x 401 window of the
  # 20-markers-per-cell configuration); the Stokes matrix arrays (MAXVAL
  # coefficients) hold the assembly of a 1001 x 401 grid.
  sed -i \
    -e 's/^#define MAXMAT .*/#define MAXMAT  8000000/' \
    -e 's/^#define MAXVAL .*/#define MAXVAL  24000000/' \
    -e 's/^#define MAXXLN .*/#define MAXXLN  1100/' \
    -e 's/^#define MAXYLN .*/#define MAXYLN  420/' \
    -e 's/^#define MAXMRK .*/#define MAXMRK  8200001/' \
    "$OUT/src/headevps.c"
fi

if [ -f "$OUT/src/headevps.c" ]; then
  MODEL=""
  case "$(uname -m)" in x86_64) MODEL="-mcmodel=medium" ;; esac
  $CC -std=gnu99 -O3 -fopenmp -fcommon -w -ffp-contract=off $MODEL \
      -I"$OUT/src" -I"$HERE/../include" -o "$OUT/v2c_ref" "$HERE/ref_harness.c" -lm
  # 2b. oracle/_ref/v2c_ref_fast -- the same build with floating-point
  #     contraction allowed, as the reference's own icc build compiles by
  #     default (compile_euler.sh): the timed CPU baseline; the build above
  #     stays the bit-exact pin.
  $CC -std=gnu99 -O3 -fopenmp -fcommon -w -ffp-contract=fast $MODEL \
      -I"$OUT/src" -I"$HERE/../include" -o "$OUT/v2c_ref_fast" "$HERE/ref_harness.c" -lm
  # 3. oracle/_ref/v2c_ref_serial -- the same sources with the OpenMP
  #    pragmas ignored (libgomp linked only for omp_get_wtime): the routines
  #    as written for one thread.  moveandrotatemarkers appends spawned
  #    markers through a reduction variable, which under OpenMP starts from
  #    0 in every thread; this build pins the restatement's serial reading.
  $CC -std=gnu99 -O3 -fopenmp-simd -fcommon -w -ffp-contract=off $MODEL \
      -I"$OUT/src" -I"$HERE/../include" -o "$OUT/v2c_ref_serial" "$HERE/ref_harness.c" \
      -lgomp -lm
else
  echo "build_ref.sh: reference sources not found; built the restatement only" >&2
fi

# 4. oracle/_ref/v2c_ref_full -- the timed build (contraction allowed, as
#    2b) with the arrays raised to the full C4 configuration: 4001 x 1001
#    grid lines, 80.1 M markers, ~24 GB of static arrays.  That is beyond the
#    default code model's reach on both architectures (x86-64: medium model;
#    AArch64: the large model, which needs a non-PIE executable).  Optional:
#    where it does not build, the reference arm times the window instead.
if [ -n "$REF" ] && [ -d "$REF/src" ]; then
  mkdir -p "$OUT/src_full"
  for f in $FILES; do cp "$REF/src/$f" "$OUT/src_full/$f"; done
  # MAXMAT: the boundary corrections of marker2nodes collect ~2 entries
  # per node in val0[] (8.0 M at C4)
  sed -i \
    -e 's/^#define MAXMAT .*/#define MAXMAT  40000000/' \
    -e 's/^#define MAXVAL .*/#define MAXVAL  24000000/' \
    -e 's/^#define MAXXLN .*/#define MAXXLN  4001/' \
    -e 's/^#define MAXYLN .*/#define MAXYLN  1001/' \
    -e 's/^#define MAXMRK .*/#define MAXMRK  80100001/' \
    "$OUT/src_full/headevps.c"
fi
if [ -f "$OUT/src_full/headevps.c" ]; then
  case "$(uname -m)" in
    x86_64) FULL="-mcmodel=medium" ;;
    aarch64) FULL="-mcmodel=large -fno-pie -no-pie" ;;
    *) FULL="" ;;
  esac
  if ! $CC -std=gnu99 -O3 -fopenmp -fcommon -w -ffp-contract=fast $FULL \
      -I"$OUT/src_full" -I"$HERE/../include" -o "$OUT/v2c_ref_full" "$HERE/ref_harness.c" -lm; then
    echo "build_ref.sh: the full-size reference build failed; the reference arm times a window" >&2
    rm -f "$OUT/v2c_ref_full"
  fi
fi
