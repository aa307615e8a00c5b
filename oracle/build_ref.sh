#!/bin/bash
# Oracle recipe: compile the reference SWIFT hydro hot path (Minimal SPH,
# Wendland C2, 3D, ideal gas gamma=5/3) straight from the reference source
# tree, without autotools or HDF5, and link the oracle's own driver
# (oracle/ref_harness.c) against it.
#
# This is test infrastructure.  Nothing from the reference is copied into the
# repository: sources are compiled where they lie; every output goes under
# oracle/_ref/ (git-ignored).  Only the build configuration header, the HDF5
# typedef stub and the abort() stubs below are written here, from scratch.
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   MODE=parity (default): -O2 -fno-fast-math -ffp-contract=off  (bit-exact pins)
#   MODE=stock           : the reference's own optimisation flags (timed baseline)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
# The reference tree: the argument, else $SWIFT_REFERENCE_ROOT, else a
# `reference` directory beside this repository.
REF="${1:-${SWIFT_REFERENCE_ROOT:-$HERE/../../reference}}"
MODE="${MODE:-parity}"
OUT="$HERE/_ref/$MODE"
if [ ! -d "$REF/src" ]; then
  echo "build_ref: reference tree not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT/include" "$OUT/objs" "$OUT/bin"

ARCH="$(uname -m)"
if [ "$MODE" = "stock" ]; then
  # The reference's configure picks these (m4/ax_cc_maxopt.m4) for gcc.
  if [ "$ARCH" = "x86_64" ]; then NATIVE="-march=native"; else NATIVE="-mcpu=native"; fi
  OPT="-O3 -ffast-math -funroll-loops -fomit-frame-pointer $NATIVE"
else
  OPT="-O2 -fno-fast-math -ffp-contract=off"
fi

# --- build configuration (the configure defaults for
#     --with-hydro=minimal --with-kernel=wendland-C2, 3D, ideal gas, 5/3) ---
{
  echo "/* generated by oracle/build_ref.sh */"
  for d in MINIMAL_SPH WENDLAND_C2_KERNEL EOS_IDEAL_GAS MULTI_SOFTENING_GRAVITY \
           NONE_MHD RIEMANN_SOLVER_NONE CHEMISTRY_NONE COOLING_NONE TRACERS_NONE \
           EXTRA_IO_NONE STARS_NONE FEEDBACK_NONE BLACK_HOLES_NONE SINK_NONE \
           FORCING_NONE EXTERNAL_POTENTIAL_NONE ENTROPY_FLOOR_NONE \
           PRESSURE_FLOOR_NONE STAR_FORMATION_NONE RT_RIEMANN_SOLVER_NONE RT_NONE \
           HAVE_PTHREAD_BARRIERS HAVE_POSIX_FALLOCATE HAVE_SINCOS HAVE_SINCOSF \
           HAVE_EXP10 HAVE_EXP10F HAVE_FE_ENABLE_EXCEPT HAVE_SETAFFINITY \
           HAVE_STDBOOL_H; do
    echo "#define $d 1"
  done
  echo "#define HYDRO_DIMENSION_3D 3"
  echo "#define HYDRO_GAMMA_5_3 (5./3.)"
  echo "#define HYDRO_GHOST_NTASK 1"
  echo "#define HYDRO_COOLING_NTASK 1"
  echo "#define STARS_GHOST_NTASK 1"
  echo "#define STARS_SELF_NTASK 1"
  echo "#define SELF_GRAVITY_MULTIPOLE_ORDER 4"
  echo "#define SWIFT_RANDOM_SEED_XOR 0"
  echo "#ifndef _GNU_SOURCE"
  echo "#define _GNU_SOURCE 1"
  echo "#endif"
  echo "#define PACKAGE_VERSION \"oracle\""
  # memswap.h uses x86 intrinsics only when this is defined.
  if [ "$ARCH" = "x86_64" ]; then echo "#define HAVE_IMMINTRIN_H 1"; fi
  echo "#include <stdbool.h>"
} > "$OUT/include/config.h"

cat > "$OUT/include/hdf5.h" <<'EOF'
/* generated by oracle/build_ref.sh: HDF5 is absent; typedefs only. */
#ifndef ORACLE_HDF5_STUB_H
#define ORACLE_HDF5_STUB_H
typedef long long hid_t;
typedef int herr_t;
typedef unsigned long long hsize_t;
typedef long long hssize_t;
typedef int htri_t;
#endif
EOF
echo '#define PACKAGE_VERSION_STR "oracle"' > "$OUT/include/version_string.h"

CF="-std=gnu11 $OPT -fcommon -ffunction-sections -fdata-sections -w -I$OUT/include -I$REF/src -I$REF/src/lightcone"

# --- compile every reference source in parallel; the handful of I/O units
#     that need real HDF5 fail and are simply left out of the archive ---
ls "$REF"/src/*.c "$REF"/src/lightcone/*.c | \
  xargs -P "$(nproc)" -I{} sh -c 'b=$(basename {} .c); gcc '"$CF"' -c {} -o '"$OUT"'/objs/$b.o 2>/dev/null || true'
rm -f "$OUT/libswiftref.a"
ar rcs "$OUT/libswiftref.a" "$OUT"/objs/*.o

gcc -std=gnu11 -O2 -c "$HERE/ref_stubs.c" -o "$OUT/ref_stubs.o"

LINK="-include float.h -include swift.h -include mhd.h"
gcc $CF $LINK "$HERE/ref_harness.c" "$OUT/libswiftref.a" "$OUT/ref_stubs.o" \
    -lm -lpthread -Wl,--gc-sections -o "$OUT/bin/ref_harness"
gcc $CF $LINK "$HERE/ref_integrate.c" "$OUT/libswiftref.a" "$OUT/ref_stubs.o" \
    -lm -lpthread -Wl,--gc-sections -o "$OUT/bin/ref_integrate"

# The reference's own hydro known-answer tests, built from its tests/ tree.
for t in test27cells test125cells testActivePair testPeriodicBC testSymmetry testKernel; do
  if [ -f "$REF/tests/$t.c" ]; then
    gcc $CF $LINK "$REF/tests/$t.c" "$OUT/libswiftref.a" "$OUT/ref_stubs.o" \
        -lm -lpthread -Wl,--gc-sections -o "$OUT/bin/$t" 2>/dev/null || \
        echo "build_ref: could not build $t" >&2
  fi
done
echo "build_ref: $MODE build in $OUT"
