#!/bin/sh
# oracle/build_ref.sh -- compile the REFERENCE's own per-tick physics sources
# (src/fields + src/sim, read in place, never copied) for the host, through the
# serial CUDA emulation in oracle/ref_emu/, into oracle/_ref/libastro_ref.so.
#
# The only source transformation is the launch syntax: `k<<<g, b>>>(...)` is
# rewritten on the fly (stdin pipe, nothing written to disk) to
# `EMU_LAUNCH((g, b), k)(...)`. The scenario loader and accept evaluation
# (src/sim/scenario.cpp, accept.cpp) are built too, and the scenario files are
# placed beside the library as test inputs. Test infrastructure only.
#
# Usage: sh oracle/build_ref.sh reference_root
#    or: AGB_REFERENCE_DIR=reference_root sh oracle/build_ref.sh
set -eu
REF="${1:-${AGB_REFERENCE_DIR:-}}"
[ -n "$REF" ] || { echo "usage: build_ref.sh reference_root (or set AGB_REFERENCE_DIR)" >&2; exit 2; }
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
[ -d "$REF/src/sim" ] || { echo "reference sources not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS="-std=c++20 -O2 -fPIC -ffp-contract=off -w -include $HERE/ref_emu/emu.h -I$HERE/ref_emu -I$REF/src -I$REF"
SRCS="src/fields/diffuse.cu src/sim/cell_store.cu src/sim/hash.cu src/sim/integrator.cu
      src/sim/thermal.cu src/sim/emission.cu src/sim/taxis.cu src/sim/flash.cu
      src/sim/predation.cu src/sim/lifecycle.cu src/sim/stats.cu src/sim/step.cu
      src/sim/snapshot.cu src/sim/scenario.cpp src/sim/accept.cpp"
OBJS=""
pids=""
for s in $SRCS; do
    o="$OUT/$(echo "$s" | tr '/' '_' | sed 's/\.cu$/.o/; s/\.cpp$/.o/')"
    OBJS="$OBJS $o"
    sed -E 's/([A-Za-z_][A-Za-z_0-9]*)<<<([^>]*)>>>/EMU_LAUNCH((\2), \1)/g' "$REF/$s" |
        $CXX $FLAGS -x c++ -c - -o "$o" &
    pids="$pids $!"
done
for p in $pids; do wait "$p"; done
$CXX $FLAGS -c "$HERE/ref_driver.cpp" -o "$OUT/ref_driver.o"
$CXX -shared -o "$OUT/libastro_ref.so" $OBJS "$OUT/ref_driver.o"
rm -f $OBJS "$OUT/ref_driver.o"
# The reference's scenario files, as inputs for the scenario tests (never committed).
mkdir -p "$OUT/scenarios"
cp "$REF"/scenarios/*.json "$OUT/scenarios/"
echo "built $OUT/libastro_ref.so"
