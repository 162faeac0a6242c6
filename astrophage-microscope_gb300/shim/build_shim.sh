#!/bin/sh
# build_shim.sh -- build libastro_sim_gb.so, the reference simulator's World API
# (src/sim/world.cuh, src/sim/cell_store.cuh) implemented over the engine's C ABI,
# and optionally link programs written against that API (the reference's own
# tests/physics/*.cu, say) to it instead of to src/sim + src/fields.
#
# The shim is compiled against the reference's headers, read in place: it needs
# a reference checkout, and the engine (libagb.so, built by build.py) beside it.
#
# Usage: sh build_shim.sh REFERENCE_ROOT [OUT_DIR [PROGRAM ...]]
#    or: AGB_REFERENCE_DIR=REFERENCE_ROOT sh build_shim.sh
# Writes OUT_DIR/libastro_sim_gb.so (OUT_DIR defaults to this folder) and one
# executable per PROGRAM, named after its first source, in OUT_DIR. A PROGRAM
# is one source file or several joined by colons (main.cpp:more.cpp), e.g. the
# reference's headless runner with its scenario loader and acceptance code:
#   REF/tools/headless.cpp:REF/src/sim/scenario.cpp:REF/src/sim/accept.cpp
set -eu
REF="${1:-${AGB_REFERENCE_DIR:-}}"
[ -n "$REF" ] || { echo "usage: build_shim.sh REFERENCE_ROOT [OUT_DIR [PROGRAM.cu ...]]" >&2; exit 2; }
[ -f "$REF/src/sim/world.cuh" ] || { echo "reference headers not found at $REF" >&2; exit 2; }
HERE="$(cd "$(dirname "$0")" && pwd)"
PKG="$(dirname "$HERE")"
INC="$(dirname "$PKG")/include"
OUT="${2:-$HERE}"
[ $# -ge 2 ] && shift 2 || shift $#
[ -f "$PKG/libagb.so" ] || { echo "libagb.so not built (python build.py)" >&2; exit 2; }
mkdir -p "$OUT"
NVCC="${NVCC:-nvcc}"
ARCH="-gencode arch=compute_103a,code=sm_103a"
FLAGS="-std=c++20 -O2 --expt-relaxed-constexpr -Xcompiler -fPIC -I$INC -I$REF/src -I$REF -I$REF/tests"
$NVCC $ARCH $FLAGS -shared "$HERE/astro_sim_gb.cu" -o "$OUT/libastro_sim_gb.so" \
    -L"$PKG" -lagb -Xlinker -rpath -Xlinker "$PKG"
pids=""
for prog in "$@"; do
    srcs="$(echo "$prog" | tr ':' ' ')"
    first="${prog%%:*}"
    name="$(basename "$(basename "$first" .cu)" .cpp)"
    $NVCC $ARCH $FLAGS $srcs -o "$OUT/$name" -L"$OUT" -lastro_sim_gb -L"$PKG" -lagb \
        -Xlinker -rpath -Xlinker "$OUT" -Xlinker -rpath -Xlinker "$PKG" &
    pids="$pids $!"
done
rc=0
for p in $pids; do wait "$p" || rc=1; done
exit $rc
