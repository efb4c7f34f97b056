#!/bin/sh
# Builds oracle/_ref/ref_driver: ugcore's own algebra classes compiled from
# the reference sources where they lie (nothing is copied into this repo),
# driven by ref_driver.cpp and the oracle's restated hierarchy/assembly.
# Needs the reference tree (default /root/reference); prints a note and exits
# 0 without building when it is absent (e.g. on a machine without it).
set -e
REF=${UG4_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -d "$REF/ugbase/lib_algebra" ]; then
    echo "build_ref: reference tree not found at $REF; skipping"
    exit 0
fi
mkdir -p "$OUT/shim/lib_disc/function_spaces" "$OUT/shim/lib_disc/common" "$OUT/shim/boost/graph" "$OUT/obj"
# empty stand-ins for headers the algebra includes but does not use (the real
# ones pull in Boost / lib_disc, which are not buildable here)
: > "$OUT/shim/lib_disc/function_spaces/approximation_space.h"
: > "$OUT/shim/lib_disc/common/function_group.h"
: > "$OUT/shim/boost/graph/adjacency_list.hpp"
: > "$OUT/shim/boost/graph/graph_traits.hpp"
# ug::crc32 only hashes DebugID names; the reference one needs boost/crc.hpp.
cat > "$OUT/crc32_stub.cpp" <<'EOC'
#include <cstdint>
namespace ug {
/* bitwise CRC-32 (reflected polynomial 0xEDB88320), used only to hash debug ids */
uint32_t crc32(const char *s)
{
    uint32_t c = 0xFFFFFFFFu;
    for (; *s; ++s) {
        c ^= (unsigned char)*s;
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return ~c;
}
}
EOC
CXX=${CXX:-g++}
FLAGS="-std=c++17 -O3 -DNDEBUG -w -I$OUT/shim -I$REF/ugbase -I$HERE"
SRCS="common/log.cpp common/debug_id.cpp common/assert.cpp common/error.cpp common/progress.cpp \
common/util/string_util.cpp common/util/ostream_buffer_splitter.cpp \
lib_algebra/algebra_common/permutation_util.cpp \
lib_algebra/ordering_strategies/algorithms/native_cuthill_mckee.cpp"
OBJS=""
for s in $SRCS; do
    o="$OUT/obj/$(echo "$s" | tr '/' '_' | sed 's/\.cpp$/.o/')"
    if [ ! -f "$o" ] || [ "$REF/ugbase/$s" -nt "$o" ]; then
        $CXX $FLAGS -c "$REF/ugbase/$s" -o "$o" &
    fi
    OBJS="$OBJS $o"
done
wait
$CXX $FLAGS -c "$OUT/crc32_stub.cpp" -o "$OUT/obj/crc32_stub.o"
for c in ug4_oracle_grid.c ug4_oracle_fv1.c ug4_oracle_solve.c ug4_oracle_api.c; do
    gcc -O2 -std=c11 -ffp-contract=off -c "$HERE/$c" -o "$OUT/obj/${c%.c}.o"
done
$CXX $FLAGS "$HERE/ref_driver.cpp" $OBJS "$OUT/obj/crc32_stub.o" \
    "$OUT/obj/ug4_oracle_grid.o" "$OUT/obj/ug4_oracle_fv1.o" "$OUT/obj/ug4_oracle_solve.o" \
    "$OUT/obj/ug4_oracle_api.o" -o "$OUT/ref_driver" -lm
echo "build_ref: built $OUT/ref_driver"
