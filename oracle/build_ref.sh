#!/bin/sh
# Builds oracle/_ref/ref_driver: ugcore's own algebra classes compiled from
# the reference sources where they lie (nothing is copied into this repo),
# driven by ref_driver.cpp and the oracle's restated hierarchy/assembly.
# Needs the reference tree (UG4_REFERENCE, else /root/reference); prints a
# note and exits 0 without building when it is absent (e.g. on a machine
# without it).  "build_ref.sh --where" only prints the tree's location (empty
# when absent): the one place tests and the build entry learn where it is.
set -e
REF=${UG4_REFERENCE:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ "$1" = "--where" ]; then
    if [ -d "$REF/ugbase/lib_algebra" ]; then echo "$REF"; fi
    exit 0
fi
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
# ugcore's MatrixMarket reader uses boost::algorithm::split / is_any_of and
# boost::lexical_cast; these stand-ins implement the behaviour it relies on
mkdir -p "$OUT/shim/boost/algorithm"
cat > "$OUT/shim/boost/algorithm/string.hpp" <<'EOC'
#pragma once
#include <string>
namespace boost {
namespace algorithm {
enum token_compress_mode_type { token_compress_on, token_compress_off };
struct any_of_pred {
    std::string set;
    bool operator()(char c) const { return set.find(c) != std::string::npos; }
};
/* tokens between separators; with token_compress_on a run of separators is one */
template <class Seq>
Seq &split(Seq &out, const std::string &in, any_of_pred p, token_compress_mode_type m = token_compress_off)
{
    out.clear();
    std::string cur;
    size_t i = 0;
    for (;;) {
        if (i == in.size()) { out.push_back(cur); break; }
        if (p(in[i])) {
            out.push_back(cur);
            cur.clear();
            ++i;
            if (m == token_compress_on)
                while (i < in.size() && p(in[i])) ++i;
            continue;
        }
        cur += in[i++];
    }
    return out;
}
}
inline algorithm::any_of_pred is_any_of(const char *s) { return algorithm::any_of_pred{s}; }
using algorithm::split;
using algorithm::token_compress_on;
using algorithm::token_compress_off;
}
EOC
cat > "$OUT/shim/boost/lexical_cast.hpp" <<'EOC'
#pragma once
#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <string>
#include <type_traits>
#include <typeinfo>
namespace boost {
struct bad_lexical_cast : std::bad_cast {};
/* the whole string must convert (integers base 10, doubles as strtod); an
   integer out of range and a double that overflows fail, an underflowing
   double converts (as a stream extraction, which lexical_cast uses, does) */
template <class T>
T lexical_cast(const std::string &s)
{
    const char *b = s.c_str();
    char *e = nullptr;
    errno = 0;
    T v;
    bool range = false;
    if (std::is_floating_point<T>::value) {
        const double d = std::strtod(b, &e);
        range = errno == ERANGE && (d == HUGE_VAL || d == -HUGE_VAL);
        v = (T)d;
    } else if (std::is_signed<T>::value) {
        v = (T)std::strtoll(b, &e, 10);
        range = errno == ERANGE;
    } else {
        if (s.find('-') != std::string::npos) throw bad_lexical_cast();
        v = (T)std::strtoull(b, &e, 10);
        range = errno == ERANGE;
    }
    if (s.empty() || e != b + s.size() || range) throw bad_lexical_cast();
    return v;
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
# ugcore's ILU(0) and Gauss-Seidel smoothers with a given row ordering (pins
# the oracle's multicolour smoothers)
$CXX $FLAGS "$HERE/ref_smoothers.cpp" $OBJS "$OUT/obj/crc32_stub.o" -o "$OUT/ref_smoothers"
# ugcore's matrix / vector file writers and readers (MatrixIOMtx, ConnectionViewer)
IOSRCS="common/util/file_util.cpp common/util/os_dependent_impl/file_util_posix.cpp \
common/util/os_dependent_impl/os_info_linux.cpp lib_algebra/common/matrixio/matrix_io.cpp \
lib_algebra/common/matrixio/matrix_io_mtx.cpp lib_algebra/common/connection_viewer_output.cpp"
IOOBJS=""
for s in $IOSRCS; do
    o="$OUT/obj/$(echo "$s" | tr '/' '_' | sed 's/\.cpp$/.o/')"
    if [ ! -f "$o" ] || [ "$REF/ugbase/$s" -nt "$o" ]; then
        $CXX $FLAGS -c "$REF/ugbase/$s" -o "$o" &
    fi
    IOOBJS="$IOOBJS $o"
done
wait
$CXX $FLAGS "$HERE/ref_io.cpp" $IOOBJS $OBJS "$OUT/obj/crc32_stub.o" -o "$OUT/ref_io"
# ugcore's FV1 element geometry and full-upwind convection shapes
# (FV1Geometry, ConvectionShapesFullUpwind) with the reference-element,
# reference-mapping and Lagrange shape-function code they use.  Their headers
# use a few boost::mpl metafunctions; this stand-in implements that subset
# (type lists, int_, fold with max, transform_view, for_each, range_c).
SHIM2="$OUT/shim_fv1"
mkdir -p "$SHIM2/boost/mpl"
cat > "$SHIM2/boost/mpl/mpl_standin.hpp" <<'EOC'
#pragma once
#include <type_traits>
namespace boost { namespace mpl {
template <int N> struct int_ { static const int value = N; typedef int_ type; typedef int value_type; };
template <typename... T> struct list { typedef list type; };
struct _1 {}; struct _2 {}; struct _ {};
template <typename A, typename B> struct max { typedef max type; };
template <typename A, typename B> struct pair { typedef A first; typedef B second; };
template <bool C, typename A, typename B> struct if_c { typedef typename std::conditional<C, A, B>::type type; };
template <typename T, T lo, T hi> struct range_c { typedef range_c type; };
template <typename Seq, typename F> struct transform_view;
template <typename... T, typename F> struct transform_view<list<T...>, F> {
    typedef list<typename F::template apply<T>::type...> type; };
/* fold is only used as the maximum of int_ values */
template <typename Seq, typename Init, typename Op> struct fold;
template <typename Init, typename Op> struct fold<list<>, Init, Op> { typedef Init type; };
template <typename H, typename... T, typename Init> struct fold<list<H, T...>, Init, max<_1, _2> > {
    typedef typename fold<list<T...>, int_<(H::value > Init::value ? H::value : Init::value)>, max<_1, _2> >::type type; };
template <typename... T, typename F, typename Init, typename Op> struct fold<transform_view<list<T...>, F>, Init, Op> {
    typedef typename fold<typename transform_view<list<T...>, F>::type, Init, Op>::type type; };
template <typename Seq> struct empty;
template <typename... T> struct empty<list<T...> > { static const bool value = sizeof...(T) == 0; typedef empty type; };
template <typename Seq> struct front;
template <typename H, typename... T> struct front<list<H, T...> > { typedef H type; };
template <typename Seq> struct pop_front;
template <typename H, typename... T> struct pop_front<list<H, T...> > { typedef list<T...> type; };
namespace standin {
template <typename Seq> struct each;
template <> struct each<list<> > { template <typename F> static void run(F &) {} };
/* the functors ugcore passes use only the argument's type: no object of it
   is constructed (grid element classes would need lib_grid) */
template <typename H, typename... T> struct each<list<H, T...> > {
    template <typename F> static void run(F &f) {
        alignas(H) unsigned char buf[sizeof(H)];
        f(*reinterpret_cast<H *>(buf));
        each<list<T...> >::run(f); } };
template <typename T, T i, T hi, bool done = (i >= hi)> struct each_range {
    template <typename F> static void run(F &f) { int_<i> x; f(x); each_range<T, i + 1, hi>::run(f); } };
template <typename T, T i, T hi> struct each_range<T, i, hi, true> { template <typename F> static void run(F &) {} };
template <typename T, T lo, T hi> struct each<range_c<T, lo, hi> > {
    template <typename F> static void run(F &f) { each_range<T, lo, hi>::run(f); } };
}
template <typename Seq, typename F> void for_each(F f) { standin::each<typename Seq::type>::run(f); }
}}
EOC
for h in transform_view fold min_max for_each list range_c; do
    echo '#include "mpl_standin.hpp"' > "$SHIM2/boost/mpl/$h.hpp"
done
# link stand-ins for lib_grid functions that the geometry's boundary-face code
# names; with no subset handler (as the driver calls it) they are never run
cat > "$OUT/lib_grid_standin.cpp" <<'EOC'
#include <stdexcept>
#include <vector>
namespace ug {
class Grid; class Edge; class Face; class Volume; class Vertex;
#define UG_STANDIN(T, E) \
    void T(std::vector<E *> &, Grid &, Edge *, bool) { throw std::logic_error(#T); } \
    void T(std::vector<E *> &, Grid &, Face *, bool) { throw std::logic_error(#T); } \
    void T(std::vector<E *> &, Grid &, Vertex *, bool) { throw std::logic_error(#T); } \
    void T(std::vector<E *> &, Grid &, Volume *, bool) { throw std::logic_error(#T); }
UG_STANDIN(CollectEdgesSorted, Edge)
UG_STANDIN(CollectFacesSorted, Face)
UG_STANDIN(CollectVertices, Vertex)
class ISubsetHandler { public: bool elements_are_supported(unsigned int) const; Grid *grid() const; };
bool ISubsetHandler::elements_are_supported(unsigned int) const { throw std::logic_error("subset handler"); }
Grid *ISubsetHandler::grid() const { throw std::logic_error("subset handler"); }
}
EOC
GFLAGS="-std=c++17 -O3 -DNDEBUG -w -I$OUT/shim -I$SHIM2 -I$REF/ugbase"
GSRCS="lib_disc/spatial_disc/disc_util/fv1_geom.cpp lib_disc/local_finite_element/lagrange/lagrange.cpp lib_disc/local_finite_element/lagrange/lagrange_local_dof.cpp lib_disc/local_finite_element/lagrange/lagrangep1.cpp lib_disc/local_finite_element/local_dof_set.cpp lib_disc/local_finite_element/local_finite_element_id.cpp lib_disc/local_finite_element/local_finite_element_provider.cpp lib_disc/local_finite_element/mini/mini.cpp lib_disc/reference_element/reference_element.cpp lib_disc/reference_element/reference_mapping_provider.cpp common/math/misc/math_util.cpp common/math/math_vector_matrix/math_vector.cpp common/math/misc/eigenvalues.cpp common/math/misc/lineintersect_utils.cpp"
GOBJS=""
for s in $GSRCS; do
    o="$OUT/obj/g_$(echo "$s" | tr '/' '_' | sed 's/\.cpp$/.o/')"
    if [ ! -f "$o" ] || [ "$REF/ugbase/$s" -nt "$o" ]; then
        $CXX $GFLAGS -c "$REF/ugbase/$s" -o "$o" &
    fi
    GOBJS="$GOBJS $o"
done
wait
$CXX $GFLAGS -c "$OUT/lib_grid_standin.cpp" -o "$OUT/obj/lib_grid_standin.o"
$CXX $GFLAGS "$HERE/ref_fv1geom.cpp" $GOBJS "$OUT/obj/lib_grid_standin.o" $OBJS "$OUT/obj/crc32_stub.o" \
    -o "$OUT/ref_fv1geom"
# ugcore's NewtonSolver and StandardLineSearch (lib_disc headers) over the
# oracle's assembly: the Boost headers lib_disc names are replaced by the
# stand-in tests/standins/boost/ug_boost_standin.hpp (the same as the bridge
# compile test's), the string stand-ins above, and ugcore's own
# registry/class_name_provider.cpp for the class-name statics.
NSHIM="$OUT/shim_newton"
for h in boost/mpl/at.hpp boost/mpl/empty.hpp boost/mpl/fold.hpp boost/mpl/for_each.hpp boost/mpl/front.hpp \
         boost/mpl/if.hpp boost/mpl/list.hpp boost/mpl/map.hpp boost/mpl/min_max.hpp boost/mpl/pop_front.hpp \
         boost/mpl/size.hpp boost/mpl/transform_view.hpp boost/optional.hpp boost/serialization/access.hpp \
         boost/serialization/export.hpp boost/serialization/level.hpp boost/serialization/nvp.hpp \
         boost/serialization/version.hpp; do
    mkdir -p "$NSHIM/$(dirname "$h")"
    echo '#include "boost/ug_boost_standin.hpp"' > "$NSHIM/$h"
done
mkdir -p "$NSHIM/boost/algorithm" "$NSHIM/boost/graph"
# the dense LU's ordering code names these; unused, empty as for the algebra build
: > "$NSHIM/boost/graph/adjacency_list.hpp"
: > "$NSHIM/boost/graph/graph_traits.hpp"
cp "$OUT/shim/boost/algorithm/string.hpp" "$NSHIM/boost/algorithm/string.hpp"
cp "$OUT/shim/boost/lexical_cast.hpp" "$NSHIM/boost/lexical_cast.hpp"
NFLAGS="-std=c++17 -O2 -DNDEBUG -w -DUG_DIM_3 -I$NSHIM -I$HERE/../tests/standins -I$REF/ugbase -I$HERE"
if [ ! -f "$OUT/obj/n_class_name_provider.o" ]; then
    $CXX $NFLAGS -c "$REF/ugbase/registry/class_name_provider.cpp" -o "$OUT/obj/n_class_name_provider.o"
fi
stale=0
for d in "$HERE/ref_newton.cpp" "$HERE"/ug4_oracle*.c "$HERE/ug4_oracle.h"; do
    if [ ! -f "$OUT/ref_newton" ] || [ "$d" -nt "$OUT/ref_newton" ]; then stale=1; fi
done
if [ "$stale" = 1 ]; then
    $CXX $NFLAGS "$HERE/ref_newton.cpp" "$OUT/obj/n_class_name_provider.o" $OBJS "$OUT/obj/crc32_stub.o" \
        "$OUT/obj/ug4_oracle_grid.o" "$OUT/obj/ug4_oracle_fv1.o" "$OUT/obj/ug4_oracle_solve.o" \
        "$OUT/obj/ug4_oracle_api.o" -o "$OUT/ref_newton" -lm
fi
# ugcore's ThetaTimeStep over the oracle's time-dependent assembly
stale=0
for d in "$HERE/ref_theta.cpp" "$HERE"/ug4_oracle*.c "$HERE/ug4_oracle.h"; do
    if [ ! -f "$OUT/ref_theta" ] || [ "$d" -nt "$OUT/ref_theta" ]; then stale=1; fi
done
if [ "$stale" = 1 ]; then
    $CXX $NFLAGS "$HERE/ref_theta.cpp" "$OUT/obj/n_class_name_provider.o" $OBJS "$OUT/obj/crc32_stub.o" \
        "$OUT/obj/ug4_oracle_grid.o" "$OUT/obj/ug4_oracle_fv1.o" "$OUT/obj/ug4_oracle_solve.o" \
        "$OUT/obj/ug4_oracle_api.o" -o "$OUT/ref_theta" -lm
fi
echo "build_ref: built $OUT/ref_driver $OUT/ref_io $OUT/ref_fv1geom $OUT/ref_newton $OUT/ref_theta"
