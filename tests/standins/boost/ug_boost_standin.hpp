// Stand-in for the parts of Boost that ugcore's headers name (mpl type lists
// and metafunctions, optional, serialization declarations), enough to
// compile the headers; nothing here is Boost code.
#pragma once
#include <cstddef>
#include <type_traits>
#include <utility>
namespace boost {
namespace mpl {
template <int N> struct int_ { static const int value = N; typedef int_ type; typedef int value_type; };
template <bool B> struct bool_ { static const bool value = B; typedef bool_ type; };
typedef bool_<true> true_;
typedef bool_<false> false_;
template <typename... T> struct list { typedef list type; };
template <typename T> struct list1 { typedef list1 type; };
struct _1 {}; struct _2 {}; struct _ {};
template <typename A, typename B> struct max { typedef max type; };
template <typename A, typename B> struct pair { typedef A first; typedef B second; };
template <bool C, typename A, typename B> struct if_c { typedef typename std::conditional<C, A, B>::type type; };
template <typename C, typename A, typename B> struct if_ { typedef typename std::conditional<C::value, A, B>::type type; };
template <typename T, T lo, T hi> struct range_c { typedef range_c type; };
template <typename Seq, typename F> struct transform_view;
template <typename... T, typename F> struct transform_view<list<T...>, F> {
    typedef list<typename F::template apply<T>::type...> type; };
template <typename Seq, typename Init, typename Op> struct fold;
template <typename Init, typename Op> struct fold<list<>, Init, Op> { typedef Init type; };
template <typename H, typename... T, typename Init> struct fold<list<H, T...>, Init, max<_1, _2> > {
    typedef typename fold<list<T...>, int_<(H::value > Init::value ? H::value : Init::value)>, max<_1, _2> >::type type; };
template <typename... T, typename F, typename Init, typename Op> struct fold<transform_view<list<T...>, F>, Init, Op> {
    typedef typename fold<typename transform_view<list<T...>, F>::type, Init, Op>::type type; };
template <typename Seq> struct empty;
template <typename... T> struct empty<list<T...> > { enum { value = sizeof...(T) == 0 }; };
template <typename T> struct empty<list1<T> > { enum { value = false }; };
template <typename Seq> struct size;
template <typename... T> struct size<list<T...> > { typedef int_<(int)sizeof...(T)> type; static const int value = sizeof...(T); };
template <typename Seq> struct front;
template <typename H, typename... T> struct front<list<H, T...> > { typedef H type; };
template <typename T> struct front<list1<T> > { typedef T type; };
template <typename Seq> struct pop_front;
template <typename H, typename T> struct pop_front<list<H, T> > { typedef list1<T> type; };
template <typename H, typename T2, typename T3, typename... T> struct pop_front<list<H, T2, T3, T...> > { typedef list<T2, T3, T...> type; };
template <typename H> struct pop_front<list<H> > { typedef list<> type; };
template <typename T> struct pop_front<list1<T> > { typedef list<> type; };
template <typename Seq, typename N> struct at;
template <typename H, typename... T> struct at<list<H, T...>, int_<0> > { typedef H type; };
template <typename H, typename... T, int N> struct at<list<H, T...>, int_<N> > { typedef typename at<list<T...>, int_<N - 1> >::type type; };
namespace standin {
template <typename Seq> struct each;
template <> struct each<list<> > { template <typename F> static void run(F &) {} };
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
}  // namespace mpl

struct none_t {};
const none_t none = none_t();
template <class T> class optional {
public:
    optional() : m_has(false), m_v() {}
    optional(none_t) : m_has(false), m_v() {}
    optional(const T &v) : m_has(true), m_v(v) {}
    explicit operator bool() const { return m_has; }
    bool operator!() const { return !m_has; }
    const T &operator*() const { return m_v; }
    T &operator*() { return m_v; }
    const T *operator->() const { return &m_v; }
    T *operator->() { return &m_v; }
    const T &get() const { return m_v; }
    T &get() { return m_v; }
    bool is_initialized() const { return m_has; }
private:
    bool m_has;
    T m_v;
};

namespace serialization {
class access {};
template <class T> struct nvp { const char *name; T *value; };
template <class T> nvp<T> make_nvp(const char *n, T &v) { return nvp<T>{n, &v}; }
template <class D, class B> inline void void_cast_register(const D *, const B *) {}
template <class B, class D> B &base_object(D &d) { return static_cast<B &>(d); }
template <class T> struct version { static const int value = 0; };
}
}  // namespace boost
#define BOOST_CLASS_EXPORT_KEY(x)
#define BOOST_CLASS_EXPORT_KEY2(x, y)
#define BOOST_CLASS_EXPORT_IMPLEMENT(x)
#define BOOST_CLASS_EXPORT(x)
#define BOOST_CLASS_VERSION(x, y)
#define BOOST_SERIALIZATION_SPLIT_MEMBER()
#define BOOST_SERIALIZATION_ASSUME_ABSTRACT(x)
