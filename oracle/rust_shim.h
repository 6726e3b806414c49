/*
 * rust_shim.h -- the Rust std and cgmath 0.18.0 semantics that the C++
 * translation of cantucci's Rust source (oracle/rust_build.py) runs on.
 *
 * TEST INFRASTRUCTURE ONLY: part of the recipe that builds
 * oracle/_ref/librust_ref.so, the reference's own mesher and estimator
 * translated mechanically from its source text.  Nothing in the product
 * includes it.
 *
 * The translator turns every Rust method call `a.m(b)` into `m_m(a, b)`,
 * every associated function `T::f(..)` into `T__f(..)`, indexing into
 * rs_index, ranges into rs_range, and keeps all arithmetic as written.  This
 * header supplies those names for the types the reference takes from
 * outside its own tree:
 *   - f32 methods of Rust std.  ln/acos/sin/cos/atan2 call glibc's logf,
 *     acosf, sinf, cosf, atan2f, as Rust std does on Linux; sqrt is the
 *     SSE sqrtss instruction that llvm.sqrt.f32 lowers to; powi is LLVM's
 *     ExpandPowI (SelectionDAGBuilder: square-and-multiply over the exponent's
 *     bits, lowest bit first), which is also the order of compiler-rt's
 *     __powisf2, so constant and run-time exponents agree.
 *   - cgmath 0.18.0 (Cargo.lock), not vendored in the reference: Point3 and
 *     Vector3 operators act componentwise in x, y, z order (its
 *     impl_operator! macros), dot = (x*x + y*y) + z*z (mul_element_wise then
 *     sum, a left fold), magnitude = sqrt(dot(v, v)), normalize =
 *     v * (1 / magnitude).
 *   - Vec, arrays, slices, tuples, Option and the iterator adapters the
 *     mesher uses (iter, cloned, map, filter, fold), evaluated eagerly in
 *     element order; the closures they take are pure, so eager and lazy
 *     evaluation give the same values.
 *   - assert! throws rsref::Panic naming the function it sits in.
 *
 * x86-64 only: the reference's Vec3 is an SSE register and its magnitude an
 * SSE4.1 dot product (_mm_dp_ps), which the translation calls as written.
 */
#ifndef CANTUCCI_RUST_SHIM_H
#define CANTUCCI_RUST_SHIM_H

#if !defined(__x86_64__)
#error "the reference's Rust source is x86-64 only (std::arch::x86_64, SSE4.1)"
#endif

#include <smmintrin.h>

#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <optional>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

namespace rsref {

/* ---- panics ---------------------------------------------------------- */
struct Panic {
    const char* where;
};
inline void rs_assert(bool ok, const char* where) {
    if (!ok) throw Panic{where};
}

/* ---- f32 / integer methods of Rust std ---------------------------------- */
inline float m_ln(float x) { return logf(x); }
inline float m_sqrt(float x) { return _mm_cvtss_f32(_mm_sqrt_ss(_mm_set_ss(x))); }
inline float m_acos(float x) { return acosf(x); }
inline float m_sin(float x) { return sinf(x); }
inline float m_cos(float x) { return cosf(x); }
inline float f32__atan2(float y, float x) { return atan2f(y, x); }
inline float f32__from_bits(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
inline bool m_is_sign_positive(float x) { return !std::signbit(x); }

/* llvm.powi.f32: ExpandPowI keeps a running square of x and multiplies it
 * into the result for each set bit of |n|, lowest bit first; the first
 * factor is taken as is (1.0 * x is never formed); n < 0 takes 1/result. */
inline float m_powi(float x, int32_t n) {
    uint32_t v = n < 0 ? 0u - static_cast<uint32_t>(n) : static_cast<uint32_t>(n);
    bool have = false;
    float res = 1.0f, sq = x;
    while (v) {
        if (v & 1u) {
            res = have ? res * sq : sq;
            have = true;
        }
        sq = sq * sq;
        v >>= 1;
    }
    return n < 0 ? 1.0f / res : res;
}

/* `x.into()`: the target type comes from the use site. */
template <class T>
struct Into {
    T v;
    template <class U>
    operator U() const { return static_cast<U>(v); }
};
template <class T>
Into<T> m_into(T x) { return Into<T>{x}; }

template <class T>
T m_pow(T base, uint32_t e) {  // integer pow (wrapping, as release builds)
    T r = 1;
    for (uint32_t i = 0; i < e; ++i) r = static_cast<T>(r * base);
    return r;
}
template <class T>
bool m_is_power_of_two(T x) { return x != 0 && (x & (x - 1)) == 0; }

constexpr uint32_t u32__MAX = 0xFFFFFFFFu;

template <class T>
T assoc__zero() { return T(0); }
template <class T>
T assoc__one() { return T(1); }

/* ---- cgmath 0.18.0 ----------------------------------------------------- */
template <class S>
struct Vector3 {
    S x, y, z;
};
template <class S>
struct Point3 {
    S x, y, z;
};

template <class A, class B, class C>
Vector3<A> Vector3__new(A x, B y, C z) { return Vector3<A>{x, static_cast<A>(y), static_cast<A>(z)}; }
template <class A, class B, class C>
Point3<A> Point3__new(A x, B y, C z) { return Point3<A>{x, static_cast<A>(y), static_cast<A>(z)}; }
inline Vector3<float> Vector3__zero() { return {0.0f, 0.0f, 0.0f}; }
inline Vector3<float> Vector3__unit_x() { return {1.0f, 0.0f, 0.0f}; }
inline Vector3<float> Vector3__unit_y() { return {0.0f, 1.0f, 0.0f}; }
inline Vector3<float> Vector3__unit_z() { return {0.0f, 0.0f, 1.0f}; }
inline Point3<float> Point3__origin() { return {0.0f, 0.0f, 0.0f}; }

template <class S>
Vector3<S> operator+(Vector3<S> a, Vector3<S> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S>
Vector3<S> operator-(Vector3<S> a, Vector3<S> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S>
Vector3<S> operator-(Vector3<S> a) { return {-a.x, -a.y, -a.z}; }
template <class S>
Vector3<S> operator*(Vector3<S> a, S s) { return {a.x * s, a.y * s, a.z * s}; }
template <class S>
Vector3<S> operator*(S s, Vector3<S> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class S>
Vector3<S> operator/(Vector3<S> a, S s) { return {a.x / s, a.y / s, a.z / s}; }
template <class S>
Point3<S> operator+(Point3<S> a, Vector3<S> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class S>
Point3<S> operator-(Point3<S> a, Vector3<S> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S>
Vector3<S> operator-(Point3<S> a, Point3<S> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class S>
Point3<S> operator*(Point3<S> a, S s) { return {a.x * s, a.y * s, a.z * s}; }
template <class S>
Point3<S> operator/(Point3<S> a, S s) { return {a.x / s, a.y / s, a.z / s}; }

template <class S>
Vector3<S> m_mul_element_wise(Vector3<S> a, Vector3<S> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class S>
Vector3<S> m_to_vec(Point3<S> p) { return {p.x, p.y, p.z}; }
template <class S>
S m_magnitude2(Vector3<S> v) { return (v.x * v.x + v.y * v.y) + v.z * v.z; }
template <class S>
S m_magnitude(Vector3<S> v) { return m_sqrt(m_magnitude2(v)); }
template <class S>
Vector3<S> m_normalize(Vector3<S> v) { return v * (S(1) / m_magnitude(v)); }

/* util::ToArr: (*self).into() -- cgmath's From<Vector3<S>> for [S; 3]. */
template <class S>
std::array<S, 3> m_to_arr(Vector3<S> v) { return {v.x, v.y, v.z}; }
template <class S>
std::array<S, 3> m_to_arr(Point3<S> p) { return {p.x, p.y, p.z}; }

/* ---- std::ops::Range ------------------------------------------------------ */
template <class T>
struct Range {
    T start, end;
};
template <class A, class B>
Range<std::common_type_t<A, B>> rs_range(A a, B b) {
    using T = std::common_type_t<A, B>;
    return Range<T>{static_cast<T>(a), static_cast<T>(b)};
}
template <class T>
Range<T> rs_range(T a, T b) { return Range<T>{a, b}; }
struct RangeFrom {
    size_t start;
};
inline RangeFrom rs_range_from(size_t a) { return RangeFrom{a}; }

template <class T>
struct IntRange {
    T a, b;
    struct It {
        T v;
        T operator*() const { return v; }
        It& operator++() { ++v; return *this; }
        bool operator!=(const It& o) const { return v != o.v; }
    };
    It begin() const { return It{a}; }
    It end() const { return It{a < b ? b : a}; }
};

/* ---- arrays, slices, Vec ----------------------------------------------------- */
template <class T>
struct Slice {
    const T* p;
    size_t n;
    const T* begin() const { return p; }
    const T* end() const { return p + n; }
};

template <class... A>
auto rs_arr(A... a) {
    return std::array<std::common_type_t<std::decay_t<A>...>, sizeof...(A)>{a...};
}
template <class T, class... A>
std::array<T, sizeof...(A)> rs_arr_as(A... a) { return std::array<T, sizeof...(A)>{T(a)...}; }

template <class T, size_t N, class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
const T& rs_index(const std::array<T, N>& a, I i) { return a.at(static_cast<size_t>(i)); }
template <class T, class I, std::enable_if_t<std::is_integral_v<I>, int> = 0>
const T& rs_index(const std::vector<T>& a, I i) { return a.at(static_cast<size_t>(i)); }
template <class T, size_t N>
Slice<T> rs_index(const std::array<T, N>& a, RangeFrom r) { return Slice<T>{a.data() + r.start, N - r.start}; }

template <class T, class X>
void m_push(std::vector<T>& v, X&& x) { v.push_back(std::forward<X>(x)); }
template <class T>
size_t m_len(const std::vector<T>& v) { return v.size(); }
template <class T, class U, size_t N>
void m_extend_from_slice(std::vector<T>& v, const std::array<U, N>& a) { v.insert(v.end(), a.begin(), a.end()); }
template <class V>
V Vec__new() { return V(); }
template <class V>
V Vec__with_capacity(size_t n) {
    V v;
    v.reserve(n);
    return v;
}

/* ---- iterators (eager) ------------------------------------------------------ */
template <class T>
struct Seq {
    std::vector<T> v;
};
template <class T, size_t N>
Seq<T> m_iter(const std::array<T, N>& a) { return Seq<T>{std::vector<T>(a.begin(), a.end())}; }
template <class T>
Seq<T> m_cloned(Seq<T> s) { return s; }
template <class T, class F>
auto m_map(Seq<T> s, F f) {
    using U = std::decay_t<decltype(f(s.v[0]))>;
    Seq<U> out;
    for (auto& x : s.v) out.v.push_back(f(x));
    return out;
}
template <class T, class F>
Seq<T> m_filter(Seq<T> s, F f) {
    Seq<T> out;
    for (auto& x : s.v)
        if (f(x)) out.v.push_back(x);
    return out;
}
template <class T, class A, class F>
A m_fold(Seq<T> s, A acc, F f) {
    for (auto& x : s.v) acc = f(acc, x);
    return acc;
}

/* ---- Option ------------------------------------------------------------------ */
template <class T>
std::optional<std::decay_t<T>> Some(T&& x) { return std::optional<std::decay_t<T>>(std::forward<T>(x)); }

/* `for x in it`: integer ranges, slices and arrays iterate directly; any other
 * value is an Iterator whose next() the translation defines. */
template <class It>
struct NextIter {
    It it;
    using Item = typename decltype(m_next(std::declval<It&>()))::value_type;
    struct Cur {
        NextIter* self;
        std::optional<Item> cur;
        const Item& operator*() const { return *cur; }
        Cur& operator++() { cur = m_next(self->it); return *this; }
        bool operator!=(const Cur&) const { return cur.has_value(); }
    };
    Cur begin() { return Cur{this, m_next(it)}; }
    Cur end() { return Cur{this, std::nullopt}; }
};
template <class T, std::enable_if_t<std::is_integral_v<T>, int> = 0>
IntRange<T> rs_iterable(Range<T> r) { return IntRange<T>{r.start, r.end}; }
template <class T>
Slice<T> rs_iterable(Slice<T> s) { return s; }
template <class T, size_t N>
const std::array<T, N>& rs_iterable(const std::array<T, N>& a) { return a; }
template <class It, std::enable_if_t<!std::is_integral_v<It>, int> = 0>
NextIter<It> rs_iterable(It it) { return NextIter<It>{it}; }

/* ---- std::time (timings are not compared) -------------------------------------- */
struct Duration {
    double s;
};
struct Instant {
    std::chrono::steady_clock::time_point t;
};
inline Instant Instant__now() { return Instant{std::chrono::steady_clock::now()}; }
inline Duration operator-(Instant a, Instant b) { return Duration{std::chrono::duration<double>(a.t - b.t).count()}; }

/* ---- observation (test hook) ------------------------------------------------------
 * The recipe asks the translation to pass the value GridTable::fill_with
 * returns through rs_observe before returning it; the last f32 and u32 tables
 * of a thread (naive_surface_nets' `dists` and `points`) are kept for the
 * tests.  It reads the table and changes nothing. */
inline thread_local std::vector<float> observed_f32;
inline thread_local std::vector<uint32_t> observed_u32;
template <class G>
void rs_observe(const G& g) {
    if constexpr (std::is_same_v<std::decay_t<decltype(g.data)>, std::vector<float>>) observed_f32 = g.data;
    if constexpr (std::is_same_v<std::decay_t<decltype(g.data)>, std::vector<uint32_t>>) observed_u32 = g.data;
}

}  // namespace rsref

#endif
