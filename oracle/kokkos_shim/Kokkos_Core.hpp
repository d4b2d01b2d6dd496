/*
 * Kokkos_Core.hpp -- a minimal, project-written stand-in for the subset of the public Kokkos
 * API that the Armon-Kokkos sources use, so that those sources compile unchanged on a host
 * without Kokkos.  TEST INFRASTRUCTURE ONLY: it exists to build the reference (under
 * oracle/_ref/) as a checker for the oracle.  It is written from the documented Kokkos
 * interface (View, RangePolicy, parallel_for/reduce, reducers, math functions), not from the
 * Kokkos sources.
 *
 * Semantics that matter for bit-level parity:
 *  - parallel_for / parallel_reduce over a RangePolicy run [begin, end) with an OpenMP static
 *    schedule (the reference's flat-range default build);
 *  - reducer partials start at the reducer's identity (Min: DBL_MAX) and are joined in thread
 *    order, so a run is deterministic for a fixed thread count;
 *  - min / max follow std::min / std::max ((b < a) ? b : a, (a < b) ? b : a);
 *  - pow / sqrt / abs / copysign call the C library (pow(x, 2.0) folds to x*x).
 */
#ifndef ARMON_KOKKOS_SHIM_CORE_HPP
#define ARMON_KOKKOS_SHIM_CORE_HPP

#include <algorithm>
#include <array>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KOKKOS_VERSION 30700
#define KOKKOS_LAMBDA [=]
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION

namespace Kokkos {

/* ---- execution / memory spaces ---- */
struct HostSpace { using size_type = std::size_t; };
struct Serial {
    using size_type = std::size_t;
    using memory_space = HostSpace;
    static int concurrency() { return 1; }
};
using DefaultExecutionSpace = Serial;
using DefaultHostExecutionSpace = Serial;

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}
inline void fence(const std::string&) {}
inline void print_configuration(std::ostream& os, bool = false)
{
    os << "Kokkos API shim (host, OpenMP static schedule)\n";
}
struct ScopeGuard {
    ScopeGuard() {}
    ScopeGuard(int&, char**) {}
};

/* ---- pairs ---- */
template <class T1, class T2>
struct pair {
    T1 first;
    T2 second;
    pair() = default;
    pair(const T1& a, const T2& b) : first(a), second(b) {}
    std::pair<T1, T2> to_std_pair() const { return {first, second}; }
};
template <class T1, class T2>
inline pair<T1, T2> make_pair(const T1& a, const T2& b) { return pair<T1, T2>(a, b); }

/* ---- math ---- */
template <class T> inline const T& min(const T& a, const T& b) { return (b < a) ? b : a; }
template <class T> inline const T& max(const T& a, const T& b) { return (a < b) ? b : a; }
inline double abs(double x) { return std::fabs(x); }
inline float abs(float x) { return std::fabs(x); }
inline double sqrt(double x) { return std::sqrt(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline double pow(double x, double y) { return std::pow(x, y); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline double copysign(double x, double y) { return std::copysign(x, y); }
inline float copysign(float x, float y) { return std::copysign(x, y); }
inline double ceil(double x) { return std::ceil(x); }
inline double hypot(double x, double y) { return std::hypot(x, y); }
inline float hypot(float x, float y) { return std::hypot(x, y); }
namespace numbers {
constexpr double sqrt2 = 1.41421356237309504880;
constexpr double pi = 3.14159265358979323846;
}

/* ---- views (1-D, labelled, 64-byte aligned, reference-counted handle) ---- */
struct WithoutInitializing_t {};
constexpr WithoutInitializing_t WithoutInitializing{};
struct ViewAllocProp { std::string label; };
inline ViewAllocProp view_alloc(const std::string& label, WithoutInitializing_t) { return {label}; }

template <class DataType, class... Props> class View;

template <class T, class... Props>
class View<T*, Props...> {
public:
    using value_type = T;
    using pointer_type = T*;
    using reference_type = T&;
    using HostMirror = View<T*, Props...>;
    using memory_space = HostSpace;
    using size_type = std::size_t;

    View() = default;
    View(const ViewAllocProp& prop, std::size_t n) { allocate(prop.label, n); }
    View(const std::string& label, std::size_t n) { allocate(label, n); }
    View(T* ptr, std::size_t n) : m_ptr(ptr), m_size(n) {}

    T& operator[](std::size_t i) const { return m_ptr[i]; }
    T& operator()(std::size_t i) const { return m_ptr[i]; }
    T* data() const { return m_ptr; }
    std::size_t size() const { return m_size; }
    std::size_t extent(int) const { return m_size; }
    std::string label() const { return m_label ? *m_label : std::string(); }

private:
    void allocate(const std::string& label, std::size_t n)
    {
        std::size_t bytes = ((n * sizeof(T) + 63) / 64) * 64;
        if (bytes == 0) bytes = 64;
        T* p = static_cast<T*>(std::aligned_alloc(64, bytes));
        if (!p) throw std::bad_alloc();
        m_owner = std::shared_ptr<T>(p, [](T* q) { std::free(q); });
        m_ptr = p;
        m_size = n;
        m_label = std::make_shared<std::string>(label);
    }

    std::shared_ptr<T> m_owner;
    T* m_ptr = nullptr;
    std::size_t m_size = 0;
    std::shared_ptr<std::string> m_label;
};

/* rank-0 unmanaged view on a value (used for reducer results) */
template <class T, class... Props>
class View {
public:
    using value_type = T;
    using memory_space = HostSpace;
    View() = default;
    View(T* ptr) : m_ptr(ptr) {}
    T* data() const { return m_ptr; }
    T& operator()() const { return *m_ptr; }
private:
    T* m_ptr = nullptr;
};

template <class V>
inline typename V::HostMirror create_mirror_view(const V& v) { return v; }

template <class T, class... P1, class... P2>
inline void deep_copy(const View<T*, P1...>& dst, const View<T*, P2...>& src)
{
    if (dst.data() != src.data())
        std::memcpy(dst.data(), src.data(), std::min(dst.size(), src.size()) * sizeof(T));
}

/* ---- policies ---- */
template <class T> struct IndexType { using type = T; };

namespace Impl {
template <class... P> struct policy_index { using type = std::size_t; };
template <class T, class... P> struct policy_index<IndexType<T>, P...> { using type = T; };
}

template <class... Props>
struct RangePolicy {
    using index_type = typename Impl::policy_index<Props...>::type;
    index_type m_begin = 0, m_end = 0;
    RangePolicy() = default;
    RangePolicy(index_type b, index_type e) : m_begin(b), m_end(e) {}
    index_type begin() const { return m_begin; }
    index_type end() const { return m_end; }
};

struct AUTO_t {};
constexpr AUTO_t AUTO{};

template <class... Props>
struct TeamPolicy {
    struct member_type {
        int league_rank() const { return 0; }
        int team_rank() const { return 0; }
        int team_size() const { return 1; }
    };
    TeamPolicy() = default;
    TeamPolicy(long, AUTO_t) {}
    TeamPolicy(long, AUTO_t, long) {}
};

template <unsigned N> struct Rank {};

template <class... Props>
struct MDRangePolicy {
    MDRangePolicy() = default;
    MDRangePolicy(std::initializer_list<long>, std::initializer_list<long>, std::initializer_list<long>) {}
};

template <class... A> inline int TeamThreadRange(A&&...) { return 0; }
template <class... A> inline int ThreadVectorRange(A&&...) { return 0; }

/* ---- reducers ---- */
template <class T> struct reduction_identity;
template <> struct reduction_identity<double> {
    static constexpr double sum() { return 0.0; }
    static constexpr double prod() { return 1.0; }
    static constexpr double max() { return -DBL_MAX; }
    static constexpr double min() { return DBL_MAX; }
    static constexpr double bor() { return 0.0; }
    static constexpr double band() { return 0.0; }
    static constexpr double lor() { return 0.0; }
    static constexpr double land() { return 0.0; }
};
template <> struct reduction_identity<float> {
    static constexpr float sum() { return 0.0f; }
    static constexpr float prod() { return 1.0f; }
    static constexpr float max() { return -FLT_MAX; }
    static constexpr float min() { return FLT_MAX; }
    static constexpr float bor() { return 0.0f; }
    static constexpr float band() { return 0.0f; }
    static constexpr float lor() { return 0.0f; }
    static constexpr float land() { return 0.0f; }
};

template <class T, class Space = HostSpace>
struct Min {
    using value_type = T;
    using result_view_type = View<T, Space>;
    T* m_ref;
    Min(T& r) : m_ref(&r) {}
    void join(T& dest, const T& src) const { if (src < dest) dest = src; }
    void init(T& v) const { v = reduction_identity<T>::min(); }
    T& reference() const { return *m_ref; }
};

template <class T, class Space = HostSpace>
struct Sum {
    using value_type = T;
    using result_view_type = View<T, Space>;
    T* m_ref;
    Sum(T& r) : m_ref(&r) {}
    void join(T& dest, const T& src) const { dest += src; }
    void init(T& v) const { v = reduction_identity<T>::sum(); }
    T& reference() const { return *m_ref; }
};

/* ---- dispatch ---- */
template <class... P, class F>
inline void parallel_for(const RangePolicy<P...>& policy, const F& f)
{
    using I = typename RangePolicy<P...>::index_type;
    const long long b = (long long)policy.begin(), e = (long long)policy.end();
#pragma omp parallel for schedule(static)
    for (long long k = b; k < e; k++) f((I)k);
}

template <class... P, class F, class R>
inline void parallel_reduce(const RangePolicy<P...>& policy, const F& f, const R& reducer)
{
    using I = typename RangePolicy<P...>::index_type;
    using V = typename R::value_type;
    const long long b = (long long)policy.begin(), e = (long long)policy.end();
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<V> partial((std::size_t)nt);
    for (auto& v : partial) reducer.init(v);
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        V local;
        reducer.init(local);
#pragma omp for schedule(static)
        for (long long k = b; k < e; k++) f((I)k, local);
        partial[(std::size_t)t] = local;
    }
    V result;
    reducer.init(result);
    for (auto& v : partial) reducer.join(result, v);
    reducer.reference() = result;
}

namespace Experimental {
template <class T> struct native_simd { static constexpr unsigned size() { return 1; } };
}

} // namespace Kokkos

#endif
