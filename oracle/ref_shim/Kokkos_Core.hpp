// Minimal host-only stand-in for the part of the Kokkos API that the AXIS
// geometry headers, the regular/rectilinear fast-path sources and the weight
// generator use (View of rank 0 to 2, RangePolicy, parallel_for/reduce,
// atomics, math wrappers, mirror/deep_copy, Device). It lets
// oracle/ref_driver.cpp, oracle/ref_fast.cpp and oracle/ref_generate.cpp
// compile the reference's code unchanged, serially, on the host.
// Test infrastructure: used only to build oracle/_ref/libaxisref.so.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#define KOKKOS_FUNCTION
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

struct Serial {};
struct HostSpace {
    using execution_space = Serial;
    using memory_space = HostSpace;
};
using DefaultHostExecutionSpace = Serial;
template <class ExecSpace, class MemSpace>
struct Device {
    using execution_space = ExecSpace;
    using memory_space = MemSpace;
};
using DefaultExecutionSpace = Serial;
struct LayoutLeft {};
struct LayoutRight {};
template <unsigned N = 0>
struct MemoryTraits {};
constexpr unsigned Unmanaged = 1;

template <class A, class B>
struct SpaceAccessibility {
    static constexpr bool accessible = true;
};

inline double sqrt(double x) { return std::sqrt(x); }
inline double atan2(double y, double x) { return std::atan2(y, x); }
inline double fabs(double x) { return std::fabs(x); }
inline double fmin(double a, double b) { return std::fmin(a, b); }
inline double fmax(double a, double b) { return std::fmax(a, b); }
inline double acos(double x) { return std::acos(x); }
inline double asin(double x) { return std::asin(x); }
inline double cos(double x) { return std::cos(x); }
inline double sin(double x) { return std::sin(x); }
inline double abs(double x) { return std::fabs(x); }
inline double floor(double x) { return std::floor(x); }
inline double round(double x) { return std::round(x); }
inline double atan(double x) { return std::atan(x); }
inline bool isnan(double x) { return std::isnan(x); }
inline bool isinf(double x) { return std::isinf(x); }
inline double nan(const char *s) { return std::nan(s); }

template <class T>
struct view_traits {  // rank 0
    using value = T;
    static constexpr int rank = 0;
    static constexpr std::size_t e1 = 1;
};
template <class U>
struct view_traits<U *> {
    using value = U;
    static constexpr int rank = 1;
    static constexpr std::size_t e1 = 1;
};
template <class U>
struct view_traits<U **> {
    using value = U;
    static constexpr int rank = 2;
    static constexpr std::size_t e1 = 0;  // run-time extent
};
template <class U, std::size_t N>
struct view_traits<U *[N]> {
    using value = U;
    static constexpr int rank = 2;
    static constexpr std::size_t e1 = N;
};

// Rank-0, rank-1 or rank-2 (column-major) host array with shared ownership.
template <class DataType, class... Props>
class View {
   public:
    using value_type = typename view_traits<DataType>::value;
    using nc_value = std::remove_const_t<value_type>;
    using memory_space = HostSpace;
    static constexpr int Rank = view_traits<DataType>::rank;

    std::shared_ptr<nc_value[]> store;
    nc_value *ptr = nullptr;
    std::size_t e0 = 0, e1 = 1;

    View() = default;
    // label only: one element for rank 0, an empty array otherwise
    explicit View(const std::string &)
        : store(new nc_value[1]()), ptr(store.get()), e0(Rank == 0 ? 1 : 0), e1(Rank > 1 ? ext1(0) : 1) {}
    View(const std::string &, std::size_t n0, std::size_t n1 = 1)
        : store(new nc_value[n0 * ext1(n1) > 0 ? n0 * ext1(n1) : 1]()), ptr(store.get()), e0(n0), e1(ext1(n1)) {}
    View(value_type *p, std::size_t n0, std::size_t n1 = 1) : ptr(const_cast<nc_value *>(p)), e0(n0), e1(Rank > 1 ? n1 : 1) {}
    template <class D2, class... P2>
    View(const View<D2, P2...> &o) : store(o.store), ptr(o.ptr), e0(o.e0), e1(o.e1) {}

    static constexpr std::size_t ext1(std::size_t n1) {
        return Rank < 2 ? 1 : (view_traits<DataType>::e1 ? view_traits<DataType>::e1 : n1);
    }
    value_type &operator()() const { return ptr[0]; }
    value_type &operator()(std::size_t i) const { return ptr[i]; }
    value_type &operator()(std::size_t i, std::size_t j) const { return ptr[i + j * e0]; }
    value_type &operator[](std::size_t i) const { return ptr[i]; }
    std::size_t extent(int d) const { return d == 0 ? e0 : (d == 1 && Rank > 1 ? e1 : 1); }
    value_type *data() const { return ptr; }
    std::size_t size() const { return e0 * e1; }
};

template <class V>
V create_mirror_view(const V &v) {
    return v;
}
template <class S, class V>
V create_mirror_view_and_copy(const S &, const V &v) {
    return v;
}
template <class A, class B>
void deep_copy(const A &dst, const B &src) {
    if constexpr (std::is_arithmetic_v<B>) {
        for (std::size_t i = 0; i < dst.size(); ++i) dst.data()[i] = src;
    } else {
        if (dst.data() != src.data())
            for (std::size_t i = 0; i < dst.size(); ++i) dst.data()[i] = src.data()[i];
    }
}

template <class ExecSpace = Serial>
struct RangePolicy {
    std::size_t b, e;
    RangePolicy(std::size_t b_, std::size_t e_) : b(b_), e(e_) {}
};

template <class T>
struct Min {
    T &ref;
    explicit Min(T &r) : ref(r) {}
    T init() const { return std::numeric_limits<T>::max(); }
};
template <class T>
struct Max {
    T &ref;
    explicit Max(T &r) : ref(r) {}
    T init() const { return std::numeric_limits<T>::lowest(); }
};

template <class E, class F>
void parallel_for(const std::string &, const RangePolicy<E> &p, F f) {
    for (std::size_t i = p.b; i < p.e; ++i) f(i);
}
template <class F>
void parallel_for(const std::string &, std::size_t n, F f) {
    for (std::size_t i = 0; i < n; ++i) f(i);
}
template <class E, class F, class R1, class R2>
void parallel_reduce(const std::string &, const RangePolicy<E> &p, F f, R1 r1, R2 r2) {
    auto a = r1.init();
    auto b = r2.init();
    for (std::size_t i = p.b; i < p.e; ++i) f(i, a, b);
    r1.ref = a;
    r2.ref = b;
}
template <class E, class F, class T>
std::enable_if_t<std::is_arithmetic_v<T>> parallel_reduce(const std::string &, const RangePolicy<E> &p, F f, T &result) {
    T s{};
    for (std::size_t i = p.b; i < p.e; ++i) f(i, s);
    result = s;
}

// Hierarchical parallelism as a host backend runs it: one thread per team,
// vector length 1, so every nested range runs in order.
constexpr int AUTO = -1;
struct TeamMember {
    int rank;
    int league_rank() const { return rank; }
    int team_rank() const { return 0; }
    int team_size() const { return 1; }
};
template <class ExecSpace = Serial>
struct TeamPolicy {
    using member_type = TeamMember;
    int league;
    TeamPolicy(int league_size, int) : league(league_size) {}
};
template <class I>
struct NestedRange {
    I b, e;
};
template <class I>
NestedRange<I> ThreadVectorRange(const TeamMember &, I n) {
    return {I(0), n};
}
template <class I>
NestedRange<I> TeamThreadRange(const TeamMember &, I n) {
    return {I(0), n};
}
template <class I, class J>
NestedRange<std::common_type_t<I, J>> TeamVectorRange(const TeamMember &, I b, J e) {
    return {static_cast<std::common_type_t<I, J>>(b), static_cast<std::common_type_t<I, J>>(e)};
}
template <class E, class F>
void parallel_for(const std::string &, const TeamPolicy<E> &p, F f) {
    for (int t = 0; t < p.league; ++t) f(TeamMember{t});
}
template <class I, class F>
void parallel_for(const NestedRange<I> &r, F f) {
    for (I i = r.b; i < r.e; ++i) f(i);
}
template <class I, class F, class T>
void parallel_reduce(const NestedRange<I> &r, F f, T &result) {
    T s{};
    for (I i = r.b; i < r.e; ++i) f(i, s);
    result = s;
}
struct PerTeamTag {};
inline PerTeamTag PerTeam(const TeamMember &) { return {}; }
template <class F>
void single(PerTeamTag, F f) {
    f();
}

template <class T, class U>
void atomic_add(T *p, U v) {
    *p += v;
}
template <class T, class U>
T atomic_fetch_add(T *p, U v) {
    const T old = *p;
    *p += v;
    return old;
}

inline void fence() {}
inline void fence(const std::string &) {}
inline bool is_initialized() { return true; }
inline void initialize() {}

}  // namespace Kokkos
