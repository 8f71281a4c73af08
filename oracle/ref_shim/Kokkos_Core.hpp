// ORACLE (test infrastructure only) -- a project-owned subset of the Kokkos
// API, written from Kokkos's documented behaviour, just large enough to compile
// ibis's own sources unchanged on the host.  It is not Kokkos: one host
// execution space (Serial, or OpenMP when IBIS_REF_OPENMP is defined), one
// memory space, Views of rank 1 and 2 (T*, T**, T*[N]) with explicit strides.
//
// Semantics kept from Kokkos because ibis relies on them:
//   * Views are reference-counted shallow handles; copies alias.  Elements
//     are value-initialised (zero) on allocation.  operator() of a const View
//     returns a mutable reference.
//   * create_mirror_view of a host View is the View itself.
//   * subview(v, ALL, j) / (i, ALL) / pair ranges give LayoutStride Views.
//   * the default layout of the host space is LayoutRight.
//   * inside parallel_for / parallel_reduce, copies and subviews of Views are
//     untracked (no reference count), as Kokkos does in parallel dispatch.
//   * parallel_reduce with Sum / Min reducers starts from
//     reduction_identity<T>::sum() / ::min() (user-specialisable) and joins
//     partial results with += / min.  The OpenMP space partitions the range
//     statically and joins the per-thread partials in thread order, so a
//     given thread count gives the same bits run to run; Serial sums in index
//     order.
#ifndef IBIS_REF_SHIM_KOKKOS_CORE_HPP
#define IBIS_REF_SHIM_KOKKOS_CORE_HPP

#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <limits>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>
#ifdef IBIS_REF_OPENMP
#include <omp.h>
#endif

#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_DEFAULTED_FUNCTION

namespace Kokkos {

struct LayoutRight {};
struct LayoutLeft {};
struct LayoutStride {};

struct HostSpace;
#ifdef IBIS_REF_OPENMP
struct OpenMP {
    using memory_space = HostSpace;
    using array_layout = LayoutRight;
    using execution_space = OpenMP;
    static int concurrency() { return omp_get_max_threads(); }
};
using DefaultExecutionSpace = OpenMP;
#else
struct Serial {
    using memory_space = HostSpace;
    using array_layout = LayoutRight;
    using execution_space = Serial;
    static int concurrency() { return 1; }
};
using DefaultExecutionSpace = Serial;
#endif
using DefaultHostExecutionSpace = DefaultExecutionSpace;
struct HostSpace {
    using memory_space = HostSpace;
    using execution_space = DefaultHostExecutionSpace;
};

inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}
inline bool is_initialized() { return true; }
inline void fence() {}
inline void fence(const std::string&) {}

// ---------------------------------------------------------------- math
using std::ceil;
using std::copysign;
using std::cos;
using std::cosh;
using std::exp;
using std::floor;
using std::isinf;
using std::isnan;
using std::log;
using std::pow;
using std::sin;
using std::sqrt;
using std::tanh;
inline double abs(double x) { return std::fabs(x); }
inline float abs(float x) { return std::fabs(x); }
inline int abs(int x) { return std::abs(x); }
inline long abs(long x) { return std::labs(x); }
inline long long abs(long long x) { return std::llabs(x); }
inline double fabs(double x) { return std::fabs(x); }
// the selection rules of Kokkos::min / Kokkos::max (those of std::min / std::max)
template <class T>
constexpr const T& min(const T& a, const T& b) { return (b < a) ? b : a; }
template <class T>
constexpr const T& max(const T& a, const T& b) { return (a < b) ? b : a; }

template <class A, class B>
using pair = std::pair<A, B>;
template <class A, class B>
inline std::pair<A, B> make_pair(A a, B b) { return std::pair<A, B>(a, b); }

struct ALL_t {};
constexpr ALL_t ALL{};

// ---------------------------------------------------------------- View
namespace impl {
// Inside a parallel dispatch, View copies and subviews are not reference
// counted (Kokkos turns allocation tracking off there as well): they are
// temporaries of one iteration, and the Views they come from are held by the
// dispatched functor.
inline bool& untracked() {
    static thread_local bool u = false;
    return u;
}
struct UntrackedScope {
    bool old;
    UntrackedScope() : old(untracked()) { untracked() = true; }
    ~UntrackedScope() { untracked() = old; }
};
template <class D>
struct data_traits;
template <class T>
struct data_traits<T*> {
    using value_type = T;
    static constexpr int rank = 1;
    static constexpr size_t static_n1 = 0;
};
template <class T>
struct data_traits<T**> {
    using value_type = T;
    static constexpr int rank = 2;
    static constexpr size_t static_n1 = 0;
};
template <class T, size_t N>
struct data_traits<T* [N]> {
    using value_type = T;
    static constexpr int rank = 2;
    static constexpr size_t static_n1 = N;
};

template <class T>
struct is_layout : std::false_type {};
template <>
struct is_layout<LayoutRight> : std::true_type {};
template <>
struct is_layout<LayoutLeft> : std::true_type {};
template <>
struct is_layout<LayoutStride> : std::true_type {};

template <class... P>
struct layout_of {
    using type = LayoutRight;
};
template <class P0, class... P>
struct layout_of<P0, P...> {
    using type = std::conditional_t<is_layout<P0>::value, P0, typename layout_of<P...>::type>;
};

template <class D, class T>
struct rebind;
template <class U, class T>
struct rebind<U*, T> {
    using type = T*;
};
template <class U, class T>
struct rebind<U**, T> {
    using type = T**;
};
template <class U, size_t N, class T>
struct rebind<U* [N], T> {
    using type = T* [N];
};
}  // namespace impl

template <class DataType, class... Props>
class View {
    using traits = impl::data_traits<DataType>;

public:
    using data_type = DataType;
    using value_type = typename traits::value_type;
    using non_const_value_type = std::remove_const_t<value_type>;
    using const_value_type = const non_const_value_type;
    using reference_type = value_type&;
    using pointer_type = value_type*;
    using array_layout = typename impl::layout_of<Props...>::type;
    using memory_space = HostSpace;
    using execution_space = DefaultHostExecutionSpace;
    using size_type = size_t;
    using non_const_data_type = typename impl::rebind<DataType, non_const_value_type>::type;
    using const_data_type = typename impl::rebind<DataType, const_value_type>::type;
    using host_mirror_type = View<non_const_data_type, array_layout, HostSpace>;
    using HostMirror = host_mirror_type;
    using non_const_type = View<non_const_data_type, array_layout, HostSpace>;
    using const_type = View<const_data_type, array_layout, HostSpace>;
    static constexpr int rank = traits::rank;
    static constexpr unsigned rank_dynamic = traits::static_n1 ? 1 : traits::rank;

    View() = default;
    View(const View& o) : alloc_(impl::untracked() ? nullptr : o.alloc_), ptr_(o.ptr_), label_() {
        ext_[0] = o.ext_[0]; ext_[1] = o.ext_[1];
        str_[0] = o.str_[0]; str_[1] = o.str_[1];
        if (!impl::untracked()) label_ = o.label_;
    }
    View& operator=(const View& o) {
        if (this != &o) {
            alloc_ = impl::untracked() ? nullptr : o.alloc_;
            ptr_ = o.ptr_;
            ext_[0] = o.ext_[0]; ext_[1] = o.ext_[1];
            str_[0] = o.str_[0]; str_[1] = o.str_[1];
            if (!impl::untracked()) label_ = o.label_;
        }
        return *this;
    }

    explicit View(const std::string& label, size_t n0 = 0, size_t n1 = 0) : label_(label) {
        allocate(n0, traits::static_n1 ? traits::static_n1 : (rank == 2 ? n1 : 1));
    }
    View(const char* label, size_t n0 = 0, size_t n1 = 0) : View(std::string(label), n0, n1) {}

    // unmanaged View of caller memory
    View(pointer_type p, size_t n0, size_t n1 = 0) : ptr_(p) {
        ext_[0] = n0;
        ext_[1] = traits::static_n1 ? traits::static_n1 : (rank == 2 ? n1 : 1);
        default_strides();
    }

    // any View of the same rank and a compatible element type (const added,
    // any layout: the strides travel with the handle)
    template <class D2, class... P2,
              class = std::enable_if_t<impl::data_traits<D2>::rank == traits::rank &&
                                       std::is_convertible_v<typename impl::data_traits<D2>::value_type*,
                                                             value_type*>>>
    View(const View<D2, P2...>& o)
        : alloc_(impl::untracked() ? nullptr : o.impl_alloc()), ptr_(o.data()),
          label_(impl::untracked() ? std::string() : o.label()) {
        ext_[0] = o.extent(0);
        ext_[1] = rank == 2 ? o.extent(1) : 1;
        str_[0] = o.stride(0);
        str_[1] = rank == 2 ? o.stride(1) : 1;
    }

    // a strided View (what subview builds)
    View(const std::shared_ptr<void>& alloc, pointer_type p, const size_t ext[2], const size_t str[2],
         const std::string& label)
        : alloc_(impl::untracked() ? nullptr : alloc), ptr_(p), label_(impl::untracked() ? std::string() : label) {
        ext_[0] = ext[0]; ext_[1] = ext[1];
        str_[0] = str[0]; str_[1] = str[1];
    }

    value_type& operator()(size_t i) const { return ptr_[i * str_[0]]; }
    value_type& operator()(size_t i, size_t j) const { return ptr_[i * str_[0] + j * str_[1]]; }
    value_type& operator[](size_t i) const { return ptr_[i * str_[0]]; }

    size_t extent(size_t r) const { return r < 2 ? (r == 0 ? ext_[0] : (rank == 2 ? ext_[1] : 1)) : 1; }
    int extent_int(size_t r) const { return (int)extent(r); }
    size_t size() const { return rank == 2 ? ext_[0] * ext_[1] : ext_[0]; }
    size_t span() const { return size(); }
    size_t stride(size_t r) const { return r == 0 ? str_[0] : str_[1]; }
    size_t stride_0() const { return str_[0]; }
    size_t stride_1() const { return str_[1]; }
    pointer_type data() const { return ptr_; }
    const std::string& label() const { return label_; }
    bool is_allocated() const { return ptr_ != nullptr; }
    long use_count() const { return alloc_.use_count(); }
    bool span_is_contiguous() const {
        return rank == 1 ? str_[0] == 1 : ((str_[1] == 1 && str_[0] == ext_[1]) || (str_[0] == 1 && str_[1] == ext_[0]));
    }
    const std::shared_ptr<void>& impl_alloc() const { return alloc_; }

private:
    void default_strides() {
        if (rank == 1) {
            str_[0] = 1; str_[1] = 1;
        } else if (std::is_same_v<array_layout, LayoutLeft>) {
            str_[0] = 1; str_[1] = ext_[0];
        } else {
            str_[0] = ext_[1]; str_[1] = 1;
        }
    }
    void allocate(size_t n0, size_t n1) {
        ext_[0] = n0;
        ext_[1] = n1;
        default_strides();
        // value-initialised, as Kokkos does, with 16 zeroed elements of slack past
        // the end (ibis's CubicSpline writes one element past an array and reads
        // two, which a padded Kokkos host allocation absorbs)
        const size_t n = std::max<size_t>(n0 * n1, 1) + 16;
        auto* mem = new non_const_value_type[n]();
        alloc_ = std::shared_ptr<void>(mem, [](void* q) { delete[] static_cast<non_const_value_type*>(q); });
        ptr_ = mem;
    }

    std::shared_ptr<void> alloc_;
    pointer_type ptr_ = nullptr;
    size_t ext_[2] = {0, 1};
    size_t str_[2] = {1, 1};
    std::string label_;
};

template <class D, class... P>
auto create_mirror_view(const View<D, P...>& v) {
    return typename View<D, P...>::host_mirror_type(v);
}
template <class Space, class D, class... P>
auto create_mirror_view(const Space&, const View<D, P...>& v) {
    return typename View<D, P...>::host_mirror_type(v);
}
template <class D, class... P>
auto create_mirror(const View<D, P...>& v) {
    using M = typename View<D, P...>::host_mirror_type;
    M m(v.label(), v.extent(0), View<D, P...>::rank == 2 ? v.extent(1) : 0);
    for (size_t i = 0; i < v.extent(0); i++)
        for (size_t j = 0; j < (View<D, P...>::rank == 2 ? v.extent(1) : 1); j++) {
            if constexpr (View<D, P...>::rank == 2) m(i, j) = v(i, j);
            else m(i) = v(i);
        }
    return m;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...>& dst, const View<D2, P2...>& src) {
    static_assert(View<D1, P1...>::rank == View<D2, P2...>::rank, "deep_copy: ranks differ");
    if ((const void*)dst.data() == (const void*)src.data() && dst.stride(0) == src.stride(0) &&
        dst.stride(1) == src.stride(1))
        return;
    if constexpr (View<D1, P1...>::rank == 1) {
        for (size_t i = 0; i < dst.extent(0); i++) dst(i) = src(i);
    } else {
        for (size_t i = 0; i < dst.extent(0); i++)
            for (size_t j = 0; j < dst.extent(1); j++) dst(i, j) = src(i, j);
    }
}
template <class D1, class... P1, class S, class = std::enable_if_t<!std::is_base_of_v<View<D1, P1...>, S>>>
void deep_copy(const View<D1, P1...>& dst, const S& value) {
    if constexpr (View<D1, P1...>::rank == 1) {
        for (size_t i = 0; i < dst.extent(0); i++) dst(i) = value;
    } else {
        for (size_t i = 0; i < dst.extent(0); i++)
            for (size_t j = 0; j < dst.extent(1); j++) dst(i, j) = value;
    }
}
template <class E, class D1, class... P1, class Src>
void deep_copy(const E&, const View<D1, P1...>& dst, const Src& src) {
    deep_copy(dst, src);
}

// ---------------------------------------------------------------- subview
namespace impl {
template <class V>
using strided1 = View<typename V::value_type*, LayoutStride, HostSpace>;
template <class V>
using strided2 = View<typename V::value_type**, LayoutStride, HostSpace>;
template <class I>
constexpr bool is_index = std::is_integral_v<I>;
}  // namespace impl

template <class D, class... P, class I, class = std::enable_if_t<impl::is_index<I>>>
auto subview(const View<D, P...>& v, ALL_t, I j) {
    const size_t ext[2] = {v.extent(0), 1}, str[2] = {v.stride(0), 1};
    return impl::strided1<View<D, P...>>(v.impl_alloc(), v.data() + (size_t)j * v.stride(1), ext, str, v.label());
}
template <class D, class... P, class I, class = std::enable_if_t<impl::is_index<I>>>
auto subview(const View<D, P...>& v, I i, ALL_t) {
    const size_t ext[2] = {v.extent(1), 1}, str[2] = {v.stride(1), 1};
    return impl::strided1<View<D, P...>>(v.impl_alloc(), v.data() + (size_t)i * v.stride(0), ext, str, v.label());
}
template <class D, class... P, class A, class B>
auto subview(const View<D, P...>& v, std::pair<A, B> r) {
    static_assert(View<D, P...>::rank == 1, "subview(v, range) needs a rank-1 View");
    const size_t ext[2] = {(size_t)r.second - (size_t)r.first, 1}, str[2] = {v.stride(0), 1};
    return impl::strided1<View<D, P...>>(v.impl_alloc(), v.data() + (size_t)r.first * v.stride(0), ext, str,
                                         v.label());
}
template <class D, class... P, class A, class B>
auto subview(const View<D, P...>& v, std::pair<A, B> r, ALL_t) {
    const size_t ext[2] = {(size_t)r.second - (size_t)r.first, v.extent(1)}, str[2] = {v.stride(0), v.stride(1)};
    return impl::strided2<View<D, P...>>(v.impl_alloc(), v.data() + (size_t)r.first * v.stride(0), ext, str,
                                         v.label());
}
template <class D, class... P, class A, class B>
auto subview(const View<D, P...>& v, ALL_t, std::pair<A, B> c) {
    const size_t ext[2] = {v.extent(0), (size_t)c.second - (size_t)c.first}, str[2] = {v.stride(0), v.stride(1)};
    return impl::strided2<View<D, P...>>(v.impl_alloc(), v.data() + (size_t)c.first * v.stride(1), ext, str,
                                         v.label());
}
template <class D, class... P, class A, class B, class C, class E>
auto subview(const View<D, P...>& v, std::pair<A, B> r, std::pair<C, E> c) {
    const size_t ext[2] = {(size_t)r.second - (size_t)r.first, (size_t)c.second - (size_t)c.first},
                 str[2] = {v.stride(0), v.stride(1)};
    return impl::strided2<View<D, P...>>(
        v.impl_alloc(), v.data() + (size_t)r.first * v.stride(0) + (size_t)c.first * v.stride(1), ext, str, v.label());
}
template <class D, class... P, class I, class J,
          class = std::enable_if_t<impl::is_index<I> && impl::is_index<J>>>
auto& subview(const View<D, P...>& v, I i, J j) {
    return v((size_t)i, (size_t)j);
}

// ---------------------------------------------------------------- dispatch
template <class E = DefaultExecutionSpace>
struct RangePolicy {
    size_t begin_ = 0, end_ = 0;
    RangePolicy(size_t b, size_t e) : begin_(b), end_(e) {}
    RangePolicy(const E&, size_t b, size_t e) : begin_(b), end_(e) {}
    size_t begin() const { return begin_; }
    size_t end() const { return end_; }
};

namespace impl {
struct Range {
    size_t b, e;
};
inline Range range_of(size_t n) { return {0, n}; }
inline Range range_of(int n) { return {0, (size_t)n}; }
inline Range range_of(long n) { return {0, (size_t)n}; }
inline Range range_of(unsigned n) { return {0, (size_t)n}; }
inline Range range_of(long long n) { return {0, (size_t)n}; }
template <class E>
Range range_of(const RangePolicy<E>& p) { return {p.begin(), p.end()}; }

template <class F>
void run_for(Range r, const F& f) {
#ifdef IBIS_REF_OPENMP
    const long long b = (long long)r.b, e = (long long)r.e;
#pragma omp parallel
    {
        UntrackedScope scope;
#pragma omp for schedule(static)
        for (long long i = b; i < e; i++) f((size_t)i);
    }
#else
    UntrackedScope scope;
    for (size_t i = r.b; i < r.e; i++) f(i);
#endif
}
}  // namespace impl

template <class Policy, class F>
void parallel_for(const std::string&, const Policy& p, const F& f) {
    impl::run_for(impl::range_of(p), f);
}
template <class Policy, class F, class = std::enable_if_t<!std::is_convertible_v<Policy, std::string>>>
void parallel_for(const Policy& p, const F& f) {
    impl::run_for(impl::range_of(p), f);
}

template <class T>
struct reduction_identity {
    static T sum() { return T(0); }
    static T min() {
        if constexpr (std::is_arithmetic_v<T>) return std::numeric_limits<T>::max();
        else return T(std::numeric_limits<double>::max());
    }
    static T max() {
        if constexpr (std::is_arithmetic_v<T>) return std::numeric_limits<T>::lowest();
        else return T(std::numeric_limits<double>::lowest());
    }
};

template <class T>
struct Sum {
    using value_type = T;
    T& ref;
    explicit Sum(T& r) : ref(r) {}
    static T init() { return reduction_identity<T>::sum(); }
    static void join(T& a, const T& b) { a += b; }
};
template <class T>
struct Min {
    using value_type = T;
    T& ref;
    explicit Min(T& r) : ref(r) {}
    static T init() { return reduction_identity<T>::min(); }
    static void join(T& a, const T& b) {
        if (b < a) a = b;
    }
};
template <class T>
struct Max {
    using value_type = T;
    T& ref;
    explicit Max(T& r) : ref(r) {}
    static T init() { return reduction_identity<T>::max(); }
    static void join(T& a, const T& b) {
        if (a < b) a = b;
    }
};

namespace impl {
template <class Red, class F>
void run_reduce(Range r, const F& f, Red red) {
    using T = typename Red::value_type;
#ifdef IBIS_REF_OPENMP
    const int nt = omp_get_max_threads();
    std::vector<T> part(nt, Red::init());
#pragma omp parallel num_threads(nt)
    {
        UntrackedScope scope;
        const int t = omp_get_thread_num(), n = omp_get_num_threads();
        const size_t len = r.e - r.b, chunk = (len + n - 1) / n;
        const size_t b = r.b + std::min(len, chunk * t), e = r.b + std::min(len, chunk * (t + 1));
        T acc = Red::init();
        for (size_t i = b; i < e; i++) f(i, acc);
        part[t] = acc;
    }
    T out = Red::init();
    for (int t = 0; t < nt; t++) Red::join(out, part[t]);
    red.ref = out;
#else
    T acc = Red::init();
    {
        UntrackedScope scope;
        for (size_t i = r.b; i < r.e; i++) f(i, acc);
    }
    red.ref = acc;
#endif
}
template <class T>
struct is_reducer : std::false_type {};
template <class T>
struct is_reducer<Sum<T>> : std::true_type {};
template <class T>
struct is_reducer<Min<T>> : std::true_type {};
template <class T>
struct is_reducer<Max<T>> : std::true_type {};
}  // namespace impl

template <class Policy, class F, class R>
void parallel_reduce(const std::string&, const Policy& p, const F& f, R&& result) {
    using RR = std::remove_cv_t<std::remove_reference_t<R>>;
    if constexpr (impl::is_reducer<RR>::value) impl::run_reduce(impl::range_of(p), f, result);
    else impl::run_reduce(impl::range_of(p), f, Sum<RR>(result));
}
template <class Policy, class F, class R, class = std::enable_if_t<!std::is_convertible_v<Policy, std::string>>>
void parallel_reduce(const Policy& p, const F& f, R&& result) {
    parallel_reduce(std::string(), p, f, std::forward<R>(result));
}

}  // namespace Kokkos

#endif
