// Host-only stand-in for the small part of the Kokkos API that qkrylov's
// sources use, so that the reference C++ sources compile unchanged into the
// oracle build (oracle/_ref).  It is test infrastructure: nothing in the
// product library includes it.
//
// Surface provided (everything the reference's src/ and include/ touch):
//   complex<T> (= std::complex<T>, layout-compatible, relied on by the
//   reinterpret_casts in src/hamiltonian/matrix_free_hamiltonian.cpp:189,199),
//   conj/abs, View<T*, props...> with shared (reference-counted) ownership and
//   zero-initialised storage, unmanaged pointer views, deep_copy (view/view,
//   view/scalar, with or without an execution-space argument),
//   create_mirror_view (aliases, as Kokkos does for host views),
//   parallel_for / parallel_reduce over RangePolicy or an integer count,
//   OpenMP / Serial / HostSpace / MemoryUnmanaged tags and initialize/finalize.
//
// Reductions: with OpenMP each thread sums a static block of the range and the
// partial sums are added in thread order, so results are deterministic for a
// fixed thread count (OMP_NUM_THREADS=1 gives the plain sequential order).
#pragma once

#include <complex>
#include <cstddef>
#include <cstring>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KOKKOS_ENABLE_OPENMP 1
#define KOKKOS_LAMBDA [=]
#define KOKKOS_INLINE_FUNCTION inline

namespace Kokkos {

template <class T> using complex = std::complex<T>;
template <class T> inline std::complex<T> conj(const std::complex<T>& z) { return std::conj(z); }
template <class T> inline T abs(const std::complex<T>& z) { return std::abs(z); }

struct HostSpace;
struct OpenMP {
    using memory_space = HostSpace;
    using execution_space = OpenMP;
};
struct HostSpace {
    using memory_space = HostSpace;
    using execution_space = OpenMP;
};
using Serial = OpenMP;  // one host backend is enough for the oracle
using DefaultExecutionSpace = OpenMP;
using DefaultHostExecutionSpace = OpenMP;
struct MemoryUnmanaged {};

namespace detail_shim {
inline bool& initialized_flag() { static bool f = false; return f; }
}
struct InitializationSettings {
    int device_id = 0;
    InitializationSettings& set_device_id(int d) { device_id = d; return *this; }
};
inline void initialize() { detail_shim::initialized_flag() = true; }
inline void initialize(const InitializationSettings&) { initialize(); }
inline void finalize() { detail_shim::initialized_flag() = false; }
inline bool is_initialized() { return detail_shim::initialized_flag(); }

template <class DataType, class... Props> class View;

// One-dimensional view.  Copies share the same storage (like Kokkos).
template <class T, class... Props>
class View<T*, Props...> {
public:
    using value_type = T;
    using non_const_value_type = std::remove_const_t<T>;
    using execution_space = OpenMP;
    using memory_space = HostSpace;

    View() = default;
    View(const std::string& /*label*/, std::size_t n)
        : owner_(std::shared_ptr<non_const_value_type[]>(new non_const_value_type[n]())),
          ptr_(owner_.get()), n_(n) {}
    View(T* p, std::size_t n) : ptr_(p), n_(n) {}

    template <class U, class... P2,
              class = std::enable_if_t<std::is_convertible_v<U*, T*>>>
    View(const View<U*, P2...>& o) : owner_(o.owner_), ptr_(o.data()), n_(o.extent(0)) {}

    T& operator()(std::size_t i) const { return ptr_[i]; }
    T& operator[](std::size_t i) const { return ptr_[i]; }
    std::size_t extent(int) const { return n_; }
    std::size_t size() const { return n_; }
    T* data() const { return ptr_; }

    std::shared_ptr<non_const_value_type[]> owner_;
private:
    T* ptr_ = nullptr;
    std::size_t n_ = 0;
};

template <class E> struct RangePolicy {
    std::size_t begin, end;
    RangePolicy(std::size_t b, std::size_t e) : begin(b), end(e) {}
};

template <class F>
inline void parallel_for(const std::string&, const RangePolicy<OpenMP>& p, const F& f) {
    const long long b = (long long)p.begin, e = (long long)p.end;
#pragma omp parallel for schedule(static)
    for (long long i = b; i < e; ++i) f(i);
}
template <class F, class I, class = std::enable_if_t<std::is_integral_v<I>>>
inline void parallel_for(const std::string& name, I n, const F& f) {
    parallel_for(name, RangePolicy<OpenMP>(0, (std::size_t)n), f);
}

template <class F, class T>
inline void parallel_reduce(const std::string&, const RangePolicy<OpenMP>& p, const F& f, T& result) {
    const long long b = (long long)p.begin, e = (long long)p.end;
#ifdef _OPENMP
    const int nt = omp_get_max_threads();
#else
    const int nt = 1;
#endif
    std::vector<T> part(nt, T());
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        const int t = omp_get_thread_num();
#else
        const int t = 0;
#endif
        T local = T();
#pragma omp for schedule(static)
        for (long long i = b; i < e; ++i) f(i, local);
        part[t] = local;
    }
    T acc = T();
    for (int t = 0; t < nt; ++t) acc += part[t];
    result = acc;
}

template <class T, class... P1, class U, class... P2>
inline void deep_copy(const View<T*, P1...>& dst, const View<U*, P2...>& src) {
    if ((const void*)dst.data() == (const void*)src.data()) return;
    const std::size_t n = dst.extent(0) < src.extent(0) ? dst.extent(0) : src.extent(0);
    std::memcpy((void*)dst.data(), (const void*)src.data(), n * sizeof(T));
}
template <class T, class... P1, class S,
          class = std::enable_if_t<std::is_convertible_v<S, std::remove_const_t<T>>>>
inline void deep_copy(const View<T*, P1...>& dst, const S& value) {
    const std::size_t n = dst.extent(0);
    std::remove_const_t<T> v = value;
    T* d = dst.data();
    for (std::size_t i = 0; i < n; ++i) d[i] = v;
}
template <class T, class... P1, class Src>
inline void deep_copy(const OpenMP&, const View<T*, P1...>& dst, const Src& src) {
    deep_copy(dst, src);
}

template <class T, class... P>
inline View<T*, P...> create_mirror_view(const View<T*, P...>& v) { return v; }

}  // namespace Kokkos
