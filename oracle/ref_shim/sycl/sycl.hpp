// Host-only subset of the SYCL 2020 API — TEST INFRASTRUCTURE for the oracle.
//
// It lets the reference's own kernels and drivers (SC-SGS/PortLBM include/lbm/**, compiled from
// their original location, unmodified) run sequentially on the CPU, so that the restated oracle
// in oracle/plbm_oracle.c can be checked against the reference's code itself.  Only what those
// sources use is provided: queue submit/copy/fill/wait, malloc_device/free, range/id/item,
// nd_range/nd_item with work-group barriers (one ucontext fiber per work-item, switched at every
// barrier), local_accessor, and the math built-ins sqrt/isnan/abs/pow.
#pragma once

#include <ucontext.h>

#include <algorithm>
#include <array>
#include <functional>
#include <future>
#include <iostream>
#include <limits>
#include <thread>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace sycl {

namespace access {
enum class mode { read, write, read_write };
}

template <int D> struct range {
    size_t v[D];
    range(size_t a) requires(D == 1) : v{ a } {}
    range(size_t a, size_t b) requires(D == 2) : v{ a, b } {}
    size_t get(int i) const { return v[i]; }
    size_t operator[](int i) const { return v[i]; }
    size_t size() const { size_t s = 1; for (int i = 0; i < D; ++i) s *= v[i]; return s; }
};

template <int D> struct id {
    size_t v[D];
    size_t get(int i) const { return v[i]; }
    size_t operator[](int i) const { return v[i]; }
    operator size_t() const requires(D == 1) { return v[0]; }
};

template <int D> struct item {
    id<D> i;
    range<D> r;
    size_t get_id(int k) const { return i.v[k]; }
    id<D> get_id() const { return i; }
    size_t get_range(int k) const { return r.v[k]; }
    size_t operator[](int k) const { return i.v[k]; }
    operator size_t() const requires(D == 1) { return i.v[0]; }
};

template <int D> struct nd_range {
    range<D> g, l;
    nd_range(range<D> global, range<D> local) : g(global), l(local) {}
};

namespace detail {
// Fiber scheduler of the work-group being executed (one at a time, on the calling thread).
struct Group {
    ucontext_t sched;
    std::vector<ucontext_t> ctx;
    size_t current = 0;
};
inline thread_local Group *g_group = nullptr;
// Thrown by a barrier reached outside a fiber: the launch is then rerun with fibers.  No kernel
// of the reference writes global memory before its first barrier, so the rerun is exact.
struct NeedsFibers {};
}  // namespace detail

template <int D> struct nd_item {
    size_t gid[D], lid[D], lr[D], grp[D];
    size_t get_global_id(int k) const { return gid[k]; }
    size_t get_local_id(int k) const { return lid[k]; }
    size_t get_local_range(int k) const { return lr[k]; }
    size_t get_group(int k) const { return grp[k]; }
    void barrier() const
    {
        detail::Group *g = detail::g_group;
        if (!g) throw detail::NeedsFibers{};
        swapcontext(&g->ctx[g->current], &g->sched);
    }
};

template <typename T, int D = 1> class local_accessor {
  public:
    template <typename H> local_accessor(range<D> r, H &) : buf_(std::make_shared<std::vector<T>>(r.size())) {}
    T &operator[](size_t i) const { return (*buf_)[i]; }

  private:
    std::shared_ptr<std::vector<T>> buf_;
};

template <typename T, int N> struct vec {
    T v[N];
    vec(T a, T b) requires(N == 2) : v{ a, b } {}
    T &operator[](int i) { return v[i]; }
    const T &operator[](int i) const { return v[i]; }
};

class handler {
  public:
    template <typename K> void parallel_for(size_t n, K k) { parallel_for(range<1>(n), k); }

    template <typename K> void parallel_for(range<1> r, K k)
    {
        for (size_t i = 0; i < r.v[0]; ++i) {
            if constexpr (std::is_invocable_v<K, item<1>>) k(item<1>{ id<1>{ { i } }, r });
            else k(id<1>{ { i } });
        }
    }

    template <typename K> void parallel_for(range<2> r, K k)
    {
        for (size_t a = 0; a < r.v[0]; ++a)
            for (size_t b = 0; b < r.v[1]; ++b) {
                if constexpr (std::is_invocable_v<K, item<2>>) k(item<2>{ id<2>{ { a, b } }, r });
                else k(id<2>{ { a, b } });
            }
    }

    // Work-groups run one after another; inside a group every work-item is a fiber that runs until
    // its next barrier, so all items reach barrier k before any passes it.
    template <typename K> void parallel_for(nd_range<2> nr, K k)
    {
        const size_t l0 = nr.l.v[0], l1 = nr.l.v[1], n = l0 * l1;
        const size_t g0 = nr.g.v[0] / l0, g1 = nr.g.v[1] / l1;
        // Barrier-free kernels run directly; the first work-item tells which kind this is.
        bool direct = true;
        try {
            k(nd_item<2>{ { 0, 0 }, { 0, 0 }, { l0, l1 }, { 0, 0 } });
        } catch (const detail::NeedsFibers &) {
            direct = false;
        }
        if (direct) {
            for (size_t ga = 0; ga < g0; ++ga)
                for (size_t gb = 0; gb < g1; ++gb)
                    for (size_t a = 0; a < l0; ++a)
                        for (size_t b = 0; b < l1; ++b) {
                            if (ga == 0 && gb == 0 && a == 0 && b == 0) continue;
                            k(nd_item<2>{ { ga * l0 + a, gb * l1 + b }, { a, b }, { l0, l1 }, { ga, gb } });
                        }
            return;
        }
        constexpr size_t STACK = 32 * 1024;
        std::unique_ptr<char[]> stacks(new char[n * STACK]);
        std::vector<nd_item<2>> items(n);
        std::vector<int> done(n);
        detail::Group grp;
        grp.ctx.resize(n);
        struct Arg { K *k; nd_item<2> *it; int *done; detail::Group *g; };
        std::vector<Arg> args(n);
        for (size_t ga = 0; ga < g0; ++ga)
            for (size_t gb = 0; gb < g1; ++gb) {
                for (size_t a = 0; a < l0; ++a)
                    for (size_t b = 0; b < l1; ++b) {
                        const size_t j = a * l1 + b;
                        items[j] = nd_item<2>{ { ga * l0 + a, gb * l1 + b }, { a, b }, { l0, l1 }, { ga, gb } };
                        done[j] = 0;
                        args[j] = Arg{ &k, &items[j], &done[j], &grp };
                        getcontext(&grp.ctx[j]);
                        grp.ctx[j].uc_stack.ss_sp = &stacks[j * STACK];
                        grp.ctx[j].uc_stack.ss_size = STACK;
                        grp.ctx[j].uc_link = &grp.sched;
                        auto entry = +[](unsigned lo, unsigned hi) {
                            Arg *x = reinterpret_cast<Arg *>(((uintptr_t)hi << 32) | (uintptr_t)lo);
                            (*x->k)(*x->it);
                            *x->done = 1;
                        };
                        const uintptr_t p = reinterpret_cast<uintptr_t>(&args[j]);
                        makecontext(&grp.ctx[j], (void (*)())entry, 2, (unsigned)(p & 0xffffffffu), (unsigned)(p >> 32));
                    }
                detail::g_group = &grp;
                bool all = false;
                while (!all) {
                    all = true;
                    for (size_t j = 0; j < n; ++j) {
                        if (done[j]) continue;
                        grp.current = j;
                        swapcontext(&grp.sched, &grp.ctx[j]);
                        if (!done[j]) all = false;
                    }
                }
                detail::g_group = nullptr;
            }
    }
};

struct event {
    void wait() {}
};

namespace info {
namespace device {
struct max_work_group_size { using return_type = size_t; };
struct name { using return_type = std::string; };
}  // namespace device
}  // namespace info

struct device {
    template <typename P> typename P::return_type get_info() const
    {
        if constexpr (std::is_same_v<P, info::device::max_work_group_size>) return 1024;
        else return std::string("host (oracle shim)");
    }
};

struct default_selector {};
struct cpu_selector {};

class queue {
  public:
    queue() = default;
    template <typename S> explicit queue(const S &) {}
    template <typename F> event submit(F f)
    {
        handler h;
        f(h);
        return {};
    }
    template <typename T> event copy(const T *src, T *dst, size_t n)
    {
        std::memmove(dst, src, n * sizeof(T));
        return {};
    }
    template <typename T> event fill(T *p, const T &v, size_t n)
    {
        std::fill(p, p + n, v);
        return {};
    }
    event memcpy(void *dst, const void *src, size_t bytes)
    {
        std::memmove(dst, src, bytes);
        return {};
    }
    void wait() {}
    device get_device() const { return {}; }
};

template <typename T> T *malloc_device(size_t n, queue &)
{
    void *p = std::aligned_alloc(64, ((n * sizeof(T) + 63) / 64) * 64 + 64);
    return static_cast<T *>(p);
}
template <typename T> void free(T *p, queue &) { std::free(p); }

inline double sqrt(double x) { return std::sqrt(x); }
inline float sqrt(float x) { return std::sqrt(x); }
inline bool isnan(double x) { return std::isnan(x); }
inline bool isnan(float x) { return std::isnan(x); }
inline unsigned abs(unsigned x) { return x; }
inline int abs(int x) { return x < 0 ? -x : x; }
inline float pow(float a, float b) { return std::pow(a, b); }
inline double pow(double a, double b) { return std::pow(a, b); }

}  // namespace sycl
