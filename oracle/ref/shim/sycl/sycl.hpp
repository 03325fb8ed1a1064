// Minimal serial host stand-in for the SYCL runtime, written for this project so that the
// reference's own sources (kernel bodies, block functions, class Fluid / XFLUIDS) compile with
// g++ and run on the CPU. Only what the reference path uses is provided: parallel_for over ranges
// and nd_ranges (executed serially, work items in order), reductions, USM allocations as host
// memory, queue/event/handler with immediate execution, and the math functions.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

namespace sycl {

// ---- math ----------------------------------------------------------------------------------
using std::ceil;
using std::exp;
using std::fabs;
using std::isinf;
using std::isnan;
using std::log;
using std::log10;
using std::pow;
using std::sqrt;
using std::tanh;
template <class T> inline T max(T a, T b) { return (a < b) ? b : a; }
template <class T> inline T min(T a, T b) { return (b < a) ? b : a; }
template <class T> inline T abs(T a) { return a < T(0) ? -a : a; }
template <class T> inline T step(T edge, T x) { return x < edge ? T(0) : T(1); }
template <class T> inline T pown(T x, int n) { return std::pow(x, n); }

// ---- index spaces ----------------------------------------------------------------------------
template <int D>
struct range {
    size_t v[3] = {1, 1, 1};
    range() = default;
    range(size_t a) { v[0] = a; }
    range(size_t a, size_t b) { v[0] = a, v[1] = b; }
    range(size_t a, size_t b, size_t c) { v[0] = a, v[1] = b, v[2] = c; }
    size_t operator[](int d) const { return v[d]; }
    size_t &operator[](int d) { return v[d]; }
    size_t size() const { return v[0] * v[1] * v[2]; }
    bool operator==(const range &o) const { return v[0] == o.v[0] && v[1] == o.v[1] && v[2] == o.v[2]; }
};
range(size_t)->range<1>;
range(size_t, size_t)->range<2>;
range(size_t, size_t, size_t)->range<3>;
template <int D>
struct id {
    size_t v[3] = {0, 0, 0};
    size_t operator[](int d) const { return v[d]; }
    operator size_t() const { return v[0]; }
};
template <int D>
struct nd_range {
    range<D> g, l;
    nd_range(range<D> global, range<D> local) : g(global), l(local) {}
    range<D> get_global_range() const { return g; }
    range<D> get_local_range() const { return l; }
};
template <int D>
struct nd_item {
    size_t gid[3], lid[3], grp[3], lr[3], gr[3];
    size_t get_global_id(int d) const { return gid[d]; }
    id<D> get_global_id() const { id<D> r; for (int q = 0; q < 3; q++) r.v[q] = gid[q]; return r; }
    size_t get_local_id(int d) const { return lid[d]; }
    size_t get_group(int d) const { return grp[d]; }
    size_t get_local_range(int d) const { return lr[d]; }
    size_t get_global_range(int d) const { return gr[d]; }
    size_t get_global_linear_id() const { return (gid[0] * gr[1] + gid[1]) * gr[2] + gid[2]; }
    void barrier() const {}
};
template <int D>
struct item {
    size_t gid[3];
    size_t operator[](int d) const { return gid[d]; }
    size_t get_id(int d) const { return gid[d]; }
};

// ---- reductions ------------------------------------------------------------------------------
template <class T = void> struct plus { T operator()(const T &a, const T &b) const { return a + b; } };
template <class T = void> struct maximum { T operator()(const T &a, const T &b) const { return (a < b) ? b : a; } };
template <class T = void> struct minimum { T operator()(const T &a, const T &b) const { return (b < a) ? b : a; } };
template <class T, class Op>
struct reducer {
    T *ptr;
    T val;
    Op op;
    void combine(const T &x) { val = op(val, x); }
    reducer &operator+=(const T &x) { val = val + x; return *this; }
};
template <class T, class Op>
struct reduction_t {
    T *ptr;
    Op op;
};
template <class T, class Op>
reduction_t<T, Op> reduction(T *ptr, Op op) { return reduction_t<T, Op>{ptr, op}; }

// ---- devices, queue, events ------------------------------------------------------------------
namespace info {
namespace device {
struct name {};
struct version {};
}  // namespace device
}  // namespace info
struct device {
    template <class P> std::string get_info() const { return "host"; }
};
struct platform {
    std::vector<device> get_devices() const { return std::vector<device>(4); }
    static std::vector<platform> get_platforms() { return std::vector<platform>(4); }
};
struct event {
    void wait() {}
};
struct handler;
struct stream {
    stream(size_t, size_t, handler &) {}
    template <class T> const stream &operator<<(const T &x) const { std::cout << x; return *this; }
};

template <int D, class F>
inline void run_nd(const nd_range<D> &r, F &&f) {
    nd_item<D> it;
    for (int q = 0; q < 3; q++) it.lr[q] = r.l.v[q], it.gr[q] = r.g.v[q];
    for (size_t a = 0; a < r.g.v[0]; a++)
        for (size_t b = 0; b < r.g.v[1]; b++)
            for (size_t c = 0; c < r.g.v[2]; c++) {
                it.gid[0] = a, it.gid[1] = b, it.gid[2] = c;
                it.lid[0] = a % r.l.v[0], it.lid[1] = b % r.l.v[1], it.lid[2] = c % r.l.v[2];
                it.grp[0] = a / r.l.v[0], it.grp[1] = b / r.l.v[1], it.grp[2] = c / r.l.v[2];
                f(it);
            }
}

struct handler {
    void depends_on(const event &) {}
    template <int D, class F>
    void parallel_for(nd_range<D> r, F f) { run_nd(r, [&](nd_item<D> &it) { f(it); }); }
    template <int D, class F>
    void parallel_for(range<D> r, F f) {
        for (size_t a = 0; a < r.v[0]; a++)
            for (size_t b = 0; b < r.v[1]; b++)
                for (size_t c = 0; c < r.v[2]; c++) f(item<D>{{a, b, c}});
    }
    // parallel_for(nd_range, reduction..., kernel): the kernel receives one reducer per reduction
    template <int D, class... A>
    void parallel_for(nd_range<D> r, A... args) {
        auto tup = std::make_tuple(args...);
        constexpr size_t N = sizeof...(A) - 1;
        run_reduce(r, tup, std::make_index_sequence<N>{});
    }
    template <int D, class Tup, size_t... I>
    void run_reduce(nd_range<D> r, Tup &tup, std::index_sequence<I...>) {
        auto &f = std::get<sizeof...(I)>(tup);
        auto reds = std::make_tuple(make_reducer(std::get<I>(tup))...);
        run_nd(r, [&](nd_item<D> &it) { f(it, std::get<I>(reds)...); });
        ((*std::get<I>(reds).ptr = std::get<I>(reds).val), ...);
    }
    template <class T, class Op>
    static reducer<T, Op> make_reducer(const reduction_t<T, Op> &rd) { return reducer<T, Op>{rd.ptr, *rd.ptr, rd.op}; }
    template <class F>
    void single_task(F f) { f(); }
};

struct queue {
    device dev;
    queue() = default;
    explicit queue(const device &d) : dev(d) {}
    template <class F>
    event submit(F f) { handler h; f(h); return event{}; }
    event memcpy(void *dst, const void *src, size_t n) { std::memmove(dst, src, n); return event{}; }
    event memset(void *dst, int v, size_t n) { std::memset(dst, v, n); return event{}; }
    template <class T> event fill(T *dst, const T &v, size_t n) { for (size_t q = 0; q < n; q++) dst[q] = v; return event{}; }
    void wait() {}
    device get_device() const { return dev; }
};

inline void *aligned(size_t bytes) {
    void *p = nullptr;
    if (posix_memalign(&p, 64, bytes ? bytes : 64) != 0) return nullptr;
    std::memset(p, 0, bytes);
    return p;
}
template <class T> T *malloc_device(size_t n, const queue &) { return (T *)aligned(n * sizeof(T)); }
template <class T> T *malloc_host(size_t n, const queue &) { return (T *)aligned(n * sizeof(T)); }
template <class T> T *malloc_shared(size_t n, const queue &) { return (T *)aligned(n * sizeof(T)); }
inline void *malloc_device(size_t n, const queue &) { return aligned(n); }
inline void *malloc_host(size_t n, const queue &) { return aligned(n); }
inline void *malloc_shared(size_t n, const queue &) { return aligned(n); }
inline void free(void *p, const queue &) { std::free(p); }

}  // namespace sycl
