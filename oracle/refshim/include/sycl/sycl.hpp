// sycl.hpp — a minimal, single-threaded host implementation of the SYCL 2020
// subset that the reference's kernel sources use, so that those sources can
// be compiled with g++ and run on the CPU to produce golden vectors.
//
// TEST INFRASTRUCTURE ONLY (golden-vector generation for the oracle); never
// part of the product.
//
// Range kernels run as plain loops.  ND-range kernels run one work-group at
// a time with every work-item as a cooperative fiber (ucontext): a barrier
// or group collective switches to the next work-item, and the group moves on
// when all of its work-items have reached the same point.  With no
// preemption, atomic_ref operations are ordinary memory operations.
#pragma once

#include <ucontext.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <tuple>
#include <type_traits>
#include <vector>

namespace std {
using ::hypotf;
}

namespace sycl {

enum class memory_order { relaxed, acquire, release, acq_rel, seq_cst };
enum class memory_scope { work_item, sub_group, work_group, device, system };
inline constexpr memory_scope memory_scope_device = memory_scope::device;
inline constexpr memory_scope memory_scope_work_group = memory_scope::work_group;

namespace access {
enum class address_space { global_space, local_space, constant_space, private_space, generic_space };
enum class fence_space { local_space, global_space, global_and_local };
}  // namespace access

template <int D>
struct range {
    size_t v[D];
    range(size_t a) requires(D == 1) : v{a} {}
    range(size_t a, size_t b) requires(D == 2) : v{a, b} {}
    size_t operator[](int i) const { return v[i]; }
    size_t size() const {
        size_t s = 1;
        for (int i = 0; i < D; i++) s *= v[i];
        return s;
    }
};
range(size_t)->range<1>;
range(size_t, size_t)->range<2>;

template <int D>
struct nd_range {
    range<D> global, local;
    nd_range(range<D> g, range<D> l) : global(g), local(l) {}
};
template <int D>
nd_range(range<D>, range<D>) -> nd_range<D>;

template <int D>
class item {
public:
    range<D> r;
    size_t i[D];
    size_t get_id(int d) const { return i[d]; }
    size_t get_range(int d) const { return r[d]; }
    size_t get_linear_id() const {
        size_t l = 0;
        for (int d = 0; d < D; d++) l = l * r[d] + i[d];
        return l;
    }
};

namespace detail {
// One work-group in flight: fibers and a scratch area for collectives.
struct GroupRun {
    std::vector<ucontext_t> ctx;
    ucontext_t sched;
    std::vector<char> done;
    size_t current = 0;
    std::vector<unsigned char> slots;  // collective operands, 16 bytes per item
};
inline thread_local GroupRun* g_run = nullptr;
inline void yield_to_scheduler() { swapcontext(&g_run->ctx[g_run->current], &g_run->sched); }
}  // namespace detail

template <int D>
class group {
public:
    size_t linear_local = 0, local_size = 0;
};

template <int D>
class nd_item {
public:
    nd_range<D> nr;
    size_t gid[D], lid[D], grp[D];
    size_t get_global_id(int d) const { return gid[d]; }
    size_t get_local_id(int d) const { return lid[d]; }
    size_t get_group(int d) const { return grp[d]; }
    size_t get_local_range(int d) const { return nr.local[d]; }
    size_t get_global_range(int d) const { return nr.global[d]; }
    size_t get_local_linear_id() const {
        size_t l = 0;
        for (int d = 0; d < D; d++) l = l * nr.local[d] + lid[d];
        return l;
    }
    group<D> get_group() const { return group<D>{get_local_linear_id(), nr.local.size()}; }
    void barrier(access::fence_space = access::fence_space::global_and_local) const { detail::yield_to_scheduler(); }
};

template <typename T, int N>
struct vec {
    T d[N];
    vec() : d{} {}
    vec(T a, T b) requires(N == 2) : d{a, b} {}
    T& operator[](int i) { return d[i]; }
    const T& operator[](int i) const { return d[i]; }
    T x() const { return d[0]; }
    T y() const { return d[1]; }
};
template <typename T>
vec(T, T) -> vec<T, 2>;

template <typename T, memory_order O, memory_scope S, access::address_space A = access::address_space::generic_space>
class atomic_ref {
    T& r;

public:
    static constexpr bool is_always_lock_free = true;
    explicit atomic_ref(T& x) : r(x) {}
    T load() const { return r; }
    void store(T v) const { r = v; }
    T fetch_add(T v) const {
        T o = r;
        r = o + v;
        return o;
    }
    T fetch_min(T v) const {
        T o = r;
        if (v < o) r = v;
        return o;
    }
};

template <typename T>
T min(T a, T b) { return b < a ? b : a; }
template <typename T>
T max(T a, T b) { return a < b ? b : a; }
template <typename T>
T clamp(T x, T lo, T hi) { return min(max(x, lo), hi); }
template <typename T>
T popcount(T x) { return (T)__builtin_popcountll((unsigned long long)x); }

template <typename T = void>
struct minimum {
    template <typename U>
    U operator()(const U& a, const U& b) const { return b < a ? b : a; }
};

// Collectives: every work-item deposits its value, waits for the group,
// then reads all values (and waits again so the slots can be reused).
template <int D, typename T, typename Op>
T reduce_over_group(group<D> g, T x, Op op) {
    static_assert(sizeof(T) <= 16);
    auto* run = detail::g_run;
    std::memcpy(&run->slots[g.linear_local * 16], &x, sizeof(T));
    detail::yield_to_scheduler();
    T acc;
    std::memcpy(&acc, &run->slots[0], sizeof(T));
    for (size_t i = 1; i < g.local_size; i++) {
        T v;
        std::memcpy(&v, &run->slots[i * 16], sizeof(T));
        acc = op(acc, v);
    }
    detail::yield_to_scheduler();
    return acc;
}
template <int D, typename T, typename Op>
T inclusive_scan_over_group(group<D> g, T x, Op op) {
    static_assert(sizeof(T) <= 16);
    auto* run = detail::g_run;
    std::memcpy(&run->slots[g.linear_local * 16], &x, sizeof(T));
    detail::yield_to_scheduler();
    T acc;
    std::memcpy(&acc, &run->slots[0], sizeof(T));
    for (size_t i = 1; i <= g.linear_local; i++) {
        T v;
        std::memcpy(&v, &run->slots[i * 16], sizeof(T));
        acc = op(acc, v);
    }
    detail::yield_to_scheduler();
    return acc;
}

class event {
public:
    void wait() {}
};

namespace detail {
struct LocalBase {
    virtual ~LocalBase() = default;
};

template <int D, typename K>
struct FiberArgs {
    const K* k;
    nd_item<D> it;
};
template <int D, typename K>
void fiber_entry(unsigned lo, unsigned hi) {
    auto* a = reinterpret_cast<FiberArgs<D, K>*>((uintptr_t)lo | ((uintptr_t)hi << 32));
    (*a->k)(a->it);
    g_run->done[g_run->current] = 1;
    // returning resumes uc_link (the scheduler)
}

template <int D, typename K>
void run_nd(nd_range<D> nr, const K& k) {
    size_t groups[D], L = nr.local.size();
    for (int d = 0; d < D; d++) groups[d] = nr.global[d] / nr.local[d];
    size_t ngroups = 1;
    for (int d = 0; d < D; d++) ngroups *= groups[d];
    constexpr size_t STACK = 256 * 1024;
    std::vector<std::unique_ptr<char[]>> stacks(L);
    for (auto& s : stacks) s.reset(new char[STACK]);
    GroupRun run;
    run.ctx.resize(L);
    run.done.assign(L, 0);
    run.slots.assign(L * 16, 0);
    std::vector<FiberArgs<D, K>> args;
    args.reserve(L);  // never reallocates: fibers keep pointers into it
    GroupRun* saved = g_run;
    g_run = &run;
    for (size_t g = 0; g < ngroups; g++) {
        size_t gi[D];
        size_t rem = g;
        for (int d = D - 1; d >= 0; d--) {
            gi[d] = rem % groups[d];
            rem /= groups[d];
        }
        args.clear();
        for (size_t l = 0; l < L; l++) {
            size_t li[D];
            size_t r2 = l;
            for (int d = D - 1; d >= 0; d--) {
                li[d] = r2 % nr.local[d];
                r2 /= nr.local[d];
            }
            nd_item<D> it{nr, {}, {}, {}};
            for (int d = 0; d < D; d++) {
                it.lid[d] = li[d];
                it.grp[d] = gi[d];
                it.gid[d] = gi[d] * nr.local[d] + li[d];
            }
            args.push_back(FiberArgs<D, K>{&k, it});
            getcontext(&run.ctx[l]);
            run.ctx[l].uc_stack.ss_sp = stacks[l].get();
            run.ctx[l].uc_stack.ss_size = STACK;
            run.ctx[l].uc_link = &run.sched;
            uintptr_t p = (uintptr_t)&args[l];
            makecontext(&run.ctx[l], (void (*)())fiber_entry<D, K>, 2, (unsigned)(p & 0xFFFFFFFFu),
                        (unsigned)(p >> 32));
            run.done[l] = 0;
        }
        bool left = true;
        while (left) {
            left = false;
            for (size_t l = 0; l < L; l++) {
                if (run.done[l]) continue;
                run.current = l;
                swapcontext(&run.sched, &run.ctx[l]);
                if (!run.done[l]) left = true;
            }
        }
    }
    g_run = saved;
}

template <int D, typename K>
void run_range(range<D> r, const K& k) {
    if constexpr (D == 1) {
        for (size_t i = 0; i < r[0]; i++) k(item<1>{r, {i}});
    } else {
        for (size_t i = 0; i < r[0]; i++)
            for (size_t j = 0; j < r[1]; j++) k(item<2>{r, {i, j}});
    }
}
}  // namespace detail

class handler {
public:
    void depends_on(const std::vector<event>&) {}
    void depends_on(event) {}
    template <int D, typename K>
    void parallel_for(nd_range<D> nr, const K& k) { detail::run_nd(nr, k); }
    template <int D, typename K>
    void parallel_for(range<D> r, const K& k) { detail::run_range(r, k); }
};

template <typename T, int D = 1>
class local_accessor {
    std::shared_ptr<std::vector<T>> data;

public:
    local_accessor(range<D> r, handler&) : data(std::make_shared<std::vector<T>>(r.size())) {}
    T& operator[](size_t i) const { return (*data)[i]; }
    T* get_pointer() const { return data->data(); }
};

class queue {
public:
    template <typename F>
    event submit(F f) {
        handler h;
        f(h);
        return event{};
    }
    template <int D, typename K>
    event parallel_for(range<D> r, const std::vector<event>&, const K& k) {
        detail::run_range(r, k);
        return event{};
    }
    template <int D, typename K>
    event parallel_for(range<D> r, event, const K& k) {
        detail::run_range(r, k);
        return event{};
    }
    template <int D, typename K>
    event parallel_for(range<D> r, const K& k) {
        detail::run_range(r, k);
        return event{};
    }
    template <int D, typename K>
    event parallel_for(nd_range<D> nr, const K& k) {
        detail::run_nd(nr, k);
        return event{};
    }
    void wait() {}
};

}  // namespace sycl
