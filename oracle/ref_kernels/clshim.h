// OpenCL C -> C++ shim for running the reference's kernel files on host cores.
//
// Test infrastructure only (the oracle's pin against the reference itself).
// A kernel file is compiled as C++ after this header: __kernel and __global
// vanish, kernel-scope __local arrays become static thread_local (one copy
// per host thread, and a work-group runs entirely on one host thread), and
// the work-item functions read the running work-item's ids.
//
// Work-items run as ucontext fibers.  A work-group's fibers are resumed in
// order, each until it reaches barrier() or returns.  A round of the group
// therefore ends only when every work-item has reached the same barrier,
// which is barrier()'s contract.  Fibers never run concurrently, so the
// __local atomics are plain read-modify-writes.  Work-groups of one launch run
// on a pool of host threads.
#pragma once
#include <ucontext.h>

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned long ulong;
struct uint2 {
    uint x, y;
};

namespace clshim {

struct Group {
    size_t group, ngroups, lsize;
    std::vector<ucontext_t> wi;
    std::vector<char> done;
    ucontext_t sched;
    const std::function<void()> *body;
};
inline thread_local Group *g_cur = nullptr;
inline thread_local size_t g_lid = 0;

inline void trampoline() {
    (*g_cur->body)();
    g_cur->done[g_lid] = 1;
    // returning switches to uc_link (the scheduler)
}

constexpr size_t kStack = 64 * 1024;

// Run one work-group to completion on this host thread.
inline void run_group(Group &G, std::vector<char> &stacks) {
    G.wi.resize(G.lsize);
    G.done.assign(G.lsize, 0);
    if (stacks.size() < G.lsize * kStack) stacks.resize(G.lsize * kStack);
    for (size_t l = 0; l < G.lsize; l++) {
        getcontext(&G.wi[l]);
        G.wi[l].uc_stack.ss_sp = stacks.data() + l * kStack;
        G.wi[l].uc_stack.ss_size = kStack;
        G.wi[l].uc_link = &G.sched;
        makecontext(&G.wi[l], trampoline, 0);
    }
    g_cur = &G;
    for (;;) {
        bool alive = false;
        for (size_t l = 0; l < G.lsize; l++) {
            if (G.done[l]) continue;
            g_lid = l;
            swapcontext(&G.sched, &G.wi[l]);
            alive = alive || !G.done[l];
        }
        if (!alive) break;
    }
    g_cur = nullptr;
}

// NDRange launch: global = ngroups * lsize work-items (the reference always
// passes a global size that is a multiple of the local size).
inline void launch(size_t global, size_t local, const std::function<void()> &body, int threads = 0) {
    if (local == 0 || global == 0) return;
    const size_t ngroups = global / local;
    unsigned nt = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
    if (nt > ngroups) nt = (unsigned)ngroups;
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        std::vector<char> stacks;
        Group G;
        G.ngroups = ngroups;
        G.lsize = local;
        G.body = &body;
        for (;;) {
            const size_t g = next.fetch_add(1);
            if (g >= ngroups) break;
            G.group = g;
            run_group(G, stacks);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; t++) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
}

}  // namespace clshim

// ---- OpenCL C work-item functions and built-ins used by the kernels -------
inline size_t get_local_id(uint d) { return d == 0 ? clshim::g_lid : 0; }
inline size_t get_group_id(uint d) { return d == 0 ? clshim::g_cur->group : 0; }
inline size_t get_local_size(uint d) { return d == 0 ? clshim::g_cur->lsize : 1; }
inline size_t get_num_groups(uint d) { return d == 0 ? clshim::g_cur->ngroups : 1; }
inline size_t get_global_id(uint d) { return d == 0 ? clshim::g_cur->group * clshim::g_cur->lsize + clshim::g_lid : 0; }
inline size_t get_global_size(uint d) { return d == 0 ? clshim::g_cur->ngroups * clshim::g_cur->lsize : 1; }

enum { CLK_LOCAL_MEM_FENCE = 1, CLK_GLOBAL_MEM_FENCE = 2 };
inline void barrier(int) { swapcontext(&clshim::g_cur->wi[clshim::g_lid], &clshim::g_cur->sched); }
inline void mem_fence(int) {}

template <class T> inline T atomic_cmpxchg(T *p, T cmp, T val) { T old = *p; if (old == cmp) *p = val; return old; }
template <class T> inline T atomic_xchg(T *p, T val) { T old = *p; *p = val; return old; }
template <class T> inline T atomic_add(T *p, T val) { T old = *p; *p = old + val; return old; }
template <class T> inline T atomic_inc(T *p) { T old = *p; *p = old + 1; return old; }

template <class A, class B> inline auto min(A a, B b) -> decltype(a + b) { return a < b ? a : b; }
template <class A, class B> inline auto max(A a, B b) -> decltype(a + b) { return a > b ? a : b; }

// Qualifiers and attributes.  Defined after every system header, so that
// only the kernel file sees them.
#define __kernel
#define __global
#define __constant const
#define __private
#define __local static thread_local
#define restrict __restrict__
#define __attribute(x)
#define __attribute__(x)
