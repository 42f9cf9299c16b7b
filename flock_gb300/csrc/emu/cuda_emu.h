// cuda_emu.h -- runs the CTA-level device code of this library on the host:
// one CTA = 32 to 256 fibers (whole warps) on one OS thread; __syncthreads is
// a CTA barrier and a warp shuffle a barrier of its warp, both checking that
// every thread arrived from the same call site; atomics are std::atomic_ref.
// Used by the host test harness (emu_check.cpp) to execute the unmodified
// device functions under AddressSanitizer / UndefinedBehaviorSanitizer, so
// that out-of-bounds accesses in the device logic show up on the CPU.
#pragma once
#include <ucontext.h>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>
#include <cstdio>

#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __noinline__
#define __launch_bounds__(...)
#define __align__(x) alignas(x)

struct int4 { int x, y, z, w; };
inline int4 make_int4(int x, int y, int z, int w) { return int4{x, y, z, w}; }
struct int2 { int x, y; };
inline int2 make_int2(int x, int y) { return int2{x, y}; }
struct EmuDim { unsigned x = 0, y = 0, z = 0; };

namespace emu {
constexpr int kMaxThreads = 256;
// One CTA = blockDim.x fibers on the calling OS thread; a barrier switches
// back to the scheduler, which resumes a warp once all its threads reached a
// warp barrier, and the CTA once every thread reached a CTA barrier.
struct Cta {
    ucontext_t sched;
    ucontext_t fib[kMaxThreads];
    std::vector<char> stack[kMaxThreads];
    int wait[kMaxThreads];     // 0 running, 1 at a CTA barrier, 2 at a warp barrier
    bool finished[kMaxThreads];
    int cur = 0;
    uint64_t xchg[kMaxThreads];
    std::atomic<int> any{0};
    int site[kMaxThreads];     // call site of each thread's current barrier
    int mismatches = 0;
    long long barriers = 0;
};
inline Cta*& cta() { static Cta* c = nullptr; return c; }
inline EmuDim tid;
}  // namespace emu

inline EmuDim blockDim{32, 1, 1};   // set before run_cta: a multiple of 32, at most kMaxThreads
static const EmuDim blockIdx{0, 0, 0};
static const EmuDim gridDim{1, 1, 1};
#define threadIdx (emu::tid)

namespace emu {
// Every barrier (including the ones inside emulated shuffles) records its call
// site; threads meeting at one barrier phase from different sites means a
// __syncthreads() was reached divergently.
inline void wait_at(int line, int kind) {
    Cta* c = cta();
    const int me = c->cur;
    c->site[me] = line;
    c->wait[me] = kind;
    swapcontext(&c->fib[me], &c->sched);
    tid.x = (unsigned)me;
}
inline void sync_at(int line) { wait_at(line, 1); }
inline void warp_sync_at(int line) { wait_at(line, 2); }
}  // namespace emu
#define __syncthreads() emu::sync_at(__LINE__)
#define __syncwarp(...) emu::warp_sync_at(-4)
#define __syncthreads_or(p) emu::sync_or(p, __LINE__)
namespace emu {
inline int sync_or(int p, int line) {
    Cta* c = cta();
    sync_at(line);
    if (p) c->any.store(1);
    sync_at(line);
    const int r = c->any.load();
    sync_at(line);
    if (threadIdx.x == 0) c->any.store(0);
    sync_at(line);
    return r;
}
}  // namespace emu

// src: the source thread (in the caller's warp)
template <class T>
inline T emu_shfl(T v, int src) {
    emu::Cta* c = emu::cta();
    uint64_t bits = 0;
    memcpy(&bits, &v, sizeof(T));
    emu::warp_sync_at(-1);
    c->xchg[threadIdx.x] = bits;
    emu::warp_sync_at(-2);
    uint64_t got = c->xchg[src];
    emu::warp_sync_at(-3);
    T out;
    memcpy(&out, &got, sizeof(T));
    return out;
}
template <class T> inline T __shfl_xor_sync(unsigned, T v, int o) { return emu_shfl(v, (int)(threadIdx.x ^ (o & 31))); }
template <class T> inline T __shfl_up_sync(unsigned, T v, int o) {
    const int lane = (int)(threadIdx.x & 31);
    return emu_shfl(v, lane >= o ? (int)threadIdx.x - o : (int)threadIdx.x);
}

// Warp reductions (32-bit): every lane of the caller's warp gets the result.
inline unsigned emu_reduce(unsigned v, bool take_max) {
    emu::Cta* c = emu::cta();
    emu::warp_sync_at(-5);
    c->xchg[threadIdx.x] = v;
    emu::warp_sync_at(-6);
    const unsigned w0 = threadIdx.x & ~31u;
    unsigned r = (unsigned)c->xchg[w0];
    for (unsigned l = 1; l < 32; l++) {
        const unsigned x = (unsigned)c->xchg[w0 + l];
        r = take_max ? (x > r ? x : r) : (x < r ? x : r);
    }
    emu::warp_sync_at(-7);
    return r;
}
inline unsigned __reduce_min_sync(unsigned, unsigned v) { return emu_reduce(v, false); }
inline unsigned __reduce_max_sync(unsigned, unsigned v) { return emu_reduce(v, true); }

// Warp sum and ballot: every lane of the caller's warp gets the result.
inline unsigned emu_gather(unsigned v, int how) {
    emu::Cta* c = emu::cta();
    emu::warp_sync_at(-8);
    c->xchg[threadIdx.x] = v;
    emu::warp_sync_at(-9);
    const unsigned w0 = threadIdx.x & ~31u;
    unsigned r = 0;
    for (unsigned l = 0; l < 32; l++) {
        const unsigned x = (unsigned)c->xchg[w0 + l];
        r += how == 0 ? x : (x ? 1u << l : 0u);
    }
    emu::warp_sync_at(-10);
    return r;
}
inline unsigned __reduce_add_sync(unsigned, unsigned v) { return emu_gather(v, 0); }
inline unsigned __ballot_sync(unsigned, int p) { return emu_gather(p ? 1u : 0u, 1); }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __ffs(int x) { return __builtin_ffs(x); }

template <class T, class U> inline T atomicAdd(T* p, U v) { return std::atomic_ref<T>(*p).fetch_add((T)v); }
template <class T, class U> inline T atomicOr(T* p, U v) { return std::atomic_ref<T>(*p).fetch_or((T)v); }
template <class T, class U> inline T atomicExch(T* p, U v) { return std::atomic_ref<T>(*p).exchange((T)v); }
template <class T, class U, class W> inline T atomicCAS(T* p, U cmp, W v) {
    T c = (T)cmp;
    std::atomic_ref<T>(*p).compare_exchange_strong(c, (T)v);
    return c;
}
template <class T, class U> inline T atomicMin(T* p, U vv) {
    const T v = (T)vv;
    std::atomic_ref<T> a(*p);
    T cur = a.load();
    while (v < cur && !a.compare_exchange_weak(cur, v)) {}
    return cur;
}
inline float __ll2float_rn(long long x) { return (float)x; }
inline unsigned __float_as_uint(float f) { unsigned u; memcpy(&u, &f, 4); return u; }
inline float __uint_as_float(unsigned u) { float f; memcpy(&f, &u, 4); return f; }
inline int __float_as_int(float f) { int u; memcpy(&u, &f, 4); return u; }
inline float __int_as_float(int u) { float f; memcpy(&f, &u, 4); return f; }
inline int __float2int_rz(float f) { return (int)f; }
template <class T> inline T __ldcs(const T* p) { return *p; }
using std::min;
using std::max;

namespace emu {
inline const std::function<void()>*& entry() { static const std::function<void()>* f = nullptr; return f; }
inline void fiber_main() {
    Cta* c = cta();
    const int me = c->cur;
    tid.x = (unsigned)me;
    (*entry())();
    c->finished[me] = true;
    swapcontext(&c->fib[me], &c->sched);
}
// Run f() on one emulated CTA of blockDim.x threads.  Returns the number of
// barrier phases whose threads arrived from different call sites (0 when
// every barrier is reached uniformly), or -1 on a deadlock.
inline int run_cta(const std::function<void()>& f) {
    const int nt = (int)blockDim.x;
    if (nt < 32 || nt > kMaxThreads || nt % 32) { fprintf(stderr, "emu: bad block size %d\n", nt); return -1; }
    Cta* c = new Cta();
    cta() = c;
    entry() = &f;
    for (int t = 0; t < nt; t++) {
        c->stack[t].resize(1 << 17);
        getcontext(&c->fib[t]);
        c->fib[t].uc_stack.ss_sp = c->stack[t].data();
        c->fib[t].uc_stack.ss_size = c->stack[t].size();
        c->fib[t].uc_link = nullptr;
        makecontext(&c->fib[t], (void (*)())fiber_main, 0);
        c->wait[t] = 0;
        c->finished[t] = false;
    }
    auto mismatch = [&](int t0, int t) {
        if (c->mismatches++ < 5)
            fprintf(stderr, "barrier mismatch: thread %d at line %d, thread %d at line %d\n", t0, c->site[t0], t,
                    c->site[t]);
    };
    int result = 0;
    for (;;) {
        for (int t = 0; t < nt; t++) {
            if (c->finished[t] || c->wait[t]) continue;
            c->cur = t;
            swapcontext(&c->sched, &c->fib[t]);
        }
        int nfin = 0, ncta = 0;
        for (int t = 0; t < nt; t++) { nfin += c->finished[t]; ncta += c->wait[t] == 1; }
        if (nfin == nt) break;
        // warps whose every thread waits at a warp barrier go on first
        bool released = false;
        for (int w = 0; w < nt / 32; w++) {
            bool all = true;
            for (int t = 32 * w; t < 32 * w + 32; t++) all = all && !c->finished[t] && c->wait[t] == 2;
            if (!all) continue;
            for (int t = 32 * w + 1; t < 32 * w + 32; t++)
                if (c->site[t] != c->site[32 * w]) { mismatch(32 * w, t); break; }
            for (int t = 32 * w; t < 32 * w + 32; t++) c->wait[t] = 0;
            released = true;
        }
        if (released) continue;
        if (nfin > 0 || ncta != nt) {
            result = -1;
            fprintf(stderr, "deadlock: %d threads finished, %d at a CTA barrier\n", nfin, ncta);
            break;
        }
        c->barriers++;
        for (int t = 1; t < nt; t++)
            if (c->site[t] != c->site[0]) { mismatch(0, t); break; }
        for (int t = 0; t < nt; t++) c->wait[t] = 0;
    }
    if (result == 0) result = c->mismatches;
    cta() = nullptr;
    delete c;
    return result;
}
}  // namespace emu
