// cuda_emu.h -- runs the CTA-level device code of this library on the host:
// one CTA = 32 fibers (one warp) on one OS thread, __syncthreads and warp
// shuffles are real barriers that also check that all threads reached the
// same call site, atomics are std::atomic_ref.  Used by the host test harness
// (emu_check.cpp) to execute the unmodified device functions under
// AddressSanitizer / UndefinedBehaviorSanitizer, so that out-of-bounds
// accesses in the device logic show up on the CPU.
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
struct EmuDim { unsigned x = 0, y = 0, z = 0; };

namespace emu {
constexpr int kLanes = 32;
// One CTA = 32 fibers on the calling OS thread; a barrier switches back to
// the scheduler, which resumes the fibers once all of them have arrived.
struct Cta {
    ucontext_t sched;
    ucontext_t fib[kLanes];
    std::vector<char> stack[kLanes];
    bool arrived[kLanes];
    bool finished[kLanes];
    int cur = 0;
    uint64_t xchg[kLanes];
    std::atomic<int> any{0};
    int site[kLanes];          // call site of each thread's current barrier
    int mismatches = 0;
    long long barriers = 0;
};
inline Cta*& cta() { static Cta* c = nullptr; return c; }
inline EmuDim tid;
}  // namespace emu

static const EmuDim blockDim{32, 1, 1};
static const EmuDim blockIdx{0, 0, 0};
static const EmuDim gridDim{1, 1, 1};
#define threadIdx (emu::tid)

namespace emu {
// Every barrier (including the ones inside emulated shuffles) records its call
// site; threads meeting at one barrier phase from different sites means a
// __syncthreads() was reached divergently.
inline void sync_at(int line) {
    Cta* c = cta();
    const int me = c->cur;
    c->site[me] = line;
    c->arrived[me] = true;
    swapcontext(&c->fib[me], &c->sched);
    tid.x = (unsigned)me;
}
}  // namespace emu
#define __syncthreads() emu::sync_at(__LINE__)
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

template <class T>
inline T emu_shfl(T v, int src_lane) {
    emu::Cta* c = emu::cta();
    uint64_t bits = 0;
    memcpy(&bits, &v, sizeof(T));
    emu::sync_at(-1);
    c->xchg[threadIdx.x] = bits;
    emu::sync_at(-2);
    uint64_t got = c->xchg[src_lane];
    emu::sync_at(-3);
    T out;
    memcpy(&out, &got, sizeof(T));
    return out;
}
template <class T> inline T __shfl_xor_sync(unsigned, T v, int o) { return emu_shfl(v, (int)(threadIdx.x ^ o)); }
template <class T> inline T __shfl_up_sync(unsigned, T v, int o) {
    const int src = (int)threadIdx.x - o;
    T got = emu_shfl(v, src < 0 ? (int)threadIdx.x : src);
    return got;
}

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
// Run f() on one emulated CTA of 32 threads.  Returns the number of barrier
// phases whose threads arrived from different call sites (0 when every
// __syncthreads() is reached uniformly), or -1 on a deadlock.
inline int run_cta(const std::function<void()>& f) {
    Cta* c = new Cta();
    cta() = c;
    entry() = &f;
    for (int t = 0; t < kLanes; t++) {
        c->stack[t].resize(1 << 17);
        getcontext(&c->fib[t]);
        c->fib[t].uc_stack.ss_sp = c->stack[t].data();
        c->fib[t].uc_stack.ss_size = c->stack[t].size();
        c->fib[t].uc_link = nullptr;
        makecontext(&c->fib[t], (void (*)())fiber_main, 0);
        c->arrived[t] = false;
        c->finished[t] = false;
    }
    int result = 0;
    for (;;) {
        for (int t = 0; t < kLanes; t++) {
            if (c->finished[t] || c->arrived[t]) continue;
            c->cur = t;
            swapcontext(&c->sched, &c->fib[t]);
        }
        int nfin = 0, narr = 0;
        for (int t = 0; t < kLanes; t++) { nfin += c->finished[t]; narr += c->arrived[t]; }
        if (nfin == kLanes) break;
        if (nfin > 0) { result = -1; fprintf(stderr, "deadlock: %d threads finished, %d at a barrier\n", nfin, narr); break; }
        c->barriers++;
        for (int t = 1; t < kLanes; t++)
            if (c->site[t] != c->site[0]) {
                if (c->mismatches++ < 5)
                    fprintf(stderr, "barrier mismatch: thread 0 at line %d, thread %d at line %d\n", c->site[0], t, c->site[t]);
                break;
            }
        for (int t = 0; t < kLanes; t++) c->arrived[t] = false;
    }
    if (result == 0) result = c->mismatches;
    cta() = nullptr;
    delete c;
    return result;
}
}  // namespace emu
