// internal.h -- layout of the per-instance working set and the batched-kernel
// arguments, shared by host and device code.
#pragma once
#include <cstddef>
#include <cstdint>

#include "device.cuh"

namespace flock {

// One instance of a batched or served launch, by absolute device pointers.
struct BatchDesc {
    int32_t m, n, ldc, index;   // index: position in the caller's instance list
    const int32_t* cost;        // m x ldc, 16-byte aligned
    const int32_t* sd;          // supplies (m) then demands (n)
    uint8_t* ws;                // working set (carve_ctx layout), 256-byte aligned
    int32_t* out;               // basis: src[V-1], dst[V-1], qty[V-1]
    int32_t* bfs;               // initial allocation list: 3 ints per cell, V-1 cells
    int64_t* pot;               // duals, V
    Scalars* sc;
    int32_t* done;              // optional completion flag in host-mapped memory
};

struct BatchArgs {
    const BatchDesc* desc;
    int32_t count;
    int32_t* next;              // work-stealing counter of this launch (zeroed before it)
    int32_t* active;            // round kernel: instances still running after the round
    int32_t maxV, maxM;         // largest instance of the launch (shared-memory staging size)
    int32_t bfs_method, mode, max_rounds;
    int32_t light;              // 1: stage only the per-step tree arrays (largest buckets)
    int32_t pricing;            // Scalars::pricing of every instance
    PhaseClock* ph;             // phase clock (the plain solver's one-launch form only; null otherwise)
    // partial pricing per instance: candidate rows and rounds between full
    // sweeps up to kPPSmallV vertices ([0], [1]) and above ([2], [3])
    int32_t pp[4];
    // one-launch form: byte offset in the dynamic shared block where the
    // instance's cost matrix is staged (0: the kernels read it from global
    // memory)
    int32_t cost_smem;
};

// A served request's device region: byte offsets of its arrays (256-aligned).
struct ServeLayout { size_t cost, sd, ws, out, bfs, pot, sc, total; };

struct Carver {
    uint8_t* g; size_t go;
    unsigned char* s; size_t so;
    __host__ __device__ void* G(size_t bytes) {
        go = (go + 255) & ~size_t(255);
        void* p = g ? (void*)(g + go) : nullptr;
        go += bytes;
        return p;
    }
    __host__ __device__ void* S(size_t bytes) {
        if (!s) return G(bytes);
        so = (so + 15) & ~size_t(15);
        void* p = (void*)(s + so);
        so += bytes;
        return p;
    }
};

// Assign every working array of `c` for instances with at most V vertices and
// M rows.  With `smem` the arrays touched by every pivot step live in shared
// memory, the rest in the global region `g`.  Returns the bytes used in both.
__host__ __device__ inline void carve_ctx(Ctx& c, uint8_t* g, int V, int M, unsigned char* smem,
                                          int64_t* pot_global, size_t* smem_bytes = nullptr,
                                          size_t* global_bytes = nullptr) {
    Carver k{g, 0, smem, 0};
    const size_t v = (size_t)V, mm = (size_t)M;
    c.parent = (int32_t*)k.S(4 * v);
    c.depth = (int32_t*)k.S(4 * v);
    c.flow = (int64_t*)k.S(8 * v);
    c.claim = (uint64_t*)k.S(8 * v);
    set_jump(c, k.S(jump_bytes(V)), V);
    c.path = c.len1;
    c.pflow = c.acc1;
    c.side = (uint8_t*)k.S(v);
    c.iv = (int2*)k.S(16 * v);
    c.row_best = (uint64_t*)k.S(8 * mm);
    c.pot = smem ? (int64_t*)k.S(8 * v) : (pot_global ? pot_global : (int64_t*)k.G(8 * v));
    c.v32 = (int32_t*)k.S(4 * v);
    c.bfs_src = (int32_t*)k.G(4 * v);
    c.bfs_dst = (int32_t*)k.G(4 * v);
    c.bfs_qty = (int32_t*)k.G(4 * v);
    c.cand = (int32_t*)k.G(4 * mm);
    c.cand_theta = (int64_t*)k.G(8 * mm);
    c.cand_q = (int32_t*)k.G(4 * mm);
    c.cand_info = (int32_t*)k.G(4 * mm);
    c.covered = (uint8_t*)k.G(v);
    c.diff = (int32_t*)k.G(4 * v);
    c.res = (int32_t*)k.G(4 * v);
    c.top2 = (int4*)k.G(16 * v);
    c.rescan = (int32_t*)k.G(4 * v);
    c.prow = (int32_t*)k.G(4 * (size_t)kPPRows);
    c.bsum = (int64_t*)k.G(8 * v);
    c.csr_start = (int32_t*)k.G(4 * (v + 1));
    c.csr_adj = (int32_t*)k.G(8 * v);
    c.order = (int32_t*)k.G(4 * v);
    c.uf = (int32_t*)k.G(4 * v);
    c.ph = nullptr;
    if (smem_bytes) *smem_bytes = k.so;
    if (global_bytes) *global_bytes = (k.go + 255) & ~size_t(255);
}

}  // namespace flock
