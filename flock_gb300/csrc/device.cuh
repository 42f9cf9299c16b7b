// device.cuh -- CTA-level building blocks of the transportation simplex.
//
// Every function here is executed by ALL threads of one CTA (block-uniform
// control flow; they synchronise internally).  The same functions serve the
// plain single-instance path (one CTA for the tree phases, a grid-wide sweep)
// and the batched persistent kernel (one CTA per instance, work stealing).
// Arrays are reached through generic pointers so one code path serves both
// placements: shared memory for small instances, global memory otherwise.
//
// Vertex numbering: rows (supplies) 0..m-1, columns (demands) m..m+n-1.
// Tree edges are identified by their child vertex; the edge of a row child
// r with parent column p is cell (r, p-m); of a column child c with parent
// row p, cell (p, c-m).  Arc direction is always row -> column.
#pragma once
#include <climits>
#include <cstdint>
#ifdef FLOCK_EMU
#include "emu/cuda_emu.h"   // host emulation for sanitizer runs of the device code
#else
#include <cuda_runtime.h>
#endif

namespace flock {

// ---------------------------------------------------------------- status ---
enum : int32_t {
    ST_ITER_CAP = 1,          // pricing-round cap reached before optimality
    ST_TREE_CORRUPT = 2,      // a tree walk or the dual recompute did not terminate
    ST_SF_FAIL = 4,           // perturbed initial flow not positive (internal)
    ST_VOGEL_UNDEF = 8,       // Vogel hit the reference's out-of-range index case
    ST_START_REPAIRED = 16,   // Vogel flows not a feasible forest: simplex starts from NW corner
    ST_CERT_FAIL = 32,        // certificate check failed
    ST_RANGE = 64,            // perturbed flows would overflow int64
};

constexpr int64_t kDeadPot = -(int64_t(1) << 61);   // dual of a zero-demand column during pivoting
// int32 column duals for the sweep: live duals must lie strictly inside
// (kDead32, -kDead32) so that c - v fits int32 for |c| <= 2^30; a dead
// (zero-demand) column is stored as kDead32 and re-checked exactly.
constexpr int32_t kDead32 = -((1 << 30) - 1);
constexpr uint64_t kNoKey = ~0ull;
// Vertices a thread handles at once in the pointer-jumping and
// k-th-ancestor passes (loads of independent vertices interleaved): the
// default of the batched kernels (64 registers) and the plain solver's.
constexpr int kJump = 2;
constexpr int kJumpPlain = 4;
constexpr int kPPRows = 128;     // partial pricing: capacity of the candidate-row list
// Partial pricing settings (Scalars::pp_rows / pp_refresh): candidate rows
// kept by a full sweep and rounds between full sweeps.  Instances of up to
// kPPSmallV vertices (a full sweep is cheap next to a round's fixed cost)
// gain from frequent full sweeps and short lists; larger ones, where a full
// sweep streams a matrix of millions of cells, from longer intervals.
constexpr int kPPSmallV = 1024;
constexpr int kPPRowsSmall = 32, kPPRefreshSmall = 8;
constexpr int kPPRowsLarge = 64, kPPRefreshLarge = 32;
// The plain solver's grid path (2400 vertices and more), whose candidate
// rounds run inside one thread-block cluster: a longer candidate list picks
// better entering cells (fewer pivots) and costs little there (8000 x 8000
// Euclidean: 57,815 pivots in 1.50 s with 64 rows / 32 rounds, 53,784 in
// 1.43 s with 128 / 32, 1.42 s with 128 / 64).
constexpr int kPPRowsGrid = 128, kPPRefreshGrid = 64;

struct Scalars {
    int32_t status;
    int32_t done;          // 1: optimal or stopped; later kernels return at once
    int32_t rounds;        // pricing rounds (full sweeps)
    int32_t pivots;        // pivots applied
    int32_t root;          // root column vertex
    int32_t v_alive;       // vertices in the pivoting tree
    int32_t events;        // Vogel events (see vogel_cta), -1: undefined case
    int32_t active;        // nonzero flows in the result
    int32_t cert;          // certificate failure bits (0: optimal)
    int32_t max_rounds;
    int32_t mode;          // 0 sequential (one pivot / round), 1 parallel multi-pivot, 2 switch (parallel, then 0)
    int32_t ncand;         // candidates in the last round
    int64_t objective;
    int64_t M;             // perturbation scale
    int64_t neg_cells;     // certificate: cells with negative reduced cost
    int64_t cells;         // cost cells priced by the CTA sweeps (all rounds)
    int32_t last_winners;
    int32_t fail_site;     // first failed internal check (0: none), see fail_check
    int32_t narrow;        // 1: every live column dual fits the int32 sweep (v32 valid)
    int32_t pricing;       // 0 full sweeps, 1 partial pricing (candidate rows)
    int32_t pp_n;          // partial pricing: candidate rows in prow[]
    int32_t pp_age;        // partial pricing: rounds since the last full sweep
    int32_t pp_rows;       // partial pricing: candidate rows kept by a full sweep (1..kPPRows)
    int32_t pp_refresh;    // partial pricing: rounds between full sweeps (>= 1)
    int32_t ivp;           // which half of Ctx::iv holds the current preorder intervals
    int32_t nwide;         // live column duals outside the int32 window (narrow == (nwide == 0))
    int32_t stale;         // 1: depth, duals and intervals must be rebuilt from parent[] (tree_build_cta)
    int32_t pad_;
};

// Phase clock of the plain solver: device time per phase of the simplex,
// the reference's model statistics (uv_model_parallel.cu:301-341, the
// PivotTimer of parallel_structs.h:244-247): duals (a rebuild of the tree's
// derived state), reduced costs (the sweeps and the choice of the entering
// cells), cycle discovery, resolve (deconfliction of parallel candidates)
// and adjustment (leaving edge, flow change, in-place update of the tree).
// Every segment runs from one mark to the next, marks read %globaltimer, and
// a kernel's first segment starts at its first block's start, so the phases
// add up to the loop's device time (launch gaps included in the phase before
// them).  Kernels that find the solve finished count as idle.
enum : int32_t { PH_BFS = 0, PH_DUAL, PH_SWEEP, PH_CYCLE, PH_RESOLVE, PH_ADJUST, PH_IDLE, kPhases };
struct __align__(16) PhaseClock {
    uint64_t last;          // globaltimer at the start of the running segment (0: none yet)
    int32_t cur;            // phase of the running segment
    int32_t pad_;
    uint64_t ns[kPhases];   // accumulated nanoseconds per phase
};

__device__ __forceinline__ uint64_t global_ns() {
#ifdef FLOCK_EMU
    return 0;
#else
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
#endif
}

// Shared-memory state of one launch's phase accounting (block 0 only).  Its
// first 16 bytes are the destination of a 16-byte cp.async, which needs a
// 16-byte aligned shared address.
struct __align__(16) PhaseLocal {
    uint64_t prev_last;     // the clock's `last` and `cur` as the previous launch left them
    int32_t prev_cur, pad_;
    uint64_t t0, t;         // this launch's start, start of its running segment
    PhaseClock* clk;        // null: no accounting in this launch
    int32_t cur, pad2_;
};

// The phase accounting of one kernel launch, kept by thread 0 of block 0;
// mark() may be called by every thread at block-uniform points (after a
// barrier).  The state lives in shared memory (nothing held in registers
// across the kernel) and the previous launch's values arrive by an
// asynchronous copy (no wait on a global load).  At scope exit, early returns
// included, it closes the previous launch's last segment at this launch's
// start and leaves its own last segment running for the next launch.
struct PhaseScope {
    PhaseLocal* s;
    __device__ __forceinline__ static bool leader() { return blockIdx.x == 0 && threadIdx.x == 0; }
    __device__ __forceinline__ PhaseScope(PhaseClock* p, PhaseLocal* sl, int phase) : s(sl) {
        if (!leader()) return;
        s->clk = p;
        if (!p) return;
#ifdef FLOCK_EMU
        s->prev_last = p->last;
        s->prev_cur = p->cur;
#else
        const unsigned dst = (unsigned)__cvta_generic_to_shared(s);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n\tcp.async.commit_group;"
                     :: "r"(dst), "l"(p) : "memory");
#endif
        s->t0 = s->t = global_ns();
        s->cur = phase;
    }
    __device__ __forceinline__ void mark(int next) {
        if (!leader() || !s->clk) return;
        const uint64_t now = global_ns();
        atomicAdd((unsigned long long*)&s->clk->ns[s->cur], (unsigned long long)(now - s->t));
        s->t = now;
        s->cur = next;
    }
    // The solve was already finished: this launch counts as idle.
    __device__ __forceinline__ void idle() {
        if (leader() && s->clk) s->cur = PH_IDLE;
    }
    __device__ __forceinline__ ~PhaseScope() {
        if (leader()) close(s);
    }
    // Out of line: the hot kernels keep their registers for their own work.
    __device__ __noinline__ static void close(PhaseLocal* s) {
        PhaseClock* ph = s->clk;
        if (!ph) return;
#ifndef FLOCK_EMU
        asm volatile("cp.async.wait_all;" ::: "memory");
#endif
        const uint64_t pl = s->prev_last, t0 = s->t0;
        const int pc = s->prev_cur;
        if (pl && (unsigned)pc < (unsigned)kPhases && t0 > pl)
            atomicAdd((unsigned long long*)&ph->ns[pc], (unsigned long long)(t0 - pl));
        ph->last = s->t;
        ph->cur = s->cur;
    }
};

// One instance as the kernels see it.
struct InstDev {
    int32_t m, n, ldc;        // rows, columns, padded row pitch (multiple of 4)
    const int32_t* cost;      // m x ldc, row-major
    const int32_t* supply;    // m
    const int32_t* demand;    // n
    // the grid path's 16-bit copy of the costs when every cost fits (m x
    // ldc16, ldc16 a multiple of 8), read by its full and candidate sweeps;
    // null otherwise
    const int16_t* cost16 = nullptr;
    int32_t ldc16 = 0;
};

// Per-instance working set.  Pointers may refer to shared or global memory.
struct Ctx {
    InstDev I;
    Scalars* sc;
    // allocation list of the initial solution (Vogel or NW corner), V-1
    int32_t* bfs_src; int32_t* bfs_dst; int32_t* bfs_qty;
    // final basis, V-1 cells with original quantities
    int32_t* out_src; int32_t* out_dst; int32_t* out_qty;
    // tree
    int32_t* parent;   // V  (-1 root, -2 not in tree)
    int64_t* flow;     // V  perturbed flow on the edge to the parent
    int32_t* depth;    // V
    int64_t* pot;      // V  duals: u_i (rows), v_j (columns)
    int32_t* v32;      // n  column duals as int32 when sc->narrow (kDead32: zero-demand column)
    // Preorder intervals, two buffers of V (sc->ivp selects the current one):
    // iv[v] = (pre, size) with the subtree of tree vertex v holding exactly
    // the vertices x with pre[v] <= pre[x] < pre[v] + size[v].  Dead vertices
    // hold (0, 0).
    int2* iv;
    // pointer-jumping scratch, one block of jump_bytes(V) (set_jump): int32
    // anc0, anc1, len0, len1 then int64 acc0, acc1; the Euler-tour ranking
    // uses the same block as two arrays of 2 V words.
    int32_t* anc0; int32_t* anc1; int32_t* len0; int32_t* len1; int64_t* acc0; int64_t* acc1;
    // single pivot scratch: cycle side of each vertex, the re-hung path by
    // index and its updated flows (V each; may alias len1 / acc1, which only
    // the rebuilds use)
    uint8_t* side;
    int32_t* path;
    int64_t* pflow;
    // pricing
    uint64_t* row_best;   // m   packed (reduced cost, column) of the best cell per row
    uint64_t* claim;      // V   edge claims
    int32_t* cand;        // m   candidate rows
    int64_t* cand_theta;  // m
    int32_t* cand_q;      // m   leaving edge (child vertex)
    int32_t* cand_info;   // m   bit0: leaving edge on the column side; bit1: winner
    // Vogel scratch
    uint8_t* covered;     // V
    int32_t* diff;        // V
    int32_t* res;         // V  residual supply (rows) / demand (columns)
    int4* top2;           // V  (c1, c2, j1, j2) two cheapest uncovered crossing cells
    int32_t* rescan;      // V  list of lines whose top2 must be rebuilt
    int32_t* prow;        // kPPRows  partial pricing: candidate rows
    // start-tree scratch
    int64_t* bsum;        // V
    int32_t* csr_start;   // V+1
    int32_t* csr_adj;     // 2V
    int32_t* order;       // V  (BFS order of the start tree)
    int32_t* uf;          // V  union-find
    // phase clock of the plain solver (null elsewhere; see PhaseClock)
    PhaseClock* ph;
};

// Size of the pointer-jumping scratch block of V vertices.
__host__ __device__ __forceinline__ size_t jump_bytes(int V) { return 32 * (size_t)V; }

// Point the six pointer-jumping arrays into one block of jump_bytes(V)
// (16-byte aligned).
__host__ __device__ __forceinline__ void set_jump(Ctx& c, void* base, int V) {
    int32_t* b = (int32_t*)base;
    c.anc0 = b; c.anc1 = b + V; c.len0 = b + 2 * (size_t)V; c.len1 = b + 3 * (size_t)V;
    c.acc0 = (int64_t*)(b + 4 * (size_t)V);
    c.acc1 = c.acc0 + V;
}

// x lies in the subtree whose interval is w (x's preorder number px).
__device__ __forceinline__ bool iv_in(int2 w, int px) { return (unsigned)(px - w.x) < (unsigned)w.y; }

// --------------------------------------------------------------- helpers ---
// A column dual as the int32 sweep sees it; sets `wide` when it does not fit.
__device__ __forceinline__ int32_t narrow_dual(int64_t p, int& wide) {
    if (p == kDeadPot) return kDead32;
    if (p > kDead32 && p < -(int64_t)kDead32) return (int32_t)p;
    wide = 1;
    return 0;
}

#define FLOCK_IN(x, V) ((unsigned)(x) < (unsigned)(V))

// An internal index check failed: record the first failing site, mark the
// solve corrupt and stop it.  The caller skips the access.
__device__ __forceinline__ void fail_check(Scalars* sc, int site) {
    atomicCAS(&sc->fail_site, 0, site);
    atomicOr(&sc->status, ST_TREE_CORRUPT);
    atomicExch(&sc->done, 1);
}

__device__ __forceinline__ int32_t f2i_x86(float f) {
    // float -> int as x86 cvttss2si: truncation, INT_MIN for NaN/out of range.
    if (!(f < 2147483648.0f) || !(f >= -2147483648.0f)) return INT32_MIN;
    return __float2int_rz(f);
}

// Packed (value, index) keys: unsigned order == (value, index) order.
__device__ __forceinline__ uint64_t pack_i32(int32_t v, uint32_t idx) {
    return ((uint64_t)((uint32_t)v ^ 0x80000000u) << 32) | idx;
}
__device__ __forceinline__ int32_t key_val(uint64_t k) { return (int32_t)((uint32_t)(k >> 32) ^ 0x80000000u); }
__device__ __forceinline__ uint32_t key_idx(uint64_t k) { return (uint32_t)k; }
__device__ __forceinline__ int32_t clamp32(int64_t r) {
    return r < INT32_MIN ? INT32_MIN : (r > INT32_MAX ? INT32_MAX : (int32_t)r);
}

// Warp minimum / maximum of 64-bit unsigned keys, exact, with the hardware
// 32-bit warp reductions: the high words first, then the low words among the
// lanes holding the winning high word.
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
    const unsigned hi = __reduce_min_sync(0xffffffffu, (unsigned)(v >> 32));
    const unsigned lo = __reduce_min_sync(0xffffffffu, (unsigned)(v >> 32) == hi ? (unsigned)v : 0xffffffffu);
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ uint64_t warp_max_u64(uint64_t v) {
    const unsigned hi = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32));
    const unsigned lo = __reduce_max_sync(0xffffffffu, (unsigned)(v >> 32) == hi ? (unsigned)v : 0u);
    return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ int64_t warp_sum_i64(int64_t v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Shared scratch for block reductions (one slot per warp, at most 32 warps).
struct BlockScratch {
    uint64_t red[32];
    uint64_t red2[32];
    uint64_t red3[32];
    uint64_t red4[32];
    uint64_t part1[32], part2[32];   // per-warp partial results (Vogel's split rescans)
    int32_t i[12];
};

// Block reductions: warp results in shared memory, then every warp reduces
// them itself (no broadcast barrier).  The leading barrier keeps the previous
// reduction's readers ahead of this one's writes.
__device__ __forceinline__ uint64_t block_min_u64(uint64_t v, BlockScratch& bs) {
    v = warp_min_u64(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) bs.red[w] = v;
    __syncthreads();
    return warp_min_u64(l < nw ? bs.red[l] : kNoKey);
}
__device__ __forceinline__ uint64_t block_max_u64(uint64_t v, BlockScratch& bs) {
    v = warp_max_u64(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) bs.red[w] = v;
    __syncthreads();
    return warp_max_u64(l < nw ? bs.red[l] : 0ull);
}
__device__ __forceinline__ int64_t block_sum_i64(int64_t v, BlockScratch& bs) {
    v = warp_sum_i64(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) bs.red[w] = (uint64_t)v;
    __syncthreads();
    if (w == 0) {
        int64_t x = l < nw ? (int64_t)bs.red[l] : 0;
        x = warp_sum_i64(x);
        if (l == 0) bs.red[0] = (uint64_t)x;
    }
    __syncthreads();
    return (int64_t)bs.red[0];
}

// Two independent lexicographic minima of (a, b) and (c, d) pairs over the
// block, in one pass of barriers; every thread gets both results.
__device__ __forceinline__ void pair_min_into(uint64_t& a, uint64_t& b, uint64_t c, uint64_t d) {
    if (c < a || (c == a && d < b)) { a = c; b = d; }
}
// Warp lexicographic minimum of (a, b), exact, in four 32-bit warp
// reductions (a's words, then b's among the lanes holding the minimal a).
__device__ __forceinline__ void warp_min_pair(uint64_t& a, uint64_t& b) {
    const unsigned ah = __reduce_min_sync(0xffffffffu, (unsigned)(a >> 32));
    const unsigned al = __reduce_min_sync(0xffffffffu, (unsigned)(a >> 32) == ah ? (unsigned)a : 0xffffffffu);
    const uint64_t amin = ((uint64_t)ah << 32) | al;
    const bool at = a == amin;
    const unsigned bh = __reduce_min_sync(0xffffffffu, at ? (unsigned)(b >> 32) : 0xffffffffu);
    const unsigned bl = __reduce_min_sync(0xffffffffu, at && (unsigned)(b >> 32) == bh ? (unsigned)b : 0xffffffffu);
    a = amin;
    b = ((uint64_t)bh << 32) | bl;
}
__device__ __forceinline__ void warp_min_pairs(uint64_t& a, uint64_t& b, uint64_t& c, uint64_t& d) {
    warp_min_pair(a, b);
    warp_min_pair(c, d);
}
__device__ __forceinline__ void block_min_pairs(uint64_t& a, uint64_t& b, uint64_t& c, uint64_t& d, BlockScratch& bs) {
    warp_min_pairs(a, b, c, d);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) { bs.red[w] = a; bs.red2[w] = b; bs.red3[w] = c; bs.red4[w] = d; }
    __syncthreads();
    a = b = c = d = kNoKey;
    if (l < nw) { a = bs.red[l]; b = bs.red2[l]; c = bs.red3[l]; d = bs.red4[l]; }
    warp_min_pairs(a, b, c, d);
}

// Two smallest keys: insert / merge.
__device__ __forceinline__ void top2_insert(uint64_t& a1, uint64_t& a2, uint64_t k) {
    if (k < a1) { a2 = a1; a1 = k; } else if (k < a2) { a2 = k; }
}
__device__ __forceinline__ void top2_merge(uint64_t& a1, uint64_t& a2, uint64_t b1, uint64_t b2) {
    uint64_t f, s;
    if (a1 < b1) { f = a1; s = a2 < b1 ? a2 : b1; }
    else         { f = b1; s = a1 < b2 ? a1 : b2; }
    a1 = f; a2 = s;
}
// Every lane ends with the warp's two smallest keys.  Keys other than kNoKey
// are distinct (they carry their index), so the second is the smallest of
// every lane's first key, except that the lane holding the overall first
// offers its second instead.
__device__ __forceinline__ void warp_top2(uint64_t& a1, uint64_t& a2) {
    const uint64_t m1 = warp_min_u64(a1);
    const uint64_t m2 = warp_min_u64(a1 == m1 ? a2 : a1);
    a1 = m1;
    a2 = m2;
}

__device__ __forceinline__ int32_t cost_of(const InstDev& I, int row, int col) {
    return I.cost[(size_t)row * I.ldc + col];
}
// cost of the tree edge whose child is v with parent p
__device__ __forceinline__ int32_t edge_cost(const InstDev& I, int v, int p) {
    return v < I.m ? cost_of(I, v, p - I.m) : cost_of(I, p, v - I.m);
}

}  // namespace flock
