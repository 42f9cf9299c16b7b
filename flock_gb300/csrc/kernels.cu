// kernels.cu -- device kernels and host orchestration of the plain and the
// batched solver, plus their C-ABI entry points (include/flock.h).
//
// Plain path (one instance, any size):
//   k_setup   <<<1 CTA>>>   Vogel (or NW corner), strongly feasible start tree, duals
//   loop in chunks captured as a CUDA graph:
//     k_sweep <<<grid>>>    fused reduced-cost sweep: int4 rows, duals of a column
//                           tile staged in shared memory, per-row best (r, j) key
//     k_pivot <<<1 CTA>>>   candidates, cycle walks, atomicMin claims, apply, duals
//   k_finalize<<<1 CTA>>>   original flows, zero-demand columns, objective, flow certificate
//   k_cert_cells<<<grid>>>  certificate: every reduced cost >= 0
// Batched path: per size bucket, k_bsetup, then chunks of k_bround (one
// pricing round of every active instance, work stealing, tree staged in
// shared memory) captured as CUDA graphs, then k_bfinal; buckets run
// concurrently on their own streams.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/flock.h"
#include "simplex.cuh"
#include "internal.h"

namespace flock {

// ------------------------------------------------------------ kernels ------
// Vogel's per-line state (diff, res, rescan list, covered: V * 13 bytes) in
// the launch's dynamic shared memory when the host gives it room: every
// refresh reads it several times per line.  The top-2 caches stay in the
// working set.
constexpr size_t kVogelStageMax = 200 * 1024;
__host__ __device__ inline size_t vogel_stage_bytes(int V) {
    return 3 * (((size_t)V * 4 + 15) & ~size_t(15)) + (((size_t)V + 15) & ~size_t(15));
}
__device__ __forceinline__ void vogel_stage(Ctx& c, unsigned char* smem, int V) {
    const size_t w = ((size_t)V * 4 + 15) & ~size_t(15);
    c.diff = reinterpret_cast<int32_t*>(smem);
    c.res = reinterpret_cast<int32_t*>(smem + w);
    c.rescan = reinterpret_cast<int32_t*>(smem + 2 * w);
    c.covered = reinterpret_cast<uint8_t*>(smem + 3 * w);
}

// Column-major copy of the cost matrix for Vogel's column scans:
// costT[j * ldcT + i] = cost[i * ldc + j], through a 32 x 33 shared tile.
__global__ void __launch_bounds__(256) k_transpose(const int32_t* cost, int m, int n, int ldc, int32_t* costT,
                                                   int ldcT) {
    __shared__ int32_t tile[32][33];
    const int j0 = blockIdx.x * 32, i0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int i = i0 + k, j = j0 + threadIdx.x;
        if (i < m && j < n) tile[k][threadIdx.x] = cost[(size_t)i * ldc + j];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int j = j0 + k, i = i0 + threadIdx.x;
        if (j < n && i < m) costT[(size_t)j * ldcT + i] = tile[threadIdx.x][k];
    }
}

// 16-bit copy of the costs (every cost fits): cost16[i * ldc16 + j], the
// padding columns zero.
__global__ void __launch_bounds__(256) k_cost16(const int32_t* cost, int m, int n, int ldc, int16_t* cost16,
                                                int ldc16) {
    const size_t cells = (size_t)m * ldc16;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < cells; k += (size_t)gridDim.x * blockDim.x) {
        const size_t i = k / ldc16, j = k % ldc16;
        cost16[k] = j < (size_t)n ? (int16_t)cost[i * ldc + j] : (int16_t)0;
    }
}

// costT: the column-major copy (null: columns are read from the rows);
// stage: the dynamic block holds vogel_stage_bytes(V).
__global__ void __launch_bounds__(1024, 1) k_setup(Ctx c, int bfs_method, const int2* rbook, const int2* cbook,
                                                   const int32_t* costT, int stage) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    extern __shared__ __align__(16) unsigned char su_smem[];
    PhaseScope ps(c.ph, &phl, PH_BFS);
    if (bfs_method == FLOCK_BFS_VOGEL) {
        Ctx cv = c;
        if (stage) vogel_stage(cv, su_smem, c.I.m + c.I.n);
        vogel_cta<true>(cv, bs, costT);
    } else if (bfs_method == FLOCK_BFS_VOGEL_DEVICE) {
        vogel_books_cta(c, rbook, cbook, bs);
    } else {
        if (threadIdx.x == 0) { nwc_thread0(c); c.sc->events = 0; }
        __syncthreads();
    }
    if (threadIdx.x == 0 && c.sc->events < 0) c.sc->status |= ST_VOGEL_UNDEF;
    ps.mark(PH_DUAL);    // the start tree and its duals
    sf_init_cta(c, bs);
    if (!c.sc->done) tree_build_cta<kJumpPlain>(c, bs);
    for (int i = threadIdx.x; i < c.I.m; i += blockDim.x) c.row_best[i] = kNoKey;
    __syncthreads();
    ps.mark(PH_SWEEP);   // the first round's sweep
}

__global__ void __launch_bounds__(1024, 1) k_vogel_only(Ctx c, const int32_t* costT, int stage) {
    __shared__ BlockScratch bs;
    extern __shared__ __align__(16) unsigned char vo_smem[];
    Ctx cv = c;
    if (stage) vogel_stage(cv, vo_smem, c.I.m + c.I.n);
    vogel_cta<true>(cv, bs, costT);
}

// "vam_device" Vogel: the books (one block per line: rows, then columns),
// then the step loop on one CTA.
constexpr int kBookThreads = 256;
constexpr int kBookLineMax = 16382;     // a line's book (+ 2 sentinels) sorts in 128 KB of shared memory
__global__ void __launch_bounds__(kBookThreads) k_books(InstDev I, int2* rbook, int2* cbook, int P) {
    extern __shared__ uint64_t book_keys[];
    const int line = blockIdx.x;
    int2* out = line < I.m ? rbook + (size_t)line * (I.n + 2) : cbook + (size_t)(line - I.m) * (I.m + 2);
    book_line_cta(I, line, book_keys, P, out);
}

__global__ void __launch_bounds__(1024, 1) k_vogel_books_only(Ctx c, const int2* rbook, const int2* cbook) {
    __shared__ BlockScratch bs;
    vogel_books_cta(c, rbook, cbook, bs);
}

// Grid-wide sweep.  blockIdx.x = tile + ntile * row_group.  The block stages
// the int32 column duals of its tile (narrow form) in shared memory; a warp
// work unit is one row segment of kSegCols columns, read as 16-byte vectors
// that bypass L1 (each cost element is used once per sweep), eight per lane
// in flight.  Units combine into row_best[] with atomicMin, so row_best must
// hold kNoKey before the sweep (k_setup and k_pivot leave it so).
constexpr int kSweepTile = 8192;   // columns per block tile (32 KB of int32 duals)
constexpr int kSegCols = 1024;     // columns per warp work unit
constexpr int kSweepThreads = 512;

__device__ __forceinline__ int4 ld_stream4(const int4* p) {
    int4 v;
    asm("ld.global.nc.L1::no_allocate.v4.s32 {%0, %1, %2, %3}, [%4];"
        : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}

// One grid-wide sweep's share of block `bid` of `nb` (nb a multiple of
// ntile): its column tile's int32 duals staged in vt, then (row, segment)
// units.  rows: price only the listed rows (c.sc->pp_n of them: partial
// pricing), null for all.  The caller orders vt's previous readers.
// Block-wide copy of ceil4(jn) int32 values from global into shared memory:
// 16-byte loads, four per thread issued before any store (one L2 round trip
// for a 512-thread block and an 8192-column tile of duals).  src and vt are
// 16-byte aligned; for a dual tile (tiles start at multiples of 4 columns)
// the rounded-up tail stays inside the dual array's allocation and is never
// read.
__device__ __forceinline__ void stage_i32(int32_t* vt, const int32_t* src, int jn) {
    const int nq = (jn + 3) >> 2, bd = (int)blockDim.x;
    const int4* s4 = reinterpret_cast<const int4*>(src);
    int4* d4 = reinterpret_cast<int4*>(vt);
    for (int q = threadIdx.x; q < nq; q += 4 * bd) {
        int4 x[4];
        #pragma unroll
        for (int k = 0; k < 4; k++)
            if (q + k * bd < nq) x[k] = __ldcg(s4 + q + k * bd);
        #pragma unroll
        for (int k = 0; k < 4; k++)
            if (q + k * bd < nq) d4[q + k * bd] = x[k];
    }
}

__device__ __forceinline__ void sweep_part(const Ctx& c, int tile, int ntile, const int32_t* rows, int32_t* vt,
                                           int bid, int nb) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n;
    const int t = bid % ntile, rg = bid / ntile, nrg = nb / ntile;
    const int j0 = t * tile;
    const int jn = min(tile, n - j0);
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const int nseg = (jn + kSegCols - 1) / kSegCols;
    const int nrows = rows ? min(max(c.sc->pp_n, 0), kPPRows) : m;
    const long long units = (long long)nrows * nseg, stride = (long long)nrg * wpb;
    if ((long long)rg * wpb >= units) return;      // no unit for this block (a candidate sweep uses few blocks)
    if (!c.sc->narrow) {
        for (long long u = (long long)rg * wpb + warp; u < units; u += stride) {
            const int i = rows ? rows[u / nseg] : (int)(u / nseg), s = (int)(u % nseg);
            if (!FLOCK_IN(i, m)) { if (lane == 0) fail_check(c.sc, 19); continue; }
            const int a = j0 + s * kSegCols, b = min(j0 + jn, a + kSegCols);
            const uint64_t k = row_best_exact(I.cost + (size_t)i * I.ldc, c.pot[i], c.pot + m, a, b);
            if (lane == 0) atomicMin((unsigned long long*)&c.row_best[i], (unsigned long long)k);
        }
        return;
    }
    stage_i32(vt, c.v32 + j0, jn);
    __syncthreads();
    const int4* v4 = reinterpret_cast<const int4*>(vt);
    for (long long u = (long long)rg * wpb + warp; u < units; u += stride) {
        const int i = rows ? rows[u / nseg] : (int)(u / nseg), s = (int)(u % nseg);
        if (!FLOCK_IN(i, m)) { if (lane == 0) fail_check(c.sc, 19); continue; }
        const int a = s * kSegCols, b = min(jn, a + kSegCols);   // tile-local columns [a, b)
        const int4* row = reinterpret_cast<const int4*>(I.cost + (size_t)i * I.ldc + j0);
        int32_t bv = INT32_MAX, bj = INT32_MAX;
        const int qa = a >> 2, qb = b >> 2;
        if (qb - qa == kSegCols / 4) {
            int4 cv[8];
            #pragma unroll
            for (int k = 0; k < 8; k++) cv[k] = ld_stream4(row + qa + lane + 32 * k);
            #pragma unroll
            for (int k = 0; k < 8; k++) {
                const int q = qa + lane + 32 * k;
                min4(bv, bj, cv[k], v4[q], j0 + 4 * q);
            }
        } else {
            for (int q = qa + lane; q < qb; q += 32) min4(bv, bj, ld_stream4(row + q), v4[q], j0 + 4 * q);
            if (lane < b - 4 * qb) {
                const int jl = 4 * qb + lane;
                const int32_t tv = I.cost[(size_t)i * I.ldc + j0 + jl] - vt[jl];
                if (tv < bv) { bv = tv; bj = j0 + jl; }
            }
        }
        const uint64_t k = narrow_row_key(c, i, j0 + a, j0 + b, bv, bj);
        if (lane == 0) atomicMin((unsigned long long*)&c.row_best[i], (unsigned long long)k);
    }
}

// ------------------------------------------------------ bulk-copy sweep ---
// The full reduced-cost sweep as a bulk-copy pipeline, one block per SM.
// blockIdx.x = tile + ntile * row_group; a block stages the int32 duals of
// its column tile and takes the work units (row i, segment of kBulkSeg
// columns) u = row_group, row_group + nrg, ...  Each warp owns kBulkDepth
// shared buffers and the block's units w, w + kBulkWarps, ...: lane 0 keeps
// kBulkDepth of them in flight with cp.async.bulk (each buffer completes on
// its own mbarrier by transaction bytes) and refills a buffer as soon as the
// warp has read it, so no warp waits for another.  The warp reduces c - v
// from shared memory into the row key (atomicMin into row_best, which holds
// kNoKey before the sweep).  Every wait is bounded: a wait that runs out
// records a failed check (the solve stops with ST_TREE_CORRUPT), and the
// warp still waits (bounded) for its copies in flight before it exits.
constexpr int kBulkSeg = 1024;                     // columns per unit: 4 KB of int32 costs
constexpr int kBulkWarps = 16;
constexpr int kBulkDepth = 3;                      // buffers (units in flight) per warp
constexpr int kBulkThreads = 32 * kBulkWarps;
constexpr size_t kBulkSmem = (size_t)kBulkWarps * kBulkDepth * kBulkSeg * 4 + (size_t)kSweepTile * 4;
constexpr long long kSpinLimit = 1ll << 22;        // polls of an mbarrier before its wait fails

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// Wait for the phase of the given parity to complete; false after kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity) {
    for (long long it = 0; it < kSpinLimit; it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(b)), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
// Global -> shared bulk copy completing on `bar` (addresses 16-byte aligned,
// bytes a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Unit k of this block: row i and tile-local columns [a, b).
struct BulkUnit {
    int i, a, b;
};
__device__ __forceinline__ BulkUnit bulk_unit(long long k, int rg, int nrg, int nseg, int jn, int segc) {
    const long long u = rg + k * nrg;
    BulkUnit w;
    w.i = (int)(u / nseg);
    w.a = (int)(u % nseg) * segc;
    w.b = min(jn, w.a + segc);
    return w;
}

__global__ void __launch_bounds__(kBulkThreads, 1) k_sweep(Ctx c, int tile, int ntile) {
    __shared__ __align__(8) uint64_t full[kBulkWarps * kBulkDepth];
    __shared__ __align__(8) uint64_t vbar;
    __shared__ PhaseLocal phl;
    extern __shared__ __align__(128) unsigned char bulk_smem[];
    // the cluster rounds that follow may be scheduled now; they wait for
    // this grid's completion before they read anything
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    PhaseScope ps(c.ph, &phl, PH_SWEEP);
    if (c.sc->done) { ps.idle(); return; }
    const InstDev& I = c.I;
    const int m = I.m, n = I.n;
    const int t = (int)blockIdx.x % ntile, rg = (int)blockIdx.x / ntile, nrg = (int)gridDim.x / ntile;
    const int j0 = t * tile, jn = min(tile, n - j0);
    // 16-bit costs (the copy exists only with narrow duals in mind): units
    // of 2 kBulkSeg columns, the same 4 KB per copy
    const bool h16 = I.cost16 != nullptr && c.sc->narrow;
    const int segc = h16 ? 2 * kBulkSeg : kBulkSeg;
    const int nseg = (jn + segc - 1) / segc;
    const long long units = (long long)m * nseg;
    const long long mine = units > rg ? (units - rg + nrg - 1) / nrg : 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // this warp's units: k = warp + j * kBulkWarps, j = 0 .. cnt-1
    const long long cnt = mine > warp ? (mine - warp + kBulkWarps - 1) / kBulkWarps : 0;
    if (!c.sc->narrow) {      // wide duals: exact int64 keys per element
        for (long long j = 0; j < cnt; j++) {
            const BulkUnit w = bulk_unit(warp + j * kBulkWarps, rg, nrg, nseg, jn, segc);
            const uint64_t key = row_best_exact(I.cost + (size_t)w.i * I.ldc, c.pot[w.i], c.pot + m, j0 + w.a, j0 + w.b);
            if (lane == 0) atomicMin((unsigned long long*)&c.row_best[w.i], (unsigned long long)key);
        }
        return;
    }
    int32_t* ring = reinterpret_cast<int32_t*>(bulk_smem) + (size_t)warp * kBulkDepth * kBulkSeg;
    int32_t* vt = reinterpret_cast<int32_t*>(bulk_smem) + (size_t)kBulkWarps * kBulkDepth * kBulkSeg;
    uint64_t* bar = full + warp * kBulkDepth;
    if (lane == 0) {
        for (int d = 0; d < kBulkDepth; d++) mbar_init(&bar[d], 1);
        if (warp == 0) mbar_init(&vbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (threadIdx.x == 0) {   // the tile's int32 duals: one bulk copy (j0 is a multiple of 4 columns; the
                              // rounded-up tail stays inside the dual array's allocation and is never read)
        const uint32_t vbytes = (uint32_t)(((jn + 3) & ~3) * 4);
        mbar_expect_tx(&vbar, vbytes);
        bulk_g2s(vt, c.v32 + j0, vbytes, &vbar);
    }
    __syncwarp();
    auto issue = [&](long long j) {          // lane 0: unit j of this warp into buffer j % kBulkDepth
        const int d = (int)(j % kBulkDepth);
        const BulkUnit w = bulk_unit(warp + j * kBulkWarps, rg, nrg, nseg, jn, segc);
        // within the row pitch (ldc = ceil4(n), ldc16 = ceil8(n))
        const uint32_t bytes = h16 ? (uint32_t)(((w.b - w.a + 7) & ~7) * 2) : (uint32_t)(((w.b - w.a + 3) & ~3) * 4);
        const void* src = h16 ? (const void*)(I.cost16 + (size_t)w.i * I.ldc16 + j0 + w.a)
                              : (const void*)(I.cost + (size_t)w.i * I.ldc + j0 + w.a);
        mbar_expect_tx(&bar[d], bytes);
        bulk_g2s(ring + (size_t)d * kBulkSeg, src, bytes, &bar[d]);
    };
    if (lane == 0)            // the first units stream while the duals land
        for (long long j = 0; j < cnt && j < kBulkDepth; j++) issue(j);
    __syncthreads();          // vbar's initialisation is visible to every warp
    // every lane waits (the copy's bytes become visible to the lanes that
    // observe the phase); the outcome is made the same for the whole warp
    const bool vt_ok = __all_sync(0xffffffffu, mbar_wait(&vbar, 0));
    for (long long j = 0; j < cnt; j++) {
        const int d = (int)(j % kBulkDepth);
        if (!vt_ok || !__all_sync(0xffffffffu, mbar_wait(&bar[d], (uint32_t)((j / kBulkDepth) & 1)))) {
            if (lane == 0) {
                fail_check(c.sc, 32);
                // the copies still in flight land before the warp exits
                const long long last = min(cnt, j + kBulkDepth);
                for (long long q = vt_ok ? j + 1 : j; q < last; q++)
                    mbar_wait(&bar[q % kBulkDepth], (uint32_t)((q / kBulkDepth) & 1));
                if (!vt_ok) mbar_wait(&vbar, 0);
            }
            return;
        }
        const BulkUnit w = bulk_unit(warp + j * kBulkWarps, rg, nrg, nseg, jn, segc);
        const int64_t ui = c.pot[w.i];                 // used after the reduction: its latency overlaps it
        const int32_t* src = ring + (size_t)d * kBulkSeg;
        const int4* s4 = reinterpret_cast<const int4*>(src);
        const int4* v4 = reinterpret_cast<const int4*>(vt + w.a);
        int32_t bv = INT32_MAX, bj = INT32_MAX;
        const int jb = j0 + w.a;
        if (h16) {
            const int nq = (w.b - w.a) >> 3;
            #pragma unroll 4
            for (int q = lane; q < nq; q += 32) min8(bv, bj, s4[q], v4[2 * q], v4[2 * q + 1], jb + 8 * q);
            if (lane < ((w.b - w.a) & 7)) {
                const int jl = 8 * nq + lane;
                const int32_t tv = (int32_t)reinterpret_cast<const int16_t*>(src)[jl] - vt[w.a + jl];
                if (tv < bv) { bv = tv; bj = jb + jl; }
            }
        } else {
            const int nq = (w.b - w.a) >> 2;
            #pragma unroll 4
            for (int q = lane; q < nq; q += 32) min4(bv, bj, s4[q], v4[q], jb + 4 * q);
            if (lane < ((w.b - w.a) & 3)) {
                const int jl = 4 * nq + lane;
                const int32_t tv = src[jl] - vt[w.a + jl];
                if (tv < bv) { bv = tv; bj = jb + jl; }
            }
        }
        __syncwarp();                                  // every lane has read the buffer
        if (lane == 0 && j + kBulkDepth < cnt) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the reads before the copy's writes
            issue(j + kBulkDepth);
        }
        // the row key as narrow_row_key forms it, the winning column's dual
        // read from the staged tile
        const uint64_t kk = warp_min_u64(pack_i32(bv, (uint32_t)bj));
        const int jw = (int)key_idx(kk);
        const int64_t r = (int64_t)key_val(kk) - ui;
        const uint64_t key = vt[jw - j0] == kDead32 || r < INT32_MIN
                                 ? row_best_exact(I.cost + (size_t)w.i * I.ldc, ui, c.pot + m, jb, j0 + w.b)
                                 : pack_i32(clamp32(r), (uint32_t)jw);
        if (lane == 0) atomicMin((unsigned long long*)&c.row_best[w.i], (unsigned long long)key);
    }
}

// Launch shape of the grid-round sweeps (k_gsweep) for an m x n instance:
// column tiles of at most kSweepTile, two blocks per SM in total, no more
// blocks than work units.  bulk_shape: k_sweep's, one block per SM.
static void sweep_shape(int m, int n, int* grid, int* tile, int* ntile);
static void bulk_shape(int m, int n, int* grid, int* tile, int* ntile);

__global__ void __launch_bounds__(1024, 1) k_pivot(Ctx c) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_SWEEP);   // the entering choice is part of pricing
    if (c.sc->done) { ps.idle(); return; }
    pivot_round_cta<kJumpPlain, true>(c, bs, false, kNoKey, &ps);
    if (threadIdx.x == 0) {
        c.sc->rounds++;
        if (!c.sc->done && c.sc->rounds >= c.sc->max_rounds) { c.sc->status |= ST_ITER_CAP; c.sc->done = 1; }
    }
    __syncthreads();
    if (!c.sc->done && c.sc->stale) {
        ps.mark(PH_DUAL);
        tree_build_cta<kJumpPlain>(c, bs);
    }
    ps.mark(PH_SWEEP);   // the key reset and the next round's sweep
    for (int i = threadIdx.x; i < c.I.m; i += blockDim.x) c.row_best[i] = kNoKey;
}

// ------------------------------------------------- grid pivot round -------
// The plain solver's rounds for large instances, spread over the whole GPU:
// six graph-captured kernels per round, the kernel boundaries the only
// synchronisation (a grid-wide barrier inside one cooperative launch costs
// as much as a boundary on this two-die part).  One pivot per round
// (Dantzig's rule: the most negative row key, first row among ties); the
// steps follow single_pivot_iv exactly (same interval membership test, tie
// rules, path reversal and in-place update of depths, duals and intervals),
// so a round costs the same six launches whatever the tree's depth.
struct GridPivot {
    uint64_t best;          // entering candidate: (reduced cost, row)
    uint64_t mk, ml;        // per side: minimum order-preserving flow
    uint64_t qk, ql;        // per side: leaving edge (depth << 32 | child)
    int32_t pad0_;
    int32_t dwide;          // change of the count of int32-window misses
    int32_t full;           // partial pricing: this round swept every row
    uint32_t fin_count;     // blocks done with the update step
    // the pivot, fixed by the pick step's last block before the update changes depths and duals
    int64_t th, r;
    int32_t ok, e, other, q, de, dq, t, dother, eside, pad2_;
    int2 Q, O;
};

// plain instances with m + n >= this use the grid round (its cluster rounds
// beat one CTA from about 2400 vertices: 1500 x 1000 uniform 82 vs 98 ms,
// 2000 x 2000 180 vs 299 ms; 1000 x 1000 Euclidean 77 vs 67 ms)
constexpr int kGridPivotV = 2400;
// The grid-round threshold in effect (FLOCK_GRID_V overrides kGridPivotV, for
// tuning; at least 64).
static int grid_pivot_v() {
    static const int v = [] {
        const char* e = getenv("FLOCK_GRID_V");
        const int x = e ? atoi(e) : 0;
        return x >= 64 ? x : kGridPivotV;
    }();
    return v;
}

__device__ __forceinline__ const int2* iv_now(const Ctx& c, int V) { return c.iv + (c.sc->ivp ? V : 0); }

// Block 0: the entering candidate (over every row after a full sweep, over
// the candidate rows otherwise: the others hold no key), the next candidate
// rows after a full sweep, the round's bookkeeping.
__device__ void grid_choose(const Ctx& c, GridPivot* gp, BlockScratch& bs, bool full, bool select) {
    const int m = c.I.m;
    const uint32_t ncols = (uint32_t)c.I.n;
    const int nrows = full ? m : min(max(c.sc->pp_n, 0), kPPRows);
    uint64_t best = kNoKey;
    for (int t = threadIdx.x; t < nrows; t += blockDim.x) {
        const int i = full ? t : c.prow[t];
        if (!FLOCK_IN(i, m)) continue;
        const uint64_t k = c.row_best[i];
        if (k != kNoKey && key_val(k) < 0) {
            if (key_idx(k) >= ncols) { fail_check(c.sc, 18); continue; }
            const uint64_t P = pack_i32(key_val(k), (uint32_t)i);
            best = P < best ? P : best;
        }
    }
    best = block_min_u64(best, bs);
    if (select) select_candidate_rows(c, bs, false);
    if (threadIdx.x == 0) {
        gp->best = best;
        gp->mk = gp->ml = kNoKey;
        gp->qk = 0;
        gp->ql = kNoKey;
        gp->dwide = 0;
        gp->ok = 0;
        gp->fin_count = 0;
        c.sc->rounds++;
        c.sc->pp_age++;
        c.sc->ncand = best == kNoKey ? 0 : 1;
        if (best == kNoKey) c.sc->done = 1;
    }
}

// Cycle membership by intervals, each side's smallest decreasing flow, and
// both cycle chains by distance from their endpoint with their flows
// (path[i] / pflow[i] for the k side, path[V-1-i] / pflow[V-1-i] for the l
// side, as single_pivot_iv records them), over the vertices v0, v0 + stride,
// ...  (iv: the current interval buffer; dk, dl: the endpoints' depths).
__device__ __forceinline__ void member_slice(const Ctx& c, const int2* iv, int k, int l, int dk, int dl, int v0,
                                             int stride, uint64_t& mk, uint64_t& ml, int2* piv = nullptr) {
    const int m = c.I.m, V = m + c.I.n;
    const int pk = iv[k].x, pl = iv[l].x;
    for (int v = v0; v < V; v += stride) {
        int side = 0;
        if (c.parent[v] >= 0) {
            const int2 w = iv[v];
            const bool on_k = iv_in(w, pk), on_l = iv_in(w, pl);
            if (on_k != on_l) side = on_k ? 1 : 2;
        }
        c.side[v] = (uint8_t)side;
        if (!side) continue;
        const int64_t f = c.flow[v];
        const int i = (side == 1 ? dk : dl) - c.depth[v];
        if (!FLOCK_IN(i, V)) { fail_check(c.sc, 17); continue; }
        const int slot = side == 1 ? i : V - 1 - i;
        c.path[slot] = v;
        c.pflow[slot] = f;
        if (piv) piv[slot] = iv[v];
        if (side == 1 && v < m) { const uint64_t o = oflow(f); mk = o < mk ? o : mk; }
        if (side == 2 && v >= m) { const uint64_t o = oflow(f); ml = o < ml ? o : ml; }
    }
}

__device__ void grid_member(const Ctx& c, GridPivot* gp, BlockScratch& bs, int bid, int nb) {
    const int m = c.I.m, V = m + c.I.n;
    const int k = (int)key_idx(gp->best);
    const int l = m + (int)key_idx(c.row_best[k]);
    uint64_t mk = kNoKey, ml = kNoKey;
    member_slice(c, iv_now(c, V), k, l, c.depth[k], c.depth[l], bid * blockDim.x + threadIdx.x, nb * blockDim.x,
                 mk, ml);
    mk = block_min_u64(mk, bs);
    ml = block_min_u64(ml, bs);
    if (threadIdx.x == 0) {
        if (mk != kNoKey) atomicMin((unsigned long long*)&gp->mk, (unsigned long long)mk);
        if (ml != kNoKey) atomicMin((unsigned long long*)&gp->ml, (unsigned long long)ml);
    }
}

// This thread's leaving-edge candidate over its vertices: among the cycle
// edges of the side whose minimum flow fmin is smaller (l side on ties), the
// (depth << 32 | child) keys with that flow -- the l side keeps the
// shallowest (minimum), the k side the deepest (maximum; 0 = none).
__device__ __forceinline__ uint64_t pick_slice(const Ctx& c, bool lside, uint64_t fmin, int v0, int stride) {
    const int m = c.I.m, V = m + c.I.n;
    uint64_t pick = lside ? kNoKey : 0ull;
    for (int v = v0; v < V; v += stride) {
        const uint64_t sd = c.side[v];
        if ((lside ? (sd == 2 && v >= m) : (sd == 1 && v < m)) && oflow(c.flow[v]) == fmin) {
            const uint64_t key = ((uint64_t)(uint32_t)c.depth[v] << 32) | (uint32_t)v;
            if (lside) pick = key < pick ? key : pick;
            else pick = key > pick ? key : pick;
        }
    }
    return pick;
}

// The leaving edge among the minima: k side the deepest, l side the shallowest.
__device__ void grid_pick(const Ctx& c, GridPivot* gp, BlockScratch& bs, int bid, int nb) {
    const int m = c.I.m, V = m + c.I.n;
    const bool lside = gp->ml <= gp->mk;
    const uint64_t fmin = lside ? gp->ml : gp->mk;
    if (fmin == kNoKey) {
        if (bid == 0 && threadIdx.x == 0) fail_check(c.sc, 16);
        return;
    }
    uint64_t pick = pick_slice(c, lside, fmin, bid * blockDim.x + threadIdx.x, nb * blockDim.x);
    pick = lside ? block_min_u64(pick, bs) : block_max_u64(pick, bs);
    if (threadIdx.x == 0) {
        if (lside && pick != kNoKey) atomicMin((unsigned long long*)&gp->ql, (unsigned long long)pick);
        if (!lside && pick != 0) atomicMax((unsigned long long*)&gp->qk, (unsigned long long)pick);
        __threadfence();
        // the last block to finish fixes the pivot's parameters for the
        // update (nothing in this step changes depths, duals or intervals)
        if (atomicAdd(&gp->fin_count, 1u) == (unsigned)nb - 1) {
            __threadfence();
            gp->fin_count = 0;
            const uint64_t q64 = lside ? *(volatile uint64_t*)&gp->ql : *(volatile uint64_t*)&gp->qk;
            const int q = (int)(uint32_t)q64;
            const int k = (int)key_idx(gp->best);
            const int l = m + (int)key_idx(c.row_best[k]);
            const int e = lside ? l : k, other = lside ? k : l;
            const int de = c.depth[e];
            const int t = (lside ? q64 != kNoKey : q64 != 0) && FLOCK_IN(q, V) ? de - c.depth[q] : -1;
            const int slot = lside ? V - 1 - t : t;
            if (!FLOCK_IN(t, V) || c.path[slot] != q) {
                fail_check(c.sc, 17);
            } else {
                const int2* iv = iv_now(c, V);
                gp->th = (int64_t)(fmin ^ 0x8000000000000000ull);
                gp->r = (int64_t)cost_of(c.I, k, l - m) - c.pot[k] - c.pot[l];
                gp->e = e; gp->other = other; gp->q = q;
                gp->de = de; gp->dq = c.depth[q]; gp->t = t;
                gp->dother = c.depth[other];
                gp->eside = lside ? 2 : 1;
                gp->Q = iv[q]; gp->O = iv[other];
                gp->ok = 1;
            }
        }
    }
}

// The pivot as the update step needs it (fixed before anything it depends
// on changes).
struct PivotParams {
    int32_t t, e, other, de, dother, eside;
    int64_t th, r;
    int2 Q, O;
};

// The tree update of single_pivot_iv over the vertices v0, v0 + stride, ...:
// the cycle's flows, new intervals into ivB (old ones read from ivA), depths
// and duals of the re-hung subtree, the reversed path's parents and flows.
// Adds the change of the int32-window miss count to dwide; sets bad on a
// failed index check.
// spv / siv (optional, shared memory): path[base + dir * i] and its old
// interval for i = 0..t, which the binary searches read in place of global
// memory.
__device__ __forceinline__ void update_slice(const Ctx& c, const PivotParams& pp, const int2* ivA, int2* ivB, int v0,
                                             int stride, int& dwide, int& bad, const int32_t* spv = nullptr,
                                             const int2* siv = nullptr) {
    const int m = c.I.m, V = m + c.I.n;
    const int t = pp.t;
    const bool lside = pp.eside == 2;
    const int base = lside ? V - 1 : 0, dir = lside ? -1 : 1;   // e's chain entry i at path[base + dir * i]
    const int2 Q = pp.Q, O = pp.O;
    const int P = Q.x, s = Q.y;
    const int ins = O.x - (O.x >= P + s ? s : 0) + 1;
    const int dnew = pp.dother + 1 - pp.de;
    const int other = pp.other;
    const bool erow = pp.e < m;
    const int64_t r = pp.r, th = pp.th;
    const int eside = pp.eside;
    const int32_t* path = c.path;
    const int64_t* pflow = c.pflow;
    for (int v = v0; v < V; v += stride) {
        if (c.parent[v] == -2) continue;
        const int2 w = ivA[v];
        const int side = c.side[v];
        int2 nw;
        if (iv_in(Q, w.x)) {
            int lo = 0, hi = t;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                const int pv = spv ? spv[mid] : path[base + dir * mid];
                if (!FLOCK_IN(pv, V)) { bad = 1; break; }
                if (iv_in(siv ? siv[mid] : ivA[pv], w.x)) hi = mid; else lo = mid + 1;
            }
            const int i = lo;
            const int pi = spv ? spv[i] : path[base + dir * i];
            if (!FLOCK_IN(pi, V)) { bad = 1; continue; }
            const int2 Pi = siv ? siv[i] : ivA[pi];
            int off = 0, rank = w.x - Pi.x;
            int pc = -1;
            if (i > 0) {
                pc = spv ? spv[i - 1] : path[base + dir * (i - 1)];
                if (!FLOCK_IN(pc, V)) { bad = 1; continue; }
                const int2 Pc = siv ? siv[i - 1] : ivA[pc];
                off = Pc.y;
                if (w.x >= Pc.x) rank -= Pc.y;
            }
            nw.x = ins + off + rank;
            nw.y = v == pi ? s - off : w.y;
            c.depth[v] = dnew + 2 * i + c.depth[v];
            const int64_t p0 = c.pot[v];
            const int64_t p1 = p0 + ((v < m) == erow ? r : -r);
            c.pot[v] = p1;
            if (v >= m) {
                int w0 = 0, w1 = 0;
                narrow_dual(p0, w0);
                c.v32[v - m] = narrow_dual(p1, w1);
                dwide += w1 - w0;
            }
            if (v == pi) {                             // the reversed path (every cycle edge in S is on it)
                c.parent[v] = i == 0 ? other : pc;
                c.flow[v] = i == 0 ? th
                                   : pflow[base + dir * (i - 1)] + ((eside == 1) == (pc < m) ? -th : th);
            }
        } else {
            if (side) c.flow[v] += (side == 1) == (v < m) ? -th : th;
            const int y = w.x - (w.x >= P + s ? s : 0);
            nw.x = y + (y >= ins ? s : 0);
            nw.y = w.y - (iv_in(w, P) ? s : 0) + (iv_in(w, O.x) ? s : 0);
        }
        ivB[v] = nw;
    }
}

// The tree update over the grid, every row key cleared for the next sweep.
// The last block to finish ends the round: the current interval buffer, the
// int32 dual flag, the pivot count and the round cap.
__device__ void grid_update(const Ctx& c, GridPivot* gp, BlockScratch& bs, int bid, int nb) {
    const int m = c.I.m, V = m + c.I.n;
    if (!gp->ok || !FLOCK_IN(gp->t, V)) {
        if (bid == 0 && threadIdx.x == 0) fail_check(c.sc, 17);
        return;
    }
    PivotParams pp;
    pp.t = gp->t; pp.e = gp->e; pp.other = gp->other; pp.de = gp->de; pp.dother = gp->dother;
    pp.eside = gp->eside; pp.th = gp->th; pp.r = gp->r; pp.Q = gp->Q; pp.O = gp->O;
    const int par = c.sc->ivp;
    if (threadIdx.x == 0) bs.i[7] = 0;
    __syncthreads();
    int dwide = 0, bad = 0;
    update_slice(c, pp, c.iv + (par ? V : 0), c.iv + (par ? 0 : V), bid * blockDim.x + threadIdx.x,
                 nb * blockDim.x, dwide, bad);
    for (int i = bid * blockDim.x + threadIdx.x; i < m; i += nb * blockDim.x) c.row_best[i] = kNoKey;
    if (bad) fail_check(c.sc, 24);
    if (dwide) atomicAdd(&bs.i[7], dwide);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (bs.i[7]) atomicAdd(&gp->dwide, bs.i[7]);
        __threadfence();
        if (atomicAdd(&gp->fin_count, 1u) == (unsigned)nb - 1) {     // every block's share is in
            __threadfence();
            c.sc->ivp ^= 1;
            c.sc->nwide += *(volatile int32_t*)&gp->dwide;
            c.sc->narrow = c.sc->nwide == 0;
            c.sc->pivots++;
            c.sc->last_winners = 1;
            if (c.sc->rounds >= c.sc->max_rounds) { c.sc->status |= ST_ITER_CAP; c.sc->done = 1; }
        }
    }
}

// Step kernels of a grid round.  Each returns at once when the solve is
// done (one thread reads the flag, so the whole block agrees).
#define FLOCK_GRID_STEP_PROLOGUE()                                 \
    if (__syncthreads_or(threadIdx.x == 0 && c.sc->done)) {        \
        ps.idle();                                                 \
        return;                                                    \
    }

// The grid sweeps keep every register for the stream (no phase scope of
// their own): the round's previous launch leaves the sweep phase running.
#define FLOCK_SWEEP_STEP_PROLOGUE() \
    if (__syncthreads_or(threadIdx.x == 0 && c.sc->done)) return

// Partial pricing decision of the round (every block computes it from the
// same scalars): sweep every row, else the candidate rows.
__device__ __forceinline__ bool grid_full_round(const Ctx& c) {
    const int pn = c.sc->pp_n;
    return !c.sc->pricing || pn <= 0 || pn > kPPRows || c.sc->pp_age >= max(c.sc->pp_refresh, 1);
}

// Round start: the sweep this round's pricing asks for.
__global__ void __launch_bounds__(kSweepThreads, 2) k_gsweep(Ctx c, GridPivot* gp, int tile, int ntile) {
    __shared__ __align__(16) int32_t vt[kSweepTile];
    FLOCK_SWEEP_STEP_PROLOGUE();
    const bool full = grid_full_round(c);
    if (blockIdx.x == 0 && threadIdx.x == 0) gp->full = full ? 1 : 0;
    sweep_part(c, tile, ntile, full ? nullptr : c.prow, vt, (int)blockIdx.x, (int)gridDim.x);
}

// After a candidate sweep: every row when the candidates hold no negative
// key (every block checks the same keys).
__global__ void __launch_bounds__(kSweepThreads, 2) k_gsweep_rest(Ctx c, GridPivot* gp, int tile, int ntile) {
    __shared__ __align__(16) int32_t vt[kSweepTile];
    FLOCK_SWEEP_STEP_PROLOGUE();
    if (grid_full_round(c)) return;
    const int m = c.I.m, pn = c.sc->pp_n;
    int neg = 0;
    for (int t = threadIdx.x; t < pn; t += blockDim.x) {
        const int i = c.prow[t];
        if (FLOCK_IN(i, m)) neg |= key_val(c.row_best[i]) < 0;
    }
    if (__syncthreads_or(neg)) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) gp->full = 1;
    sweep_part(c, tile, ntile, nullptr, vt, (int)blockIdx.x, (int)gridDim.x);
}

__global__ void __launch_bounds__(1024, 1) k_gchoose(Ctx c, GridPivot* gp) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_SWEEP);   // the entering choice is part of pricing
    FLOCK_GRID_STEP_PROLOGUE();
    const bool full = gp->full != 0;
    grid_choose(c, gp, bs, full, full && c.sc->pricing);
}

// The full round ahead of the cluster rounds: the entering cell over every
// row (the bulk sweep just priced them all) and the next candidate rows.
__global__ void __launch_bounds__(1024, 1) k_gchoose_all(Ctx c, GridPivot* gp) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_SWEEP);
    FLOCK_GRID_STEP_PROLOGUE();
    grid_choose(c, gp, bs, true, c.sc->pricing != 0);
}

__global__ void __launch_bounds__(256) k_gmember(Ctx c, GridPivot* gp) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_CYCLE);
    FLOCK_GRID_STEP_PROLOGUE();
    grid_member(c, gp, bs, (int)blockIdx.x, (int)gridDim.x);
}

__global__ void __launch_bounds__(256) k_gpick(Ctx c, GridPivot* gp) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_ADJUST);   // leaving edge: the reference's adjustment step
    FLOCK_GRID_STEP_PROLOGUE();
    grid_pick(c, gp, bs, (int)blockIdx.x, (int)gridDim.x);
}

__global__ void __launch_bounds__(256) k_gupdate(Ctx c, GridPivot* gp) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_ADJUST);
    FLOCK_GRID_STEP_PROLOGUE();
    grid_update(c, gp, bs, (int)blockIdx.x, (int)gridDim.x);
    ps.mark(PH_SWEEP);   // the next round's sweeps
}

// ------------------------------------------------- cluster pivot rounds ---
// The partial-pricing rounds of the grid path in ONE launch of a single
// thread-block cluster (up to kClusterMax CTAs of kCRoundThreads threads on
// one GPC), the hardware cluster barrier in place of the kernel boundaries
// of the six-kernel round.  A round:
//   sweep of the candidate rows (their keys hold kNoKey)          barrier 1
//   the entering cell (every CTA reduces the same keys), snapshots of the
//   values the update will change, membership and side minima of each
//   CTA's vertex slice                                             barrier 2
//   the leaving edge's candidates of each slice                    barrier 3
//   the pivot's parameters (every CTA reduces the same slots), the in-place
//   update of each slice                                           barrier 0
// with the same steps and tie rules as grid_member / grid_pick /
// grid_update, so the pivot sequence is the six-kernel rounds'.  The rounds
// stop -- every CTA decides from the same values, written before a barrier
// and not rewritten until after the next one -- when the candidates hold no
// negative key (the next full sweep decides optimality), when pp_refresh
// rounds have passed since the last full sweep, at the round cap, or after
// a failed check.  What the CTAs share lives in global memory in per-CTA
// slots (ClusterPivot), so nothing is reset between rounds; the solve's
// scalars are read at the start and written back by CTA 0 at the end.  The
// cluster barrier waits for every thread of the cluster that has not
// exited, and every loop here is bounded, so the barriers cannot hang.
constexpr int kCRoundThreads = 1024;
constexpr int kClusterMax = 16;

struct ClusterPivot {
    int32_t dwide[kClusterMax];                    // update step: change of the int32-window miss count
    int32_t abort[2];                              // a failed check in the round of that parity
};

__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// Another CTA's copy of a shared variable (distributed shared memory): the
// writer stores it before a cluster barrier, the readers load it after.
__device__ __forceinline__ uint32_t dsmem_of(const void* local, int rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(local)), "r"(rank));
    return r;
}
__device__ __forceinline__ uint64_t dsmem_ld_u64(uint32_t a) {
    uint64_t v;
    asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(a) : "memory");
    return v;
}

__device__ __forceinline__ int cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return (int)r;
}
__device__ __forceinline__ int cluster_ctas() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return (int)r;
}

// The cluster rounds' register form (every thread owns at most one vertex:
// V <= CTAs x threads).  During the rounds the owner is the only writer of
// its vertex's parent, depth, flow, interval and dual, so it keeps them in
// registers and writes them through for the other readers (the candidate
// sweep's duals, the entering cell's endpoints, the path cache, the next
// launch).
struct OwnVertex {
    int32_t v, parent, depth, side;
    int64_t flow, pot;
    int2 iv;
};

__device__ __forceinline__ void own_load(const Ctx& c, OwnVertex& o, int v, const int2* ivA) {
    const int V = c.I.m + c.I.n;
    o.v = v;
    o.side = 0;
    if (v < V) { o.parent = c.parent[v]; o.depth = c.depth[v]; o.flow = c.flow[v]; o.pot = c.pot[v]; o.iv = ivA[v]; }
    else { o.parent = -2; o.depth = 0; o.flow = 0; o.pot = 0; o.iv = make_int2(0, 0); }
}

// member_slice for the owned vertex (its side kept in the register state).
__device__ __forceinline__ void member_one(const Ctx& c, OwnVertex& o, int pk, int pl, int dk, int dl,
                                           uint64_t& mk, uint64_t& ml, int2* piv) {
    const int m = c.I.m, V = m + c.I.n;
    o.side = 0;
    if (o.v >= V || o.parent < 0) return;
    const bool on_k = iv_in(o.iv, pk), on_l = iv_in(o.iv, pl);
    if (on_k == on_l) return;
    o.side = on_k ? 1 : 2;
    const int i = (o.side == 1 ? dk : dl) - o.depth;
    if (!FLOCK_IN(i, V)) { fail_check(c.sc, 17); return; }
    const int slot = o.side == 1 ? i : V - 1 - i;
    c.path[slot] = o.v;
    c.pflow[slot] = o.flow;
    piv[slot] = o.iv;
    if (o.side == 1 && o.v < m) { const uint64_t f = oflow(o.flow); mk = f < mk ? f : mk; }
    if (o.side == 2 && o.v >= m) { const uint64_t f = oflow(o.flow); ml = f < ml ? f : ml; }
}

// pick_slice for the owned vertex.
__device__ __forceinline__ uint64_t pick_one(const Ctx& c, const OwnVertex& o, bool lside, uint64_t fmin) {
    const int m = c.I.m;
    if ((lside ? (o.side == 2 && o.v >= m) : (o.side == 1 && o.v < m)) && oflow(o.flow) == fmin)
        return ((uint64_t)(uint32_t)o.depth << 32) | (uint32_t)o.v;
    return lside ? kNoKey : 0ull;
}

// update_slice for the owned vertex, its register state updated with it.
__device__ __forceinline__ void update_one(const Ctx& c, const PivotParams& pp, OwnVertex& o, const int2* ivA,
                                           int2* ivB, int& dwide, int& bad, const int32_t* spv, const int2* siv) {
    const int m = c.I.m, V = m + c.I.n;
    const int v = o.v;
    if (v >= V || o.parent == -2) return;
    const int t = pp.t;
    const bool lside = pp.eside == 2;
    const int base = lside ? V - 1 : 0, dir = lside ? -1 : 1;   // e's chain entry i at path[base + dir * i]
    const int2 Q = pp.Q, O = pp.O;
    const int P = Q.x, s = Q.y;
    const int ins = O.x - (O.x >= P + s ? s : 0) + 1;
    const int2 w = o.iv;
    int2 nw;
    if (iv_in(Q, w.x)) {
        int lo = 0, hi = t;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const int pv = spv ? spv[mid] : c.path[base + dir * mid];
            if (!FLOCK_IN(pv, V)) { bad = 1; break; }
            if (iv_in(siv ? siv[mid] : ivA[pv], w.x)) hi = mid; else lo = mid + 1;
        }
        const int i = lo;
        const int pi = spv ? spv[i] : c.path[base + dir * i];
        if (!FLOCK_IN(pi, V)) { bad = 1; return; }
        const int2 Pi = siv ? siv[i] : ivA[pi];
        int off = 0, rank = w.x - Pi.x;
        int pc = -1;
        if (i > 0) {
            pc = spv ? spv[i - 1] : c.path[base + dir * (i - 1)];
            if (!FLOCK_IN(pc, V)) { bad = 1; return; }
            const int2 Pc = siv ? siv[i - 1] : ivA[pc];
            off = Pc.y;
            if (w.x >= Pc.x) rank -= Pc.y;
        }
        nw.x = ins + off + rank;
        nw.y = v == pi ? s - off : w.y;
        o.depth = pp.dother + 1 - pp.de + 2 * i + o.depth;
        c.depth[v] = o.depth;
        const int64_t p0 = o.pot;
        const int64_t p1 = p0 + ((v < m) == (pp.e < m) ? pp.r : -pp.r);
        o.pot = p1;
        c.pot[v] = p1;
        if (v >= m) {
            int w0 = 0, w1 = 0;
            narrow_dual(p0, w0);
            c.v32[v - m] = narrow_dual(p1, w1);
            dwide += w1 - w0;
        }
        if (v == pi) {                             // the reversed path (every cycle edge in S is on it)
            o.parent = i == 0 ? pp.other : pc;
            o.flow = i == 0 ? pp.th : c.pflow[base + dir * (i - 1)] + ((pp.eside == 1) == (pc < m) ? -pp.th : pp.th);
            c.parent[v] = o.parent;
            c.flow[v] = o.flow;
        }
    } else {
        if (o.side) {
            o.flow += (o.side == 1) == (v < m) ? -pp.th : pp.th;
            c.flow[v] = o.flow;
        }
        const int y = w.x - (w.x >= P + s ? s : 0);
        nw.x = y + (y >= ins ? s : 0);
        nw.y = w.y - (iv_in(w, P) ? s : 0) + (iv_in(w, O.x) ? s : 0);
    }
    o.iv = nw;
    ivB[v] = nw;
}

// Sweep of the candidate rows prow[0..pn) (the launch's shared copy of
// c.prow) over the cluster: (row, segment of kSegCols columns) units, one
// warp each, keys into row_best by atomicMin.
__device__ uint64_t cluster_cand_sweep(const Ctx& c, const int32_t* prow, int pn, bool narrow, int rank, int nctas,
                                       int* bad) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n;
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const int gw = rank * wpb + (threadIdx.x >> 5), nw = nctas * wpb;
    // 16-bit costs: units of 2 kSegCols columns, the same 8 vectors per lane
    const bool h16 = I.cost16 != nullptr && narrow;
    const int segc = h16 ? 2 * kSegCols : kSegCols;
    const int nseg = (n + segc - 1) / segc;
    const int units = pn * nseg;
    const int4* v4 = reinterpret_cast<const int4*>(c.v32);
    uint64_t best = kNoKey;
    for (int u = gw; u < units; u += nw) {
        const int i = prow[u / nseg], sg = u % nseg;
        if (!FLOCK_IN(i, m)) { *bad = 1; continue; }
        const int a = sg * segc, b = min(n, a + segc);
        const int64_t ui = c.pot[i];                   // used after the reduction: its latency overlaps it
        uint64_t key;
        if (!narrow) {
            key = row_best_exact(I.cost + (size_t)i * I.ldc, ui, c.pot + m, a, b);
        } else if (h16) {
            const int4* row = reinterpret_cast<const int4*>(I.cost16 + (size_t)i * I.ldc16);
            int32_t bv = INT32_MAX, bj = INT32_MAX, bdual = 0;
            const int qa = a >> 3, qb = b >> 3;
            auto take8 = [&](const int4 cv, int q) {      // 8 costs against their duals (the winner's kept)
                const int4 va = v4[2 * q], vb = v4[2 * q + 1];
                const uint32_t w[4] = {(uint32_t)cv.x, (uint32_t)cv.y, (uint32_t)cv.z, (uint32_t)cv.w};
                const int32_t v[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
                #pragma unroll
                for (int k = 0; k < 8; k++) {
                    const int32_t t = (int32_t)(int16_t)(uint16_t)(w[k >> 1] >> (16 * (k & 1))) - v[k];
                    if (t < bv) { bv = t; bj = 8 * q + k; bdual = v[k]; }
                }
            };
            if (qb - qa == kSegCols / 4) {
                // a full segment: the lane's 8 cost vectors in flight at once
                int4 cv[kSegCols / 128];
                #pragma unroll
                for (int k = 0; k < kSegCols / 128; k++) cv[k] = ld_stream4(row + qa + lane + 32 * k);
                #pragma unroll
                for (int k = 0; k < kSegCols / 128; k++) take8(cv[k], qa + lane + 32 * k);
            } else {
                for (int q = qa + lane; q < qb; q += 32) take8(row[q], q);
            }
            if (lane < b - 8 * qb) {
                const int j = 8 * qb + lane;
                const int32_t vj = c.v32[j];
                const int32_t tv = (int32_t)I.cost16[(size_t)i * I.ldc16 + j] - vj;
                if (tv < bv) { bv = tv; bj = j; bdual = vj; }
            }
            // the row key as narrow_row_key forms it; the winning column's
            // dual comes from the lane that found it
            const uint64_t mine = pack_i32(bv, (uint32_t)bj);
            const uint64_t kk = warp_min_u64(mine);
            const unsigned who = __ballot_sync(0xffffffffu, mine == kk);
            const int32_t vw = __shfl_sync(0xffffffffu, bdual, __ffs(who) - 1);
            const int64_t r = (int64_t)key_val(kk) - ui;
            key = vw == kDead32 || r < INT32_MIN ? row_best_exact(I.cost + (size_t)i * I.ldc, ui, c.pot + m, a, b)
                                                 : pack_i32(clamp32(r), (uint32_t)key_idx(kk));
        } else {
            const int4* row = reinterpret_cast<const int4*>(I.cost + (size_t)i * I.ldc);
            int32_t bv = INT32_MAX, bj = INT32_MAX, bdual = 0;
            const int qa = a >> 2, qb = b >> 2;
            auto take = [&](const int4 cv, const int4 vv, int q) {
                int32_t t;
                t = cv.x - vv.x; if (t < bv) { bv = t; bj = 4 * q; bdual = vv.x; }
                t = cv.y - vv.y; if (t < bv) { bv = t; bj = 4 * q + 1; bdual = vv.y; }
                t = cv.z - vv.z; if (t < bv) { bv = t; bj = 4 * q + 2; bdual = vv.z; }
                t = cv.w - vv.w; if (t < bv) { bv = t; bj = 4 * q + 3; bdual = vv.w; }
            };
            if (qb - qa == kSegCols / 4) {
                // a full segment: the lane's 8 cost vectors in flight at once
                // (one L2 round trip); the duals are read as they are used
                int4 cv[kSegCols / 128];
                #pragma unroll
                for (int k = 0; k < kSegCols / 128; k++) cv[k] = ld_stream4(row + qa + lane + 32 * k);
                #pragma unroll
                for (int k = 0; k < kSegCols / 128; k++) {
                    const int q = qa + lane + 32 * k;
                    take(cv[k], v4[q], q);
                }
            } else {
                for (int q = qa + lane; q < qb; q += 32) take(row[q], v4[q], q);
            }
            if (lane < b - 4 * qb) {
                const int j = 4 * qb + lane;
                const int32_t vj = c.v32[j];
                const int32_t tv = I.cost[(size_t)i * I.ldc + j] - vj;
                if (tv < bv) { bv = tv; bj = j; bdual = vj; }
            }
            // the row key as narrow_row_key forms it; the winning column's
            // dual comes from the lane that found it
            const uint64_t mine = pack_i32(bv, (uint32_t)bj);
            const uint64_t kk = warp_min_u64(mine);
            const unsigned who = __ballot_sync(0xffffffffu, mine == kk);
            const int32_t vw = __shfl_sync(0xffffffffu, bdual, __ffs(who) - 1);
            const int jw = (int)key_idx(kk);
            const int64_t r = (int64_t)key_val(kk) - ui;
            key = vw == kDead32 || r < INT32_MIN ? row_best_exact(I.cost + (size_t)i * I.ldc, ui, c.pot + m, a, b)
                                                 : pack_i32(clamp32(r), (uint32_t)jw);
        }
        if (lane == 0) atomicMin((unsigned long long*)&c.row_best[i], (unsigned long long)key);
        // the sequential rule's entering row over this warp's units: the
        // smallest (reduced cost, row) among the negative unit keys, which
        // over all units equals the smallest (row key, row) of the rows
        if (key != kNoKey && key_val(key) < 0) {
            const uint64_t P = pack_i32(key_val(key), (uint32_t)i);
            best = P < best ? P : best;
        }
    }
    return best;
}

// Entries of the re-hung path the cluster rounds cache in shared memory for
// the update's binary searches (a longer path is searched in global memory).
constexpr int kPathCache = 8192;
constexpr size_t kCRoundSmem = (size_t)kPathCache * (sizeof(int2) + sizeof(int32_t));

// full_first: round 0 is the full round that the bulk sweep has just priced
// (every row key current): the cluster chooses its entering cell and the
// next candidate rows (select_candidate_rows' rule), counts it, pivots, and
// the update clears every row key for the coming candidate sweeps.  (gp: the
// grid rounds' block, unused by this form.)
template <bool kOne>
__global__ void __launch_bounds__(kCRoundThreads, 1) k_cround(Ctx c, ClusterPivot* cp, const GridPivot* gp,
                                                              int full_first) {
    (void)gp;
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    // this CTA's share of the round's cluster-wide minima, read by warp 0 of
    // every CTA through distributed shared memory (s_red: the results)
    __shared__ uint64_t x_best, x_mk, x_ml, x_pick, s_red[2];
    __shared__ int32_t s_prow[kPPRows];    // the candidate rows: fixed for the launch
    // the full round's candidate selection: this CTA's smallest key value,
    // histogram and count of kept rows, read through distributed shared memory
    __shared__ int32_t x_rmin, x_hist[32], x_cnt, s_sel[3], s_wsum[32];
    extern __shared__ __align__(16) unsigned char cr_smem[];
    int2* siv = reinterpret_cast<int2*>(cr_smem);
    int32_t* spv = reinterpret_cast<int32_t*>(siv + kPathCache);
    // launched as the full sweep's programmatic dependent: the cluster is
    // scheduled while the sweep drains, and waits here for its completion
    // (and its writes) before reading anything
    asm volatile("griddepcontrol.wait;" ::: "memory");
    PhaseScope ps(c.ph, &phl, PH_SWEEP);
    const int rank = cluster_rank(), nctas = cluster_ctas();
    const int m = c.I.m, V = m + c.I.n;
    // the solve's scalars, read by every CTA before any CTA can change them
    const int done0 = c.sc->done;
    int pn = min(max(c.sc->pp_n, 0), kPPRows);
    const int refresh = max(c.sc->pp_refresh, 1);
    const int max_rounds = c.sc->max_rounds;
    int rounds = c.sc->rounds, age = c.sc->pp_age, pivots = c.sc->pivots, ivp = c.sc->ivp, nwide = c.sc->nwide;
    const int pivots0 = pivots;
    const bool partial = c.sc->pricing != 0;
    const int lane = threadIdx.x & 31;
    uint64_t full_best = kNoKey;
    bool optimal = false;
    if (full_first && !done0) {
        // The full round's entering cell and candidate rows (the full sweep
        // has just priced every row): select_candidate_rows' rule over the
        // cluster.  CTA q takes a contiguous range of rows, a thread a
        // contiguous chunk of it (row order = thread order); the smallest
        // key value, the 32-bin histogram and the kept rows' counts are
        // combined across the CTAs through distributed shared memory.
        const int ncols = c.I.n;
        const int per = (m + nctas - 1) / nctas, r0 = min(m, rank * per), r1 = min(m, r0 + per);
        const int chunk = (r1 - r0 + (int)blockDim.x - 1) / (int)blockDim.x;
        const int t0 = min(r1, r0 + (int)threadIdx.x * chunk), t1 = min(r1, t0 + chunk);
        uint64_t pb = kNoKey;
        int32_t rmn = 0;
        int bad = 0;
        for (int i = t0; i < t1; i++) {
            const uint64_t k = c.row_best[i];
            const int32_t v = key_val(k);
            rmn = min(rmn, v);
            if (k != kNoKey && v < 0) {
                if ((int)key_idx(k) >= ncols) { bad = 1; continue; }
                const uint64_t P = pack_i32(v, (uint32_t)i);
                pb = P < pb ? P : pb;
            }
        }
        if (bad) fail_check(c.sc, 18);
        pb = block_min_u64(pb, bs);
        rmn = key_val(block_min_u64(pack_i32(rmn, 0u), bs));
        if (threadIdx.x == 0) { x_best = pb; x_rmin = rmn; }
        if (threadIdx.x < 32) x_hist[threadIdx.x] = 0;
        cluster_sync_all();                                      // selection barrier 1
        if (threadIdx.x < 32) {
            const uint64_t b = warp_min_u64(lane < nctas ? dsmem_ld_u64(dsmem_of(&x_best, lane)) : kNoKey);
            int32_t rq = 0;
            if (lane < nctas) {
                uint32_t a = dsmem_of(&x_rmin, lane), r;
                asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(r) : "r"(a) : "memory");
                rq = (int32_t)r;
            }
            const int32_t rm = key_val(warp_min_u64(pack_i32(rq, 0u)));
            if (lane == 0) { s_red[0] = b; s_sel[0] = rm; }
        }
        __syncthreads();
        full_best = s_red[0];
        const int32_t rmin = s_sel[0];
        const int64_t span = rmin < 0 ? -(int64_t)rmin : 1;
        if (rmin < 0)
            for (int i = t0; i < t1; i++) {
                const int32_t v = key_val(c.row_best[i]);
                if (v < 0) atomicAdd(&x_hist[((int64_t)v - rmin) * 32 / span], 1);
            }
        __syncthreads();
        cluster_sync_all();                                      // selection barrier 2: every histogram complete
        const int cap = min(max(c.sc->pp_rows, 1), kPPRows);
        if (threadIdx.x < 32) {
            int h = 0;
            for (int q = 0; q < nctas; q++) {
                uint32_t a = dsmem_of(&x_hist[lane], q), r;
                asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(r) : "r"(a) : "memory");
                h += (int)r;
            }
            s_wsum[lane] = h;
            __syncwarp();
            if (lane == 0) {
                int last = -1;
                if (rmin < 0) {
                    int cum = s_wsum[0];
                    last = 0;
                    for (int b = 1; b < 32 && cum + s_wsum[b] <= cap; b++) { cum += s_wsum[b]; last = b; }
                }
                s_sel[1] = last;
            }
        }
        __syncthreads();
        const int last = s_sel[1];
        // this thread's kept rows, then their positions in row order
        int mine = 0;
        if (last >= 0)
            for (int i = t0; i < t1; i++) {
                const int32_t v = key_val(c.row_best[i]);
                mine += v < 0 && ((int64_t)v - rmin) * 32 / span <= last;
            }
        int incl = mine;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        if (lane == 31) s_wsum[w] = incl;
        __syncthreads();
        if (threadIdx.x < 32) {
            int x = lane < nw ? s_wsum[lane] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane < nw) s_wsum[lane] = x;              // inclusive per-warp sums
            if (lane == 31) x_cnt = x;                    // this CTA's kept rows
        }
        __syncthreads();
        const int before_w = (w > 0 ? s_wsum[w - 1] : 0) + incl - mine;
        cluster_sync_all();                                      // selection barrier 3: every count complete
        if (threadIdx.x < 32) {
            int cq = 0;
            if (lane < nctas) {
                uint32_t a = dsmem_of(&x_cnt, lane), r;
                asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(r) : "r"(a) : "memory");
                cq = (int)r;
            }
            const int lower = (int)__reduce_add_sync(0xffffffffu, lane < rank ? (unsigned)cq : 0u);
            const int total = (int)__reduce_add_sync(0xffffffffu, (unsigned)cq);
            if (lane == 0) { s_sel[0] = lower; s_sel[2] = total; }
        }
        __syncthreads();
        int slot = s_sel[0] + before_w;
        if (last >= 0)
            for (int i = t0; i < t1; i++) {
                const int32_t v = key_val(c.row_best[i]);
                if (v < 0 && ((int64_t)v - rmin) * 32 / span <= last) {
                    if (slot < cap) c.prow[slot] = i;
                    slot++;
                }
            }
        pn = min(s_sel[2], cap);
        rounds++;                    // the full round
        age = 1;                     // a full sweep resets the age; this round counts
        optimal = full_best == kNoKey;
        cluster_sync_all();                                      // selection barrier 4: every kept row written
    }
    for (int t = threadIdx.x; t < pn; t += blockDim.x) s_prow[t] = c.prow[t];   // visible after barrier 0
    if (rank == 0 && threadIdx.x == 0) { cp->abort[0] = 0; cp->abort[1] = 0; }
    if (threadIdx.x == 0) cp->dwide[rank] = 0;
    const int v0 = rank * blockDim.x + threadIdx.x, stride = nctas * blockDim.x;
    OwnVertex own;
    if (kOne) own_load(c, own, v0, c.iv + (ivp ? V : 0));
    // the path entries' old intervals, written with the entries by the
    // membership step: the pointer-jumping scratch acc0 (8 bytes per
    // vertex), which only the rebuilds use and the cluster rounds never run
    int2* piv = reinterpret_cast<int2*>(c.acc0);
    enum { kRun, kExhausted, kAged, kCapped, kFailed };
    int why = kRun;
    for (int r = 0;; r++) {
        cluster_sync_all();                                      // barrier 0
        if (r > 0) {
            for (int q = 0; q < nctas; q++) nwide += cp->dwide[q];
            if (cp->abort[(r - 1) & 1]) { why = kFailed; break; }
        }
        const bool full_round = full_first && r == 0;   // the same in every CTA
        if (done0 || optimal || (!full_round && (!partial || pn <= 0))) { why = kAged; break; }
        if (!full_round && rounds >= max_rounds) { why = kCapped; break; }
        if (!full_round && age >= refresh) { why = kAged; break; }
        ps.mark(PH_SWEEP);
        int bad = 0;
        if (!full_round) {
            // this CTA's smallest (reduced cost, row), for the cluster's entering cell
            const uint64_t mine = block_min_u64(cluster_cand_sweep(c, s_prow, pn, nwide == 0, rank, nctas, &bad), bs);
            if (threadIdx.x == 0) x_best = mine;
        }
        if (bad) { fail_check(c.sc, 19); cp->abort[r & 1] = 1; }
        cluster_sync_all();                                      // barrier 1
        if (rank == 0 && threadIdx.x == 0 && r > 0) cp->abort[(r - 1) & 1] = 0;   // read by all before barrier 1
        // the entering cell: the full round's, else the smallest (reduced
        // cost, row) over the CTAs' units (distributed shared memory)
        uint64_t best = kNoKey;
        if (full_round) {
            best = full_best;
        } else {
            if (threadIdx.x < 32) {
                const uint64_t b = warp_min_u64(lane < nctas ? dsmem_ld_u64(dsmem_of(&x_best, lane)) : kNoKey);
                if (lane == 0) s_red[0] = b;
            }
            __syncthreads();
            best = s_red[0];
        }
        if (best == kNoKey || !FLOCK_IN((int)key_idx(best), m)) { why = kExhausted; break; }
        if (!full_round) {           // the full round was counted when it was priced
            rounds++;
            age++;
        }
        ps.mark(PH_CYCLE);
        const int k = (int)key_idx(best);
        const int l = m + (int)key_idx(c.row_best[k]);
        const int2* ivA = c.iv + (ivp ? V : 0);
        int2* ivB = c.iv + (ivp ? 0 : V);
        // values the update changes, read before any CTA's update of this round
        const int dk = c.depth[k], dl = c.depth[l];
        const int64_t r_enter = (int64_t)cost_of(c.I, k, l - m) - c.pot[k] - c.pot[l];
        uint64_t mk = kNoKey, ml = kNoKey;
        if (kOne) member_one(c, own, ivA[k].x, ivA[l].x, dk, dl, mk, ml, piv);
        else member_slice(c, ivA, k, l, dk, dl, v0, stride, mk, ml, piv);
        mk = block_min_u64(mk, bs);
        ml = block_min_u64(ml, bs);
        if (threadIdx.x == 0) { x_mk = mk; x_ml = ml; }
        cluster_sync_all();                                      // barrier 2
        ps.mark(PH_ADJUST);
        if (threadIdx.x < 32) {
            const uint64_t a = warp_min_u64(lane < nctas ? dsmem_ld_u64(dsmem_of(&x_mk, lane)) : kNoKey);
            const uint64_t b = warp_min_u64(lane < nctas ? dsmem_ld_u64(dsmem_of(&x_ml, lane)) : kNoKey);
            if (lane == 0) { s_red[0] = a; s_red[1] = b; }
        }
        __syncthreads();
        const uint64_t gmk = s_red[0], gml = s_red[1];
        const bool lside = gml <= gmk;
        const uint64_t fmin = lside ? gml : gmk;
        uint64_t pick = fmin == kNoKey ? (lside ? kNoKey : 0ull)
                                       : kOne ? pick_one(c, own, lside, fmin) : pick_slice(c, lside, fmin, v0, stride);
        pick = lside ? block_min_u64(pick, bs) : block_max_u64(pick, bs);
        if (threadIdx.x == 0) x_pick = pick;
        cluster_sync_all();                                      // barrier 3
        if (threadIdx.x < 32) {
            const uint64_t x = lane < nctas ? dsmem_ld_u64(dsmem_of(&x_pick, lane)) : (lside ? kNoKey : 0ull);
            const uint64_t y = lside ? warp_min_u64(x) : warp_max_u64(x);
            if (lane == 0) s_red[0] = y;
        }
        __syncthreads();
        const uint64_t q64 = s_red[0];
        const int q = (int)(uint32_t)q64;
        const int e = lside ? l : k, other = lside ? k : l;
        const int de = lside ? dl : dk;
        const int t = fmin != kNoKey && (lside ? q64 != kNoKey : q64 != 0) && FLOCK_IN(q, V)
                          ? de - (int)(uint32_t)(q64 >> 32) : -1;
        const int slot = lside ? V - 1 - t : t;
        if (!FLOCK_IN(t, V) || c.path[slot] != q) {               // the same outcome in every CTA
            if (rank == 0 && threadIdx.x == 0) fail_check(c.sc, 17);
            why = kFailed;
            break;
        }
        PivotParams pp;
        pp.t = t; pp.e = e; pp.other = other; pp.de = de; pp.dother = lside ? dk : dl;
        pp.eside = lside ? 2 : 1;
        pp.th = (int64_t)(fmin ^ 0x8000000000000000ull);
        pp.r = r_enter;
        pp.Q = ivA[q];            // intervals of the old buffer: no CTA writes it this round
        pp.O = ivA[other];
        // e's chain p_0..p_t and its old intervals, for the binary searches
        const bool cached = t < kPathCache;
        if (cached) {
            const int base = lside ? V - 1 : 0, dir = lside ? -1 : 1;
            for (int i = threadIdx.x; i <= t; i += blockDim.x) {
                spv[i] = c.path[base + dir * i];
                siv[i] = piv[base + dir * i];      // written with the path entry (ivA of it)
            }
        }
        if (threadIdx.x == 0) bs.i[7] = 0;
        __syncthreads();
        int dwide = 0, ubad = 0;
        if (kOne) update_one(c, pp, own, ivA, ivB, dwide, ubad, cached ? spv : nullptr, cached ? siv : nullptr);
        else update_slice(c, pp, ivA, ivB, v0, stride, dwide, ubad, cached ? spv : nullptr, cached ? siv : nullptr);
        if (ubad) { fail_check(c.sc, 24); cp->abort[r & 1] = 1; }
        if (dwide) atomicAdd(&bs.i[7], dwide);
        __syncthreads();
        if (threadIdx.x == 0) cp->dwide[rank] = bs.i[7];
        // the keys read by every CTA before barrier 2, cleared for the next
        // sweep: every row's after the full round, else the candidates'
        if (full_round) {
            for (int i = v0; i < m; i += stride) c.row_best[i] = kNoKey;
        } else if (rank == 0) {
            for (int t2 = threadIdx.x; t2 < pn; t2 += blockDim.x) {
                const int i = s_prow[t2];
                if (FLOCK_IN(i, m)) c.row_best[i] = kNoKey;
            }
        }
        ivp ^= 1;
        pivots++;
    }
    // every CTA leaves the loop at the same point; none exits while another
    // may still read its shared variables or the candidate keys
    cluster_sync_all();
    // CTA 0 writes the scalars back
    if (why == kExhausted) {
        if (rank == 0)
            for (int t2 = threadIdx.x; t2 < pn; t2 += blockDim.x) {
                const int i = s_prow[t2];
                if (FLOCK_IN(i, m)) c.row_best[i] = kNoKey;
            }
    }
    if (rank == 0 && threadIdx.x == 0 && !done0) {
        if (full_first) {            // the full round's selection (select_candidate_rows' scalars)
            c.sc->pp_n = pn;
            c.sc->ncand = optimal ? 0 : 1;
            if (optimal) c.sc->done = 1;
        }
        c.sc->rounds = rounds;
        c.sc->pp_age = why == kExhausted ? refresh : age;     // the next round sweeps every row
        c.sc->pivots = pivots;
        c.sc->ivp = ivp;
        c.sc->nwide = nwide;
        c.sc->narrow = nwide == 0;
        if (pivots > pivots0) c.sc->last_winners = 1;
        if (why == kCapped) { c.sc->status |= ST_ITER_CAP; c.sc->done = 1; }
    }
    ps.mark(PH_SWEEP);       // the next full round's sweep
}

__global__ void __launch_bounds__(1024, 1) k_finalize(Ctx c) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    PhaseScope ps(c.ph, &phl, PH_IDLE);   // closes the loop's last phase
    if (c.sc->status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE)) return;
    finalize_cta(c, bs);
    certify_flows_cta(c, bs);
}

__global__ void __launch_bounds__(256) k_cert_cells(Ctx c) {
    if (c.sc->status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE)) return;
    const InstDev& I = c.I;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    unsigned long long neg = 0;
    for (int i = blockIdx.x * wpb + warp; i < I.m; i += gridDim.x * wpb) {
        const int4* row = reinterpret_cast<const int4*>(I.cost + (size_t)i * I.ldc);
        const int64_t u = c.pot[i];
        for (int q = lane; q * 4 < I.n; q += 32) {
            const int4 cv = row[q];
            const int32_t cc[4] = {cv.x, cv.y, cv.z, cv.w};
            for (int e = 0; e < 4; e++)
                if (q * 4 + e < I.n) neg += ((int64_t)cc[e] - u - c.pot[I.m + q * 4 + e]) < 0;
        }
    }
    for (int o = 16; o > 0; o >>= 1) neg += __shfl_xor_sync(0xffffffffu, neg, o);
    if (lane == 0 && neg) {
        atomicAdd((unsigned long long*)&c.sc->neg_cells, neg);
        atomicOr(&c.sc->cert, 8);
    }
}


// int32 column duals and the narrow flag from pot[] (benchmark hook: the
// solver publishes them from the dual recompute).
__global__ void __launch_bounds__(1024) k_publish_duals(Ctx c) {
    const int m = c.I.m, n = c.I.n;
    int wide = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) c.v32[j] = narrow_dual(c.pot[m + j], wide);
    wide = __syncthreads_or(wide);
    if (threadIdx.x == 0) c.sc->narrow = !wide;
}

// Test hook: the CTA-local sweep on one instance (one block).
__global__ void __launch_bounds__(1024) k_sweep_cta_only(Ctx c) { sweep_cta(c); }

__global__ void k_fill_bench(int32_t* cost, size_t cells, int64_t* pot, int V) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < cells; k += (size_t)gridDim.x * blockDim.x)
        cost[k] = (int32_t)((k * 2654435761u) % 1414u);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < (size_t)V; k += (size_t)gridDim.x * blockDim.x)
        pot[k] = (int64_t)((k * 40503u) % 700u);
}

// L2 read bandwidth: `passes` grid-stride passes over an L2-resident buffer,
// L1 bypassed (ld.global.cg), four independent 16-byte loads in flight per
// thread.  The xor of what was read is written only if it matches a value no
// fill produces, so the loads cannot be dropped.
__global__ void __launch_bounds__(512) k_l2_read(const int4* buf, size_t n4, int passes, int* sink) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    int acc = 0;
    for (int p = 0; p < passes; p++) {
        size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
        for (; k + 3 * stride < n4; k += 4 * stride) {
            const int4 a = __ldcg(buf + k), b = __ldcg(buf + k + stride);
            const int4 c = __ldcg(buf + k + 2 * stride), d = __ldcg(buf + k + 3 * stride);
            acc ^= a.x ^ a.y ^ a.z ^ a.w ^ b.x ^ b.y ^ b.z ^ b.w ^ c.x ^ c.y ^ c.z ^ c.w ^ d.x ^ d.y ^ d.z ^ d.w;
        }
        for (; k < n4; k += stride) {
            const int4 a = __ldcg(buf + k);
            acc ^= a.x ^ a.y ^ a.z ^ a.w;
        }
    }
    if (acc == 0x7fffabcd) *sink = acc;
}


// ------------------------------------------------------- batched kernels ---
// The batched form runs many instances side by side, one CTA per instance at
// a time, with work stealing over a size bucket's instance list:
//   k_bsetup  Vogel (or NW corner) and the strongly feasible start tree, per
//             instance, in the instance's global working set
//   k_bround  ONE pricing round of every active instance: the tree arrays are
//             staged into shared memory, duals recomputed, the CTA-local sweep
//             and the deconflicted pivots run there, and parent/flow/duals are
//             written back; the host captures chunks of rounds in a CUDA graph
//   k_bfinal  original flows, objective and the exact certificate
__device__ __forceinline__ bool batch_desc_ok(const BatchArgs& a, const BatchDesc& d) {
    return d.m >= 1 && d.n >= 1 && d.m + d.n <= a.maxV && d.m <= a.maxM && d.ldc >= d.n && !(d.ldc & 3) &&
           !((uintptr_t)d.cost & 15) && !((uintptr_t)d.ws & 255) && d.sd && d.out && d.bfs && d.pot && d.sc;
}

__device__ __forceinline__ void batch_ctx(const BatchArgs& a, const BatchDesc& d, Ctx& g) {
    const int V1 = d.m + d.n - 1;
    g.I.m = d.m; g.I.n = d.n; g.I.ldc = d.ldc;
    g.I.cost = d.cost;
    g.I.supply = d.sd;
    g.I.demand = d.sd + d.m;
    g.sc = d.sc;
    g.out_src = d.out; g.out_dst = d.out + V1; g.out_qty = d.out + 2 * V1;
    carve_ctx(g, d.ws, d.m + d.n, d.m, nullptr, d.pot);
}

// returns the next instance of this launch for the CTA, or -1
__device__ __forceinline__ int batch_next(const BatchArgs& a, int* s_idx) {
    if (threadIdx.x == 0) *s_idx = atomicAdd(a.next, 1);
    __syncthreads();
    const int idx = *s_idx;
    __syncthreads();
    return idx < a.count ? idx : -1;
}

// Shared-memory staging of the setup: the initial allocation list (kept from
// Vogel to the start tree), then Vogel's per-line arrays or, in the same
// space once Vogel is done, the start tree's scratch, parents and depths.
// setup_stage_bytes() below follows the same carving.
struct SetupStage {
    template <class K> __host__ __device__ static void list(Ctx& c, K& k, int V) {
        c.bfs_src = (int32_t*)k.S(4 * (size_t)V);
        c.bfs_dst = (int32_t*)k.S(4 * (size_t)V);
        c.bfs_qty = (int32_t*)k.S(4 * (size_t)V);
    }
    template <class K> __host__ __device__ static void vogel(Ctx& c, K& k, int V) {
        c.top2 = (int4*)k.S(16 * (size_t)V);
        c.diff = (int32_t*)k.S(4 * (size_t)V);
        c.res = (int32_t*)k.S(4 * (size_t)V);
        c.rescan = (int32_t*)k.S(4 * (size_t)V);
        c.covered = (uint8_t*)k.S((size_t)V);
    }
    template <class K> __host__ __device__ static void tree(Ctx& c, K& k, int V) {
        c.bsum = (int64_t*)k.S(8 * (size_t)V);
        c.csr_adj = (int32_t*)k.S(8 * (size_t)V);
        c.csr_start = (int32_t*)k.S(4 * ((size_t)V + 1));
        c.order = (int32_t*)k.S(4 * (size_t)V);
        c.uf = (int32_t*)k.S(4 * (size_t)V);
        c.parent = (int32_t*)k.S(4 * (size_t)V);
        c.depth = (int32_t*)k.S(4 * (size_t)V);
    }
};

inline size_t setup_stage_bytes(int V) {
    Ctx c;
    Carver k{nullptr, 0, (unsigned char*)16, 0};
    SetupStage::list(c, k, V);
    Carver kv = k, kt = k;
    SetupStage::vogel(c, kv, V);
    SetupStage::tree(c, kt, V);
    return (std::max(kv.so, kt.so) + 15) & ~size_t(15);
}

// Initial solution and strongly feasible start tree of one instance.  With
// kStage the working arrays live in shared memory (the persistent kernel's
// dynamic block, free until the rounds stage the tree) and the parents are
// copied to the instance's working set at the end; else everything is in
// the working set.
template <bool kStage>
__device__ __forceinline__ void bsetup_one(const BatchArgs& a, const BatchDesc& d, BlockScratch& bs,
                                           unsigned char* smem, PhaseScope* ps = nullptr) {
    Ctx c;
    batch_ctx(a, d, c);
    const Ctx g = c;
    const int V = d.m + d.n;
    Carver k{nullptr, 0, smem, 0};
    if (kStage) {
        SetupStage::list(c, k, V);
        Carver kv = k;
        SetupStage::vogel(c, kv, V);
    }
    if (threadIdx.x == 0) {
        Scalars z;
        memset(&z, 0, sizeof(z));
        z.max_rounds = a.max_rounds;
        z.mode = a.mode;
        z.pricing = a.pricing;
        const bool small = d.m + d.n <= kPPSmallV;
        z.pp_rows = min(max(small ? a.pp[0] : a.pp[2], 1), kPPRows);
        z.pp_refresh = max(small ? a.pp[1] : a.pp[3], 1);
        *c.sc = z;
    }
    __syncthreads();
    if (a.bfs_method == FLOCK_BFS_VOGEL) {
        vogel_cta(c, bs);
    } else {
        if (threadIdx.x == 0) nwc_thread0(c);
        __syncthreads();
    }
    if (threadIdx.x == 0 && c.sc->events < 0) c.sc->status |= ST_VOGEL_UNDEF;
    if (ps) ps->mark(PH_DUAL);    // the start tree and its duals
    for (int q = threadIdx.x; q < V - 1; q += blockDim.x) {
        d.bfs[3 * q + 0] = c.bfs_src[q];
        d.bfs[3 * q + 1] = c.bfs_dst[q];
        d.bfs[3 * q + 2] = c.bfs_qty[q];
    }
    __syncthreads();
    if (kStage) {
        Carver kt = k;
        SetupStage::tree(c, kt, V);
    }
    sf_init_cta(c, bs);
    if (kStage) {
        for (int v = threadIdx.x; v < V; v += blockDim.x) g.parent[v] = c.parent[v];
    }
    __syncthreads();
}

__device__ __forceinline__ void bdesc_reject(const BatchArgs& a, const BatchDesc& d) {
    if (threadIdx.x == 0 && d.sc) { d.sc->status = ST_TREE_CORRUPT; d.sc->fail_site = 1; d.sc->done = 1; }
}

__global__ void __launch_bounds__(256) k_bsetup(BatchArgs a) {
    __shared__ BlockScratch bs;
    __shared__ int s_idx;
    for (int idx; (idx = batch_next(a, &s_idx)) >= 0;) {
        const BatchDesc d = a.desc[idx];
        if (!batch_desc_ok(a, d)) { bdesc_reject(a, d); continue; }
        bsetup_one<false>(a, d, bs, nullptr);
    }
}

// Shared-memory staging of the arrays every pivot step touches: the tree,
// the duals, the row keys and the preorder intervals; unless kLight (the
// largest instances), also the single pivot's cycle chains and their
// flows.  The edge claims of multi-pivot rounds and the pointer-jumping
// block of the rebuilds (the first round and the rounds after multi-pivot
// rounds) stay in the instance's global working set, which keeps the staged
// block small enough for several instances per SM.  Every pointer is carved
// from the extern shared base and the flag is a compile-time constant, so
// the compiler knows they address shared memory (shared loads and atomics
// rather than generic ones).  staged_bytes() below follows the same order.
template <bool kLight>
__device__ __forceinline__ void stage_hot(Ctx& c, unsigned char* smem, int V, int M) {
    Carver k{nullptr, 0, smem, 0};
    c.parent = (int32_t*)k.S(4 * (size_t)V);
    c.depth = (int32_t*)k.S(4 * (size_t)V);
    c.flow = (int64_t*)k.S(8 * (size_t)V);
    c.row_best = (uint64_t*)k.S(8 * (size_t)M);
    c.pot = (int64_t*)k.S(8 * (size_t)V);
    c.v32 = (int32_t*)k.S(4 * (size_t)V);
    c.iv = (int2*)k.S(16 * (size_t)V);
    if (kLight) return;
    c.pflow = (int64_t*)k.S(8 * (size_t)V);
    c.path = (int32_t*)k.S(4 * (size_t)V);
}

// Rounds staging; the launch's dynamic block also holds the staged setup
// (launch_smem_bytes).
inline size_t staged_bytes(int V, int M, bool light) {
    Carver k{nullptr, 0, (unsigned char*)16, 0};
    k.S(4 * (size_t)V); k.S(4 * (size_t)V); k.S(8 * (size_t)V); k.S(8 * (size_t)M); k.S(8 * (size_t)V);
    k.S(4 * (size_t)V); k.S(16 * (size_t)V);
    if (!light) { k.S(8 * (size_t)V); k.S(4 * (size_t)V); }
    return (k.so + 15) & ~size_t(15);
}

inline size_t launch_smem_bytes(int V, int M, bool light) {
    return std::max(staged_bytes(V, M, light), setup_stage_bytes(V));
}

// Largest dynamic shared memory a staged launch may use (the 227 KB of a
// block less the kernels' static BlockScratch and work-stealing slot).
constexpr size_t kStageSmemMax = 225 * 1024;

// Staging of a launch whose largest instance is maxV x (rows maxM): full
// whenever it fits.
inline bool stage_light(int maxV, int maxM) { return staged_bytes(maxV, maxM, false) > kStageSmemMax; }

// Pricing rounds of one instance with its tree staged in shared memory:
// `max_here` rounds at most (1 for the round-kernel form), or until done.
// The staged state starts from parent[] and flow[] (a rebuild in the first
// round); single pivots keep it current, multi-pivot rounds mark it stale.
template <bool kLight>
__device__ void brounds_one(const BatchArgs& a, const BatchDesc& d, BlockScratch& bs, unsigned char* smem,
                            int max_here, PhaseScope* ps = nullptr) {
    Ctx g;
    batch_ctx(a, d, g);
    Ctx c = g;
    stage_hot<kLight>(c, smem, a.maxV, a.maxM);
    const int V = d.m + d.n;
    for (int v = threadIdx.x; v < V; v += blockDim.x) { c.parent[v] = g.parent[v]; c.flow[v] = g.flow[v]; }
    if (threadIdx.x == 0) c.sc->stale = 1;
    __syncthreads();
    for (int r = 0; r < max_here; r++) {
        if (c.sc->stale) {
            if (ps) ps->mark(PH_DUAL);
            tree_build_cta(c, bs);
        }
        if (!c.sc->done) {
            if (ps) ps->mark(PH_SWEEP);
            uint64_t entering = kNoKey;
            const bool partial = c.sc->pricing != 0;
            if (partial) entering = sweep_partial_cta(c, bs);
            else sweep_cta(c);
            pivot_round_cta(c, bs, partial, entering, ps);
        }
        if (threadIdx.x == 0) {
            c.sc->rounds++;
            if (!c.sc->done && c.sc->rounds >= c.sc->max_rounds) { c.sc->status |= ST_ITER_CAP; c.sc->done = 1; }
            if (!c.sc->done && a.active && r + 1 == max_here) atomicAdd(a.active, 1);
        }
        __syncthreads();
        if (c.sc->done) break;       // written before the barrier: every thread reads the same value
    }
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        g.parent[v] = c.parent[v]; g.flow[v] = c.flow[v]; g.pot[v] = c.pot[v];
    }
    __syncthreads();
}

__device__ void bfinal_one(const BatchArgs& a, const BatchDesc& d, BlockScratch& bs) {
    if (d.sc->status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE)) return;   // uniform
    Ctx c;
    batch_ctx(a, d, c);
    finalize_cta(c, bs);
    certify_flows_cta(c, bs);
    certify_cells_cta(c, bs);
    __syncthreads();
}

__global__ void __launch_bounds__(256) k_bround(BatchArgs a) {
    __shared__ BlockScratch bs;
    __shared__ int s_idx;
    extern __shared__ __align__(16) unsigned char smem[];
    for (int idx; (idx = batch_next(a, &s_idx)) >= 0;) {
        const BatchDesc d = a.desc[idx];
        if (!batch_desc_ok(a, d)) continue;
        if (d.sc->done) continue;          // every thread reads the same value
        if (a.light) brounds_one<true>(a, d, bs, smem, 1);
        else brounds_one<false>(a, d, bs, smem, 1);
    }
}

__global__ void __launch_bounds__(256) k_bfinal(BatchArgs a) {
    __shared__ BlockScratch bs;
    __shared__ int s_idx;
    for (int idx; (idx = batch_next(a, &s_idx)) >= 0;) {
        const BatchDesc d = a.desc[idx];
        if (!batch_desc_ok(a, d)) continue;
        bfinal_one(a, d, bs);
    }
}

// Served form: after the instance's results are in device memory, raise its
// completion flag in host-mapped memory (the host polls it, then copies).
__device__ __forceinline__ void publish_done(const BatchDesc& d) {
    __syncthreads();
    if (threadIdx.x == 0 && d.done) {
        __threadfence_system();
        *(volatile int32_t*)d.done = 1;
    }
}

// Persistent form: a CTA takes the next instance of the bucket (largest
// first) and runs it from the initial solution to the certificate, all
// pricing rounds inside with the tree resident in shared memory.
template <int kThreads, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_bsolve(BatchArgs a) {
    __shared__ BlockScratch bs;
    __shared__ int s_idx;
    extern __shared__ __align__(16) unsigned char smem[];
    for (int idx; (idx = batch_next(a, &s_idx)) >= 0;) {
        const BatchDesc d = a.desc[idx];
        if (!batch_desc_ok(a, d)) { bdesc_reject(a, d); publish_done(d); continue; }
        bsetup_one<true>(a, d, bs, smem);
        if (!d.sc->done) {
            if (a.light) brounds_one<true>(a, d, bs, smem, 1 << 30);
            else brounds_one<false>(a, d, bs, smem, 1 << 30);
        }
        bfinal_one(a, d, bs);
        publish_done(d);
    }
}

// The plain solver's one-launch form (instances below the grid-round size):
// one CTA runs the persistent kernel's work on a single instance -- initial
// solution, start tree, every pricing round with the tree staged in shared
// memory, retrieval and the certificate -- and keeps the phase clock.
template <int kThreads>
__global__ void __launch_bounds__(kThreads, 1) k_solve_one(BatchArgs a) {
    __shared__ BlockScratch bs;
    __shared__ PhaseLocal phl;
    extern __shared__ __align__(16) unsigned char smem[];
    PhaseScope ps(a.ph, &phl, PH_BFS);
    BatchDesc d = a.desc[0];
    if (!batch_desc_ok(a, d)) { bdesc_reject(a, d); return; }
    if (a.cost_smem > 0) {      // the whole matrix (m rows of ldc) fits beside the staging: read it from there
        int32_t* cs = reinterpret_cast<int32_t*>(smem + a.cost_smem);
        stage_i32(cs, d.cost, d.m * d.ldc);
        __syncthreads();
        d.cost = cs;
    }
    bsetup_one<true>(a, d, bs, smem, &ps);
    if (!d.sc->done) {
        if (a.light) brounds_one<true>(a, d, bs, smem, 1 << 30, &ps);
        else brounds_one<false>(a, d, bs, smem, 1 << 30, &ps);
    }
    ps.mark(PH_IDLE);
    bfinal_one(a, d, bs);
}

// Block size of the one-launch form by instance size (FLOCK_PLAIN_THREADS=128,
// 256 or 1024 overrides it, for tuning; 128 runs the 256-thread kernel).
static int solve_one_threads(int V) {
    const char* e = getenv("FLOCK_PLAIN_THREADS");
    if (e && (!strcmp(e, "128") || !strcmp(e, "256") || !strcmp(e, "1024"))) return atoi(e);
    return V <= 512 ? 256 : 1024;
}
static const void* solve_one_fn(int threads) {
    return threads <= 256 ? (const void*)k_solve_one<256> : (const void*)k_solve_one<1024>;
}

// The persistent kernel compiled for the block size: up to 256 threads four
// blocks per SM (64 registers), 512 two, 1024 one.
static const void* bsolve_fn(int threads) {
    if (threads <= 256) return (const void*)k_bsolve<256, 4>;
    if (threads <= 512) return (const void*)k_bsolve<512, 2>;
    return (const void*)k_bsolve<1024, 1>;
}

}  // namespace flock

// =================================================================== host ===
namespace flock {

static thread_local std::string g_err;
void set_error(const std::string& s) { g_err = s; }
static int cuda_fail(const char* what, cudaError_t e) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return FLOCK_ERR_CUDA;
}
#define FLOCK_CK(x) do { cudaError_t _e = (x); if (_e != cudaSuccess) return cuda_fail(#x, _e); } while (0)

static int num_sms() {
    static int s = 0;
    if (!s) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
        if (s <= 0) s = 1;
    }
    return s;
}

struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr; cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <class T> T* as(size_t byte_off = 0) const { return (T*)((char*)p + byte_off); }
};
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr; cap = 0;
        cudaError_t e = cudaMallocHost(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <class T> T* as(size_t byte_off = 0) const { return (T*)((char*)p + byte_off); }
};

static size_t al256(size_t x) { return (x + 255) & ~size_t(255); }
static const int32_t kFailMask = ST_ITER_CAP | ST_TREE_CORRUPT | ST_SF_FAIL | ST_CERT_FAIL | ST_RANGE;

// Every check of validate_instance except the per-cost range check.
static int validate_shape(const flock_instance* I, std::string* msg) {
    if (!I || !I->supply || !I->demand || !I->cost || I->m < 1 || I->n < 1) { *msg = "invalid instance"; return FLOCK_ERR_ARG; }
    if ((int64_t)I->m + I->n > (1 << 28) || (int64_t)I->m * I->n > ((int64_t)1 << 34)) { *msg = "instance too large"; return FLOCK_ERR_RANGE; }
    int64_t S = 0, D = 0;
    for (int i = 0; i < I->m; i++) { if (I->supply[i] < 0) { *msg = "negative supply"; return FLOCK_ERR_ARG; } S += I->supply[i]; }
    for (int j = 0; j < I->n; j++) { if (I->demand[j] < 0) { *msg = "negative demand"; return FLOCK_ERR_ARG; } D += I->demand[j]; }
    if (S != D) { *msg = "unbalanced instance"; return FLOCK_ERR_UNBALANCED; }
    return FLOCK_OK;
}

static bool costs_in_range(const int32_t* c, size_t cnt, int32_t* lo_out = nullptr, int32_t* hi_out = nullptr) {
    int32_t lo = INT32_MAX, hi = INT32_MIN;
    for (size_t k = 0; k < cnt; k++) { lo = std::min(lo, c[k]); hi = std::max(hi, c[k]); }
    if (lo_out) *lo_out = lo;
    if (hi_out) *hi_out = hi;
    return cnt == 0 || (lo >= -(1 << 30) && hi <= (1 << 30));
}

// Copy one cost row and check the accepted range |c| <= 2^30 in the same pass.
static bool copy_costs_checked(int32_t* dst, const int32_t* src, int n) {
    int bad = 0;
    for (int j = 0; j < n; j++) {
        const int32_t v = src[j];
        dst[j] = v;
        bad |= (v > (1 << 30)) | (v < -(1 << 30));
    }
    return !bad;
}

// Host worker pool behind parallel_for.  The workers start once (first use)
// and sleep on a condition variable between jobs, so a batch call's
// validation, packing and result collection start no threads.  One job at a
// time: a caller that finds the pool busy with another host thread's job runs
// its loop alone.  A job is a body that every participant runs (the body
// hands out the work itself); the caller runs it too, then closes the job
// (no worker joins after that) and waits for the workers that joined.
class HostPool {
public:
    static HostPool& get() {
        static HostPool* p = new HostPool();     // never destroyed: its workers sleep until the process exits
        return *p;
    }
    int size() const { return nworkers_ + 1; }
    // Runs body on the caller and up to want - 1 workers; false (nothing run)
    // when another job holds the pool.
    bool try_run(int want, const std::function<void()>& body) {
        std::unique_lock<std::mutex> job(job_mu_, std::try_to_lock);
        if (!job.owns_lock()) return false;
        {
            std::lock_guard<std::mutex> lk(mu_);
            body_ = &body;
            slots_ = std::min(want - 1, nworkers_);
            gen_++;
        }
        cv_.notify_all();
        body();
        std::unique_lock<std::mutex> lk(mu_);
        slots_ = 0;
        done_cv_.wait(lk, [&] { return joined_ == 0; });
        body_ = nullptr;
        return true;
    }

private:
    HostPool() {
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        nworkers_ = std::min(hw, 32) - 1;
        for (int t = 0; t < nworkers_; t++) std::thread([this] { loop(); }).detach();
    }
    void loop() {
        uint64_t seen = 0;
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [&] { return gen_ != seen; });
            seen = gen_;
            if (slots_ <= 0) continue;
            slots_--;
            joined_++;
            const std::function<void()>* b = body_;
            lk.unlock();
            (*b)();
            lk.lock();
            if (--joined_ == 0) done_cv_.notify_all();
        }
    }
    std::mutex job_mu_, mu_;
    std::condition_variable cv_, done_cv_;
    const std::function<void()>* body_ = nullptr;
    uint64_t gen_ = 0;
    int slots_ = 0, joined_ = 0, nworkers_ = 0;
};

// Run f(0..count-1) on up to 32 host threads of the pool (dynamic chunks of 8).
template <class F>
static void parallel_for(int count, const F& f) {
    HostPool& pool = HostPool::get();
    const int nt = std::min(pool.size(), std::max(1, count / 16));
    if (nt <= 1) { for (int k = 0; k < count; k++) f(k); return; }
    std::atomic<int> next{0};
    const std::function<void()> body = [&] {
        for (;;) {
            const int k0 = next.fetch_add(8);
            if (k0 >= count) return;
            for (int k = k0; k < std::min(count, k0 + 8); k++) f(k);
        }
    };
    if (!pool.try_run(nt, body)) body();
}

// Shape and cost checks; with fits16, whether every cost fits in 16 bits.
static int validate_instance_range(const flock_instance* I, bool* fits16) {
    std::string msg;
    const int rc = validate_shape(I, &msg);
    if (rc) { set_error(msg); return rc; }
    int32_t lo = 0, hi = 0;
    if (!costs_in_range(I->cost, (size_t)I->m * I->n, &lo, &hi)) { set_error("cost out of range"); return FLOCK_ERR_RANGE; }
    if (fits16) *fits16 = lo >= INT16_MIN && hi <= INT16_MAX;
    return FLOCK_OK;
}
int validate_instance(const flock_instance* I) { return validate_instance_range(I, nullptr); }

// Scalars::mode of a pivot method: 0 sequential, 1 parallel, 2 switch, 3
// parallel stepping stone.
static int pivot_mode(const flock_options& o) {
    switch (o.pivot_method) {
        case FLOCK_PIVOT_SEQUENTIAL: return 0;
        case FLOCK_PIVOT_PARALLEL: return 1;
        case FLOCK_PIVOT_SS: return 3;
        default: return 2;
    }
}

// BatchArgs::pp: the partial-pricing settings of the block forms
// (kPPRowsSmall, kPPRefreshSmall, kPPRowsLarge, kPPRefreshLarge);
// FLOCK_BPP="r,k,R,K" overrides them, for tuning.
static void block_pricing(int32_t* pp) {
    pp[0] = kPPRowsSmall; pp[1] = kPPRefreshSmall; pp[2] = kPPRowsLarge; pp[3] = kPPRefreshLarge;
    if (const char* e = getenv("FLOCK_BPP")) {
        int v[4];
        if (sscanf(e, "%d,%d,%d,%d", &v[0], &v[1], &v[2], &v[3]) == 4)
            for (int k = 0; k < 4; k++) pp[k] = v[k];
    }
}

// Scalars::pricing of the options: partial pricing unless FULL was asked for
// or the pivot method prices every cell (parallel stepping stone).
static int pricing_of(const flock_options& o) {
    return o.pricing == FLOCK_PRICING_PARTIAL && o.pivot_method != FLOCK_PIVOT_SS ? 1 : 0;
}

static int threads_for(int V) {
    int t = ((V + 31) / 32) * 32;
    return std::max(128, std::min(1024, t));
}

// --------------------------------------------------------- plain solver ----
struct PlainSolver {
    std::mutex mu;
    DevBuf ws, cost, sd;
    DevBuf books;                   // "vam_device" Vogel: row and column books
    DevBuf costT;                   // Vogel's column-major copy of the costs
    DevBuf cost16;                  // grid path: 16-bit copy of the costs for the sweeps
    DevBuf one;                     // one-launch form: working set, basis, duals, scalars, descriptor
    HostBuf h_one;                  // one-launch form: pinned staging of its upload and download regions
    GridPivot* gp = nullptr;        // grid pivot round state (large instances)
    PhaseClock* ph = nullptr;       // device time per simplex phase
    ClusterPivot* cp = nullptr;     // cluster rounds' per-CTA slots
    int cluster_ctas = 0;           // CTAs of the cluster rounds (0: the six-kernel rounds only)
    HostBuf h_sc;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    bool init = false;

    int setup() {
        if (init) return FLOCK_OK;
        FLOCK_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        for (auto& e : ev) FLOCK_CK(cudaEventCreate(&e));
        FLOCK_CK(h_sc.ensure(sizeof(Scalars)));
        FLOCK_CK(cudaFuncSetAttribute(k_books, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(sizeof(uint64_t) * 16384)));
        for (int t : {256, 1024})
            FLOCK_CK(cudaFuncSetAttribute(solve_one_fn(t), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)kStageSmemMax));
        FLOCK_CK(cudaFuncSetAttribute(k_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBulkSmem));
        FLOCK_CK(cudaFuncSetAttribute(k_setup, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kVogelStageMax));
        FLOCK_CK(cudaFuncSetAttribute(k_vogel_only, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kVogelStageMax));
        // the largest cluster the cluster rounds can be launched with (one cluster)
        cluster_ctas = 0;
        if (cudaFuncSetAttribute(k_cround<true>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            cudaFuncSetAttribute(k_cround<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCRoundSmem) ==
                cudaSuccess &&
            cudaFuncSetAttribute(k_cround<false>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess &&
            cudaFuncSetAttribute(k_cround<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCRoundSmem) ==
                cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(kClusterMax);
            cfg.blockDim = dim3(kCRoundThreads);
            cfg.dynamicSmemBytes = kCRoundSmem;
            int cs = 0, cs1 = 0;
            if (cudaOccupancyMaxPotentialClusterSize(&cs, (const void*)k_cround<false>, &cfg) == cudaSuccess &&
                cudaOccupancyMaxPotentialClusterSize(&cs1, (const void*)k_cround<true>, &cfg) == cudaSuccess)
                cluster_ctas = std::min(std::min(cs, cs1), kClusterMax);
        }
        if (cluster_ctas < 2) cluster_ctas = 0;
        cudaGetLastError();
        init = true;
        return FLOCK_OK;
    }

    // Sort the "vam_device" Vogel's books of the prepared instance on the
    // stream (rows' books first, then the columns').
    int build_books(const Ctx& c, int2** rb, int2** cb) {
        const int m = c.I.m, n = c.I.n;
        if (m > kBookLineMax || n > kBookLineMax) {
            set_error("vam_device Vogel: a line longer than 16382 cells");
            return FLOCK_ERR_RANGE;
        }
        FLOCK_CK(books.ensure(book_entries(m, n) * sizeof(int2)));
        *rb = books.as<int2>();
        *cb = *rb + (size_t)m * (n + 2);
        int P = 1;
        while (P < std::max(m, n) + 2) P <<= 1;
        k_books<<<m + n, kBookThreads, sizeof(uint64_t) * P, stream>>>(c.I, *rb, *cb, P);
        FLOCK_CK(cudaGetLastError());
        return FLOCK_OK;
    }

    // Upload the instance and lay out the working set.
    int prepare(const flock_instance* I, Ctx& c, int32_t** out3) {
        const int m = I->m, n = I->n, V = m + n;
        const int ldc = (n + 3) & ~3;
        FLOCK_CK(cost.ensure((size_t)m * ldc * 4 + 16));
        FLOCK_CK(sd.ensure((size_t)V * 4));
        size_t gbytes = 0;
        Ctx probe;
        carve_ctx(probe, nullptr, V, m, nullptr, nullptr, nullptr, &gbytes);
        const size_t extra_off = al256(gbytes);
        const size_t out_bytes = al256((size_t)3 * V * 4);
        FLOCK_CK(ws.ensure(extra_off + out_bytes + al256(sizeof(Scalars)) + al256(sizeof(GridPivot)) +
                           al256(sizeof(PhaseClock)) + al256(sizeof(ClusterPivot))));
        carve_ctx(c, ws.as<uint8_t>(), V, m, nullptr, nullptr);
        gp = ws.as<GridPivot>(extra_off + out_bytes + al256(sizeof(Scalars)));
        ph = ws.as<PhaseClock>(extra_off + out_bytes + al256(sizeof(Scalars)) + al256(sizeof(GridPivot)));
        cp = ws.as<ClusterPivot>(extra_off + out_bytes + al256(sizeof(Scalars)) + al256(sizeof(GridPivot)) +
                                 al256(sizeof(PhaseClock)));
        c.out_src = ws.as<int32_t>(extra_off);
        c.out_dst = c.out_src + V;
        c.out_qty = c.out_dst + V;
        *out3 = c.out_src;
        c.sc = ws.as<Scalars>(extra_off + out_bytes);
        c.I.m = m; c.I.n = n; c.I.ldc = ldc;
        c.I.cost = cost.as<int32_t>();
        c.I.supply = sd.as<int32_t>();
        c.I.demand = sd.as<int32_t>() + m;
        FLOCK_CK(cudaMemcpy2DAsync(cost.p, (size_t)ldc * 4, I->cost, (size_t)n * 4, (size_t)n * 4, m,
                                   cudaMemcpyHostToDevice, stream));
        FLOCK_CK(cudaMemcpyAsync(sd.p, I->supply, (size_t)m * 4, cudaMemcpyHostToDevice, stream));
        FLOCK_CK(cudaMemcpyAsync(sd.as<int32_t>() + m, I->demand, (size_t)n * 4, cudaMemcpyHostToDevice, stream));
        return FLOCK_OK;
    }

    // The column-major copy of the uploaded costs for Vogel's column scans
    // (null when it cannot be allocated: the scans then read the rows).
    const int32_t* transposed(const Ctx& c) {
        const int m = c.I.m, n = c.I.n, ldcT = (m + 3) & ~3;
        if (costT.ensure((size_t)n * ldcT * 4 + 16) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        k_transpose<<<dim3((n + 31) / 32, (m + 31) / 32), dim3(32, 8), 0, stream>>>(c.I.cost, m, n, c.I.ldc,
                                                                                   costT.as<int32_t>(), ldcT);
        return cudaGetLastError() == cudaSuccess ? costT.as<int32_t>() : nullptr;
    }
    // The 16-bit copy of the uploaded costs into c.I (grid path, every cost
    // fits); without room for it the sweeps read the int32 costs.
    void narrow_copy(Ctx& c) {
        const int m = c.I.m, n = c.I.n, ldc16 = (n + 7) & ~7;
        if (cost16.ensure((size_t)m * ldc16 * 2 + 16) != cudaSuccess) { cudaGetLastError(); return; }
        const size_t cells = (size_t)m * ldc16;
        const int grid = (int)std::min<size_t>(4 * (size_t)num_sms(), (cells + 255) / 256);
        k_cost16<<<std::max(1, grid), 256, 0, stream>>>(c.I.cost, m, n, c.I.ldc, cost16.as<int16_t>(), ldc16);
        if (cudaGetLastError() != cudaSuccess) return;
        c.I.cost16 = cost16.as<int16_t>();
        c.I.ldc16 = ldc16;
    }
    // Dynamic shared memory of the Vogel launches (0: the line state stays
    // in the working set).
    static size_t vogel_smem(int V) { return vogel_stage_bytes(V) <= kVogelStageMax ? vogel_stage_bytes(V) : 0; }

    int reset_scalars(Scalars* dsc, int mode, int max_rounds, bool partial = false) {
        Scalars z;
        memset(&z, 0, sizeof(z));
        z.mode = mode;
        z.max_rounds = max_rounds;
        z.pricing = partial ? 1 : 0;
        z.pp_rows = kPPRowsGrid;              // partial pricing runs on the plain path from kGridPivotV vertices
        z.pp_refresh = kPPRefreshGrid;
        // FLOCK_PP_ROWS (1..kPPRows) / FLOCK_PP_REFRESH (>= 1) override them, for tuning
        if (const char* e = getenv("FLOCK_PP_ROWS")) z.pp_rows = std::min(kPPRows, std::max(1, atoi(e)));
        if (const char* e = getenv("FLOCK_PP_REFRESH")) z.pp_refresh = std::max(1, atoi(e));
        memcpy(h_sc.p, &z, sizeof(z));
        FLOCK_CK(cudaMemcpyAsync(dsc, h_sc.p, sizeof(z), cudaMemcpyHostToDevice, stream));
        return FLOCK_OK;
    }
};

static PlainSolver& plain() {
    static PlainSolver* s = new PlainSolver();
    return *s;
}

static void fill_flows_from_basis(int V, const int32_t* src, const int32_t* dst, const int32_t* qty,
                                  flock_flow* flows) {
    int w = 0;
    for (int k = 0; k < V - 1; k++) if (qty[k] > 0) flows[w++] = {src[k], dst[k], qty[k]};
    for (int k = 0; k < V - 1; k++) if (qty[k] <= 0) flows[w++] = {src[k], dst[k], qty[k]};
}

static size_t instance_ws_bytes(int V, int m);

// The plain solve of an instance below the grid-round size in ONE launch
// (k_solve_one).  P.one holds, in this order, the upload region -- the
// descriptor, the padded cost matrix, supplies and demands, the zeroed phase
// clock -- and the download region -- the phase clock again, the basis, the
// initial list, the duals and the scalars -- then the working set: one
// host-to-device copy from pinned memory before the launch and one
// device-to-host copy after it.  Same results and statistics as the round
// form; the phase clock splits the launch's device time.
static int solve_one_launch(PlainSolver& P, const flock_instance* I, const flock_options& opt, int bfs,
                            int max_rounds, flock_flow* flows, int64_t* du, int64_t* dv, flock_stats* st,
                            std::chrono::steady_clock::time_point t0) {
    const int m = I->m, n = I->n, V = m + n, V1 = V - 1, ldc = (n + 3) & ~3;
    size_t o = 0;
    const size_t o_desc = o; o = al256(o + sizeof(BatchDesc));
    const size_t o_cost = o; o = al256(o + (size_t)m * ldc * 4);
    const size_t o_sd = o;   o = al256(o + (size_t)V * 4);
    const size_t o_ph = o;   o = al256(o + sizeof(PhaseClock));
    const size_t up_end = o_ph + sizeof(PhaseClock);
    const size_t o_out = o;  o = al256(o + (size_t)3 * V1 * 4);
    const size_t o_bfs = o;  o = al256(o + (size_t)3 * V1 * 4);
    const size_t o_pot = o;  o = al256(o + (size_t)V * 8);
    const size_t o_sc = o;   o = al256(o + sizeof(Scalars));
    const size_t down_end = o_sc + sizeof(Scalars);
    const size_t o_ws = o;   o = al256(o + instance_ws_bytes(V, m));
    FLOCK_CK(P.one.ensure(o));
    FLOCK_CK(P.h_one.ensure(down_end));
    uint8_t* h = P.h_one.as<uint8_t>();
    BatchDesc* hd = P.h_one.as<BatchDesc>(o_desc);
    hd->m = m; hd->n = n; hd->ldc = ldc; hd->index = 0;
    hd->cost = P.one.as<int32_t>(o_cost);
    hd->sd = P.one.as<int32_t>(o_sd);
    hd->ws = P.one.as<uint8_t>(o_ws);
    hd->out = P.one.as<int32_t>(o_out);
    hd->bfs = P.one.as<int32_t>(o_bfs);
    hd->pot = P.one.as<int64_t>(o_pot);
    hd->sc = P.one.as<Scalars>(o_sc);
    hd->done = nullptr;
    int32_t* hc = P.h_one.as<int32_t>(o_cost);
    for (int i = 0; i < m; i++) {
        memcpy(hc + (size_t)i * ldc, I->cost + (size_t)i * n, (size_t)n * 4);
        for (int j = n; j < ldc; j++) hc[(size_t)i * ldc + j] = 0;
    }
    memcpy(P.h_one.as<int32_t>(o_sd), I->supply, (size_t)m * 4);
    memcpy(P.h_one.as<int32_t>(o_sd) + m, I->demand, (size_t)n * 4);
    memset(h + o_ph, 0, sizeof(PhaseClock));
    FLOCK_CK(cudaMemcpyAsync(P.one.p, h, up_end, cudaMemcpyHostToDevice, P.stream));
    PhaseClock* d_ph = P.one.as<PhaseClock>(o_ph);
    BatchArgs a;
    a.desc = P.one.as<BatchDesc>(o_desc);
    a.count = 1;
    a.next = nullptr;
    a.active = nullptr;
    a.maxV = V; a.maxM = m;
    a.bfs_method = bfs == FLOCK_BFS_NWC ? FLOCK_BFS_NWC : FLOCK_BFS_VOGEL;
    a.mode = pivot_mode(opt);
    a.pricing = pricing_of(opt);
    a.max_rounds = max_rounds;
    a.light = stage_light(V, m) ? 1 : 0;
    a.ph = d_ph;
    block_pricing(a.pp);
    size_t smem = launch_smem_bytes(V, m, a.light != 0);
    // the cost matrix into the same dynamic block when it fits (Vogel's
    // rescans, the sweeps and the certificate then read shared memory)
    a.cost_smem = 0;
    const size_t cost_off = (smem + 15) & ~size_t(15), cost_bytes = (size_t)m * ldc * 4;
    const char* cs_env = getenv("FLOCK_COST_SMEM");
    if (cost_off + cost_bytes <= kStageSmemMax && !(cs_env && !strcmp(cs_env, "0"))) {
        a.cost_smem = (int32_t)cost_off;
        smem = cost_off + cost_bytes;
    }
    const int threads = solve_one_threads(V);
    const void* fn = solve_one_fn(threads);
    void* kargs[] = {&a};
    FLOCK_CK(cudaEventRecord(P.ev[0], P.stream));
    FLOCK_CK(cudaLaunchKernel(fn, dim3(1), dim3(threads), kargs, smem, P.stream));
    FLOCK_CK(cudaEventRecord(P.ev[2], P.stream));
    FLOCK_CK(cudaMemcpyAsync(h + o_ph, P.one.as<uint8_t>(o_ph), down_end - o_ph, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaStreamSynchronize(P.stream));
    float ms_all = 0;
    cudaEventElapsedTime(&ms_all, P.ev[0], P.ev[2]);
    const int32_t* h3 = P.h_one.as<int32_t>(o_out);
    const int64_t* pot = P.h_one.as<int64_t>(o_pot);
    const Scalars S = *P.h_one.as<Scalars>(o_sc);
    const PhaseClock hph = *P.h_one.as<PhaseClock>(o_ph);
    const bool broken = S.status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE);
    if (flows && !broken) fill_flows_from_basis(V, h3, h3 + V1, h3 + 2 * V1, flows);
    if (du && !broken) for (int i = 0; i < m; i++) du[i] = pot[i];
    if (dv && !broken) for (int j = 0; j < n; j++) dv[j] = pot[m + j];
    int status = S.status & kFailMask;
    if (opt.verify && S.cert) status |= ST_CERT_FAIL;
    if (st) {
        st->notes = (S.status & ~kFailMask) | (S.fail_site << 8);
        st->objective = S.objective;
        st->iterations = S.rounds;
        st->pivots = S.pivots;
        st->active_flows = broken ? 0 : S.active;
        st->status = status;
        st->certified = (!broken && S.cert == 0) ? 1 : 0;
        st->vogel_events = S.events;
        st->ms_bfs = hph.ns[PH_BFS] * 1e-6;
        st->ms_dual = hph.ns[PH_DUAL] * 1e-6;
        st->ms_sweep = hph.ns[PH_SWEEP] * 1e-6;
        st->ms_cycle = hph.ns[PH_CYCLE] * 1e-6;
        st->ms_resolve = hph.ns[PH_RESOLVE] * 1e-6;
        st->ms_adjust = hph.ns[PH_ADJUST] * 1e-6;
        st->ms_pivot = st->ms_cycle + st->ms_resolve + st->ms_adjust;
        // the loop's device time: the launch less its setup (BFS) and its
        // retrieval and certificate (the idle tail)
        st->ms_simplex = std::max(0.0, (double)ms_all - st->ms_bfs - hph.ns[PH_IDLE] * 1e-6);
        st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return status ? FLOCK_ERR_NOT_OPTIMAL : FLOCK_OK;
}

static int solve_plain(const flock_instance* I, const flock_options* opt_in, flock_flow* flows,
                       int64_t* du, int64_t* dv, flock_stats* st) {
    const auto t0 = std::chrono::steady_clock::now();
    bool fits16 = false;
    int rc = validate_instance_range(I, &fits16);
    if (rc) return rc;
    flock_options opt;
    flock_default_options(&opt);
    if (opt_in) opt = *opt_in;
    const int max_rounds = opt.max_iterations > 0 ? opt.max_iterations : (1 << 30);
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    if ((rc = P.setup())) return rc;
    const int m = I->m, n = I->n, V = m + n;
    const int bfs = opt.bfs_method == FLOCK_BFS_NWC || opt.bfs_method == FLOCK_BFS_VOGEL_DEVICE ? opt.bfs_method
                                                                                                  : FLOCK_BFS_VOGEL;
    // the one-launch form below the grid size (the stepping-stone mode runs
    // its rounds on the round kernel at every size)
    if (V < grid_pivot_v() && bfs != FLOCK_BFS_VOGEL_DEVICE && pivot_mode(opt) != 3)
        return solve_one_launch(P, I, opt, bfs, max_rounds, flows, du, dv, st, t0);
    Ctx c;
    int32_t* out3 = nullptr;
    if ((rc = P.prepare(I, c, &out3))) return rc;
    // the grid path's sweeps read 16-bit costs when every cost fits
    // (FLOCK_COST16=0 keeps them on the int32 costs)
    const char* c16_env = getenv("FLOCK_COST16");
    if (fits16 && V >= grid_pivot_v() && !(c16_env && !strcmp(c16_env, "0"))) P.narrow_copy(c);
    // partial pricing runs on the plain path from kGridPivotV vertices (grid rounds)
    const bool partial = pricing_of(opt) && V >= grid_pivot_v();
    if ((rc = P.reset_scalars(c.sc, pivot_mode(opt), max_rounds, partial))) return rc;
    FLOCK_CK(cudaMemsetAsync(P.ph, 0, sizeof(PhaseClock), P.stream));
    c.ph = P.ph;
    const int nt = threads_for(V);
    FLOCK_CK(cudaEventRecord(P.ev[0], P.stream));
    int2 *rbook = nullptr, *cbook = nullptr;
    if (bfs == FLOCK_BFS_VOGEL_DEVICE && (rc = P.build_books(c, &rbook, &cbook))) return rc;
    const int32_t* costT = bfs == FLOCK_BFS_VOGEL ? P.transposed(c) : nullptr;
    const size_t vsm = bfs == FLOCK_BFS_VOGEL ? PlainSolver::vogel_smem(V) : 0;
    k_setup<<<1, nt, vsm, P.stream>>>(c, bfs, rbook, cbook, costT, vsm ? 1 : 0);
    FLOCK_CK(cudaGetLastError());
    FLOCK_CK(cudaEventRecord(P.ev[1], P.stream));
    int grid = 0, tile = 0, ntile = 0, bgrid = 0, btile = 0, bntile = 0;
    sweep_shape(m, n, &grid, &tile, &ntile);
    bulk_shape(m, n, &bgrid, &btile, &bntile);
    Scalars* hs = P.h_sc.as<Scalars>();
    // the grid rounds apply single pivots: the parallel stepping stone's
    // multi-pivot rounds run on one block at every size
    if (V >= grid_pivot_v() && pivot_mode(opt) != 3) {
        // large instance: the pivot round over the whole GPU, chunks of
        // rounds captured once as a CUDA graph
        FLOCK_CK(cudaMemsetAsync(P.gp, 0, sizeof(GridPivot), P.stream));
        FLOCK_CK(cudaMemsetAsync(P.cp, 0, sizeof(ClusterPivot), P.stream));
        const int gg = std::max(1, std::min((V + 255) / 256, 2 * num_sms()));
        // Partial pricing: each iteration is a full round (the bulk sweep of
        // every row, the next candidate rows, one pivot over the grid) and
        // then the candidate rounds inside one thread-block cluster, until
        // the candidates run out or pp_refresh rounds have passed.  The
        // six-kernel rounds otherwise (FULL pricing, no cluster launch on
        // this device, or FLOCK_GRID_FORM=rounds).
        const char* form = getenv("FLOCK_GRID_FORM");
        const bool clustered = partial && P.cluster_ctas >= 2 && !(form && !strcmp(form, "rounds"));
        cudaLaunchConfig_t ccfg = {};
        cudaLaunchAttribute cattr[2];
        ccfg.gridDim = dim3(P.cluster_ctas);
        ccfg.blockDim = dim3(kCRoundThreads);
        ccfg.dynamicSmemBytes = kCRoundSmem;
        ccfg.stream = P.stream;
        cattr[0].id = cudaLaunchAttributeClusterDimension;
        cattr[0].val.clusterDim.x = P.cluster_ctas;
        cattr[0].val.clusterDim.y = 1;
        cattr[0].val.clusterDim.z = 1;
        ccfg.attrs = cattr;
        // the cluster launch is the full sweep's programmatic dependent
        // (FLOCK_PDL=0: an ordinary stream dependency)
        cattr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        cattr[1].val.programmaticStreamSerializationAllowed = 1;
        const char* pdl_env = getenv("FLOCK_PDL");
        ccfg.numAttrs = pdl_env && !strcmp(pdl_env, "0") ? 1 : 2;
        int chunk = clustered ? 2 : 8;
        cudaGraphExec_t exec = nullptr;
        int exec_chunk = 0;
        for (;;) {
            if (exec_chunk != chunk) {
                if (exec) cudaGraphExecDestroy(exec);
                exec = nullptr;
                cudaGraph_t g;
                FLOCK_CK(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
                for (int r = 0; r < chunk; r++) {
                    if (clustered) {
                        // the cluster rounds leave only full sweeps to the grid: the bulk-copy sweep
                        // (the full round's entering cell and candidate rows are chosen in the cluster)
                        k_sweep<<<bgrid, kBulkThreads, kBulkSmem, P.stream>>>(c, btile, bntile);
                    } else {
                        k_gsweep<<<grid, kSweepThreads, 0, P.stream>>>(c, P.gp, tile, ntile);
                        if (partial) k_gsweep_rest<<<grid, kSweepThreads, 0, P.stream>>>(c, P.gp, tile, ntile);
                        k_gchoose<<<1, 1024, 0, P.stream>>>(c, P.gp);
                    }
                    if (clustered) {
                        // the full round's pivot and the candidate rounds in one cluster launch
                        // the register form when every thread owns at most one vertex
                        if (V <= P.cluster_ctas * kCRoundThreads)
                            FLOCK_CK(cudaLaunchKernelEx(&ccfg, k_cround<true>, c, P.cp, (const GridPivot*)P.gp, 1));
                        else
                            FLOCK_CK(cudaLaunchKernelEx(&ccfg, k_cround<false>, c, P.cp, (const GridPivot*)P.gp, 1));
                    } else {
                        k_gmember<<<gg, 256, 0, P.stream>>>(c, P.gp);
                        k_gpick<<<gg, 256, 0, P.stream>>>(c, P.gp);
                        k_gupdate<<<gg, 256, 0, P.stream>>>(c, P.gp);
                    }
                }
                FLOCK_CK(cudaStreamEndCapture(P.stream, &g));
                FLOCK_CK(cudaGraphInstantiate(&exec, g, 0));
                cudaGraphDestroy(g);
                exec_chunk = chunk;
            }
            FLOCK_CK(cudaGraphLaunch(exec, P.stream));
            FLOCK_CK(cudaMemcpyAsync(hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, P.stream));
            FLOCK_CK(cudaStreamSynchronize(P.stream));
            if (hs->done) break;
            if (chunk < (clustered ? 16 : 256)) chunk *= 2;
        }
        if (exec) cudaGraphExecDestroy(exec);
    } else {
        // pivot loop: chunks of rounds (grid sweep, one-CTA pivot round)
        // captured once as a CUDA graph
        int chunk = 8;
        cudaGraphExec_t exec = nullptr;
        int exec_chunk = 0;
        for (;;) {
            if (exec_chunk != chunk) {
                if (exec) cudaGraphExecDestroy(exec);
                exec = nullptr;
                cudaGraph_t g;
                FLOCK_CK(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
                for (int r = 0; r < chunk; r++) {
                    k_sweep<<<bgrid, kBulkThreads, kBulkSmem, P.stream>>>(c, btile, bntile);
                    k_pivot<<<1, nt, 0, P.stream>>>(c);
                }
                FLOCK_CK(cudaStreamEndCapture(P.stream, &g));
                FLOCK_CK(cudaGraphInstantiate(&exec, g, 0));
                cudaGraphDestroy(g);
                exec_chunk = chunk;
            }
            FLOCK_CK(cudaGraphLaunch(exec, P.stream));
            FLOCK_CK(cudaMemcpyAsync(hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, P.stream));
            FLOCK_CK(cudaStreamSynchronize(P.stream));
            if (hs->done) break;
            if (chunk < 256) chunk *= 2;
        }
        if (exec) cudaGraphExecDestroy(exec);
    }
    FLOCK_CK(cudaEventRecord(P.ev[2], P.stream));
    k_finalize<<<1, nt, 0, P.stream>>>(c);
    FLOCK_CK(cudaGetLastError());
    if (opt.verify) {
        const int g2 = std::max(1, std::min((m + 7) / 8, 4 * num_sms()));
        k_cert_cells<<<g2, 256, 0, P.stream>>>(c);
        FLOCK_CK(cudaGetLastError());
    }
    std::vector<int32_t> h3((size_t)3 * V);
    FLOCK_CK(cudaMemcpyAsync(h3.data(), out3, (size_t)3 * V * 4, cudaMemcpyDeviceToHost, P.stream));
    std::vector<int64_t> pot((size_t)V);
    FLOCK_CK(cudaMemcpyAsync(pot.data(), c.pot, (size_t)V * 8, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, P.stream));
    PhaseClock hph;
    FLOCK_CK(cudaMemcpyAsync(&hph, P.ph, sizeof(PhaseClock), cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaStreamSynchronize(P.stream));
    float ms_bfs = 0, ms_loop = 0;
    cudaEventElapsedTime(&ms_bfs, P.ev[0], P.ev[1]);
    cudaEventElapsedTime(&ms_loop, P.ev[1], P.ev[2]);
    const Scalars S = *hs;
    const bool broken = S.status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE);
    if (flows && !broken) fill_flows_from_basis(V, h3.data(), h3.data() + V, h3.data() + 2 * V, flows);
    if (du && !broken) for (int i = 0; i < m; i++) du[i] = pot[i];
    if (dv && !broken) for (int j = 0; j < n; j++) dv[j] = pot[m + j];
    int status = S.status & kFailMask;
    if (opt.verify && S.cert) status |= ST_CERT_FAIL;
    if (st) {
        st->notes = (S.status & ~kFailMask) | (S.fail_site << 8);
        st->objective = S.objective;
        st->iterations = S.rounds;
        st->pivots = S.pivots;
        st->active_flows = broken ? 0 : S.active;
        st->status = status;
        st->certified = (opt.verify && !broken && S.cert == 0) ? 1 : 0;
        st->vogel_events = S.events;
        // the setup launch's start tree counts toward the loop (phase clock)
        st->ms_bfs = std::min((double)ms_bfs, hph.ns[PH_BFS] * 1e-6);
        st->ms_simplex = ms_loop + (ms_bfs - st->ms_bfs);
        st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        st->ms_dual = hph.ns[PH_DUAL] * 1e-6;
        st->ms_sweep = hph.ns[PH_SWEEP] * 1e-6;
        st->ms_cycle = hph.ns[PH_CYCLE] * 1e-6;
        st->ms_resolve = hph.ns[PH_RESOLVE] * 1e-6;
        st->ms_adjust = hph.ns[PH_ADJUST] * 1e-6;
        st->ms_pivot = st->ms_cycle + st->ms_resolve + st->ms_adjust;
    }
    return status ? FLOCK_ERR_NOT_OPTIMAL : FLOCK_OK;
}

// Status of a Vogel-only kernel: an internal check that failed on the device
// becomes FLOCK_ERR_CUDA with its site (flock_vogel, flock_vogel_device and
// flock_vogel_static report it alike).
int vogel_status_check(const Scalars& S, const char* who) {
    if (S.status & ST_TREE_CORRUPT) {
        set_error(std::string(who) + ": internal check failed at site " + std::to_string(S.fail_site));
        return FLOCK_ERR_CUDA;
    }
    return FLOCK_OK;
}

static int vogel_plain(const flock_instance* I, flock_flow* flows, int32_t* events, bool books = false) {
    int rc = validate_instance(I);
    if (rc) return rc;
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    if ((rc = P.setup())) return rc;
    const int V = I->m + I->n;
    Ctx c;
    int32_t* out3 = nullptr;
    if ((rc = P.prepare(I, c, &out3))) return rc;
    if ((rc = P.reset_scalars(c.sc, 1, 1))) return rc;
    if (books) {
        int2 *rbook = nullptr, *cbook = nullptr;
        if ((rc = P.build_books(c, &rbook, &cbook))) return rc;
        k_vogel_books_only<<<1, threads_for(V), 0, P.stream>>>(c, rbook, cbook);
    } else {
        const size_t vsm = PlainSolver::vogel_smem(V);
        k_vogel_only<<<1, threads_for(V), vsm, P.stream>>>(c, P.transposed(c), vsm ? 1 : 0);
    }
    FLOCK_CK(cudaGetLastError());
    std::vector<int32_t> a((size_t)V), b((size_t)V), q((size_t)V);
    FLOCK_CK(cudaMemcpyAsync(a.data(), c.bfs_src, (size_t)(V - 1) * 4, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(b.data(), c.bfs_dst, (size_t)(V - 1) * 4, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(q.data(), c.bfs_qty, (size_t)(V - 1) * 4, cudaMemcpyDeviceToHost, P.stream));
    Scalars* hs = P.h_sc.as<Scalars>();
    FLOCK_CK(cudaMemcpyAsync(hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaStreamSynchronize(P.stream));
    if ((rc = vogel_status_check(*hs, books ? "flock_vogel_device" : "flock_vogel"))) return rc;
    for (int k = 0; k < V - 1; k++) flows[k] = {a[k], b[k], q[k]};
    if (events) *events = hs->events;
    return FLOCK_OK;
}



// Benchmark hook: time `iters` launches of the fused sweep on an m x n matrix
// with random costs and duals already resident (no pivots).  Writes the
// average launch time (CUDA events on the launching stream).
static void bulk_shape(int m, int n, int* grid, int* tile, int* ntile) {
    const int ldc = (n + 3) & ~3;
    *tile = std::min(ldc, kSweepTile);
    *ntile = (n + *tile - 1) / *tile;
    const long long units = (long long)m * ((std::min(*tile, n) + kBulkSeg - 1) / kBulkSeg);
    const int nrg = (int)std::max(1LL, std::min(units, (long long)std::max(1, num_sms() / *ntile)));
    *grid = *ntile * nrg;
}

static void sweep_shape(int m, int n, int* grid, int* tile, int* ntile) {
    const int ldc = (n + 3) & ~3;
    *tile = std::min(ldc, kSweepTile);
    *ntile = (n + *tile - 1) / *tile;
    const int nseg = (std::min(*tile, n) + kSegCols - 1) / kSegCols;
    const long long wpb = kSweepThreads / 32;
    const long long want = ((long long)m * nseg + wpb - 1) / wpb;
    const long long cap = std::max(1, (2 * num_sms()) / *ntile);
    const int nrg = (int)std::max(1LL, std::min(want, cap));
    *grid = *ntile * nrg;
}

// Test hook: one sweep over caller-given costs (m x n, row-major) and duals
// (pot[V], rows then columns; kDeadPot marks a zero-demand column), row keys
// back in keys[m].  cta_form: 0 grid-wide k_sweep, 1 the CTA-local sweep of
// the batched form with `threads` threads.
static int test_sweep(int m, int n, const int32_t* cost, const int64_t* pot, uint64_t* keys, int cta_form,
                      int threads) {
    if (m < 1 || n < 1 || !cost || !pot || !keys) return FLOCK_ERR_ARG;
    if (cta_form > 0 && (threads < 32 || threads > 1024 || threads % 32)) return FLOCK_ERR_ARG;
    if (cta_form < 0)        // the bulk sweep on the 16-bit copy: every cost must fit
        for (size_t k = 0; k < (size_t)m * n; k++)
            if (cost[k] < INT16_MIN || cost[k] > INT16_MAX) return FLOCK_ERR_RANGE;
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    int rc = P.setup();
    if (rc) return rc;
    const int V = m + n, ldc = (n + 3) & ~3;
    FLOCK_CK(P.cost.ensure((size_t)m * ldc * 4 + 16));
    size_t gbytes = 0;
    Ctx probe;
    carve_ctx(probe, nullptr, V, m, nullptr, nullptr, nullptr, &gbytes);
    FLOCK_CK(P.ws.ensure(al256(gbytes) + al256(sizeof(Scalars))));
    Ctx c;
    carve_ctx(c, P.ws.as<uint8_t>(), V, m, nullptr, nullptr);
    c.sc = P.ws.as<Scalars>(al256(gbytes));
    c.I.m = m; c.I.n = n; c.I.ldc = ldc; c.I.cost = P.cost.as<int32_t>();
    if ((rc = P.reset_scalars(c.sc, 1, 1))) return rc;
    FLOCK_CK(cudaMemsetAsync(P.cost.p, 0x7f, (size_t)m * ldc * 4, P.stream));   // padding: never read
    FLOCK_CK(cudaMemcpy2DAsync(P.cost.p, (size_t)ldc * 4, cost, (size_t)n * 4, (size_t)n * 4, m,
                               cudaMemcpyHostToDevice, P.stream));
    FLOCK_CK(cudaMemcpyAsync(c.pot, pot, (size_t)V * 8, cudaMemcpyHostToDevice, P.stream));
    k_publish_duals<<<1, 1024, 0, P.stream>>>(c);
    FLOCK_CK(cudaMemsetAsync(c.row_best, 0xff, (size_t)m * 8, P.stream));
    if (cta_form < 0) {
        P.narrow_copy(c);
        if (!c.I.cost16) { set_error("no room for the 16-bit copy"); return FLOCK_ERR_CUDA; }
    }
    if (cta_form > 0) {
        k_sweep_cta_only<<<1, threads, 0, P.stream>>>(c);
    } else {
        int grid = 0, tile = 0, ntile = 0;
        bulk_shape(m, n, &grid, &tile, &ntile);
        k_sweep<<<grid, kBulkThreads, kBulkSmem, P.stream>>>(c, tile, ntile);
    }
    FLOCK_CK(cudaGetLastError());
    FLOCK_CK(cudaMemcpyAsync(keys, c.row_best, (size_t)m * 8, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaStreamSynchronize(P.stream));
    return FLOCK_OK;
}

// Test hook: candidate-row selection (select_candidate_rows, clearing the
// other rows) over host row keys of an m-row instance.
__global__ void __launch_bounds__(1024) k_test_select(Ctx c, uint64_t* best) {
    __shared__ BlockScratch bs;
    const uint64_t b = select_candidate_rows(c, bs, true);
    if (threadIdx.x == 0) *best = b;
}

static int test_select_rows(int m, const uint64_t* keys, uint64_t* keys_out, int32_t* prow, int32_t* pn,
                            int32_t* pp_rows, uint64_t* best, int threads) {
    if (m < 1 || !keys || !keys_out || !prow || !pn || !pp_rows || !best) return FLOCK_ERR_ARG;
    if (threads < 32 || threads > 1024 || threads % 32) return FLOCK_ERR_ARG;
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    int rc = P.setup();
    if (rc) return rc;
    const int n = 1, V = m + n;
    size_t gbytes = 0;
    Ctx probe;
    carve_ctx(probe, nullptr, V, m, nullptr, nullptr, nullptr, &gbytes);
    FLOCK_CK(P.ws.ensure(al256(gbytes) + al256(sizeof(Scalars)) + 256));
    Ctx c;
    carve_ctx(c, P.ws.as<uint8_t>(), V, m, nullptr, nullptr);
    c.sc = P.ws.as<Scalars>(al256(gbytes));
    uint64_t* d_best = P.ws.as<uint64_t>(al256(gbytes) + al256(sizeof(Scalars)));
    c.I.m = m; c.I.n = n; c.I.ldc = 4;
    if ((rc = P.reset_scalars(c.sc, 0, 1))) return rc;
    FLOCK_CK(cudaMemcpyAsync(c.row_best, keys, (size_t)m * 8, cudaMemcpyHostToDevice, P.stream));
    k_test_select<<<1, threads, 0, P.stream>>>(c, d_best);
    FLOCK_CK(cudaGetLastError());
    FLOCK_CK(cudaMemcpyAsync(keys_out, c.row_best, (size_t)m * 8, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(prow, c.prow, (size_t)kPPRows * 4, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(best, d_best, 8, cudaMemcpyDeviceToHost, P.stream));
    Scalars* hs = P.h_sc.as<Scalars>();
    FLOCK_CK(cudaMemcpyAsync(hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaStreamSynchronize(P.stream));
    *pn = hs->pp_n;
    *pp_rows = hs->pp_rows;
    return FLOCK_OK;
}

static int bench_sweep(int m, int n, int iters, float* avg_ms, int* tile_out) {
    if (m < 1 || n < 1 || iters < 1 || !avg_ms) return FLOCK_ERR_ARG;
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    int rc = P.setup();
    if (rc) return rc;
    const int V = m + n, ldc = (n + 3) & ~3;
    FLOCK_CK(P.cost.ensure((size_t)m * ldc * 4 + 16));
    size_t gbytes = 0;
    Ctx probe;
    carve_ctx(probe, nullptr, V, m, nullptr, nullptr, nullptr, &gbytes);
    FLOCK_CK(P.ws.ensure(al256(gbytes) + al256(3 * (size_t)V * 4) + al256(sizeof(Scalars))));
    Ctx c;
    carve_ctx(c, P.ws.as<uint8_t>(), V, m, nullptr, nullptr);
    c.sc = P.ws.as<Scalars>(al256(gbytes) + al256(3 * (size_t)V * 4));
    c.I.m = m; c.I.n = n; c.I.ldc = ldc; c.I.cost = P.cost.as<int32_t>();
    if ((rc = P.reset_scalars(c.sc, 1, 1))) return rc;
    k_fill_bench<<<std::min(4096, (int)(((size_t)m * ldc + 255) / 256)), 256, 0, P.stream>>>(
        P.cost.as<int32_t>(), (size_t)m * ldc, c.pot, V);
    FLOCK_CK(cudaGetLastError());
    k_publish_duals<<<1, 1024, 0, P.stream>>>(c);
    FLOCK_CK(cudaMemsetAsync(c.row_best, 0xff, (size_t)m * 8, P.stream));
    int grid = 0, tile = 0, ntile = 0;
    bulk_shape(m, n, &grid, &tile, &ntile);
    for (int w = 0; w < 3; w++) k_sweep<<<grid, kBulkThreads, kBulkSmem, P.stream>>>(c, tile, ntile);
    FLOCK_CK(cudaEventRecord(P.ev[0], P.stream));
    for (int k = 0; k < iters; k++) k_sweep<<<grid, kBulkThreads, kBulkSmem, P.stream>>>(c, tile, ntile);
    FLOCK_CK(cudaEventRecord(P.ev[1], P.stream));
    FLOCK_CK(cudaEventSynchronize(P.ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, P.ev[0], P.ev[1]);
    *avg_ms = ms / iters;
    if (tile_out) *tile_out = tile;
    return FLOCK_OK;
}

// Average device time of one k_l2_read launch over a buffer of `bytes`
// (filled once, read `passes` times per launch), after one warm-up launch
// that brings the buffer into L2.
static int bench_l2(long long bytes, int passes, int iters, float* avg_ms) {
    if (bytes < 16 || passes < 1 || iters < 1 || !avg_ms) return FLOCK_ERR_ARG;
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    int rc = P.setup();
    if (rc) return rc;
    const size_t n4 = (size_t)bytes / 16;
    FLOCK_CK(P.cost.ensure(n4 * 16 + 16));
    k_fill_bench<<<std::min(4096, (int)((n4 * 4 + 255) / 256)), 256, 0, P.stream>>>(P.cost.as<int32_t>(), n4 * 4,
                                                                                    nullptr, 0);
    FLOCK_CK(cudaGetLastError());
    const int grid = 4 * num_sms();
    int* sink = P.ws.ensure(256) == cudaSuccess ? P.ws.as<int>() : nullptr;
    if (!sink) return FLOCK_ERR_CUDA;
    const int4* buf = reinterpret_cast<const int4*>(P.cost.as<int32_t>());
    k_l2_read<<<grid, 512, 0, P.stream>>>(buf, n4, passes, sink);
    FLOCK_CK(cudaEventRecord(P.ev[0], P.stream));
    for (int k = 0; k < iters; k++) k_l2_read<<<grid, 512, 0, P.stream>>>(buf, n4, passes, sink);
    FLOCK_CK(cudaEventRecord(P.ev[1], P.stream));
    FLOCK_CK(cudaEventSynchronize(P.ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, P.ev[0], P.ev[1]);
    *avg_ms = ms / iters;
    return FLOCK_OK;
}

// -------------------------------------------------------- batched solver ---
// Size buckets by V = m + n.  Instances above the last edge run on the plain
// path (their staged tree would not fit in shared memory).
// A bucket stages fully when its largest instance fits (56 V + 8 M bytes: up
// to V = 3500 or so); the others stage lightly (staged_bytes(4096, 4095,
// true) = 208 KB).
static const int kBucketEdges[] = {64, 128, 256, 512, 1024, 2048, 2944, 4096};
static const int kNumBuckets = 8;
static const int kMaxStagedV = 4096;
static const int kMaxChunk = 64;

static int bucket_of(int V) {
    int b = 0;
    while (b < kNumBuckets && V > kBucketEdges[b]) b++;
    return b;   // kNumBuckets: plain path
}

// Launch configuration of a bucket.  threads: block size of the kernels;
// persistent: 1 = one k_bsolve launch (every round inside), 0 = k_bsetup,
// graph-captured chunks of k_bround, k_bfinal; grid_mult: resident CTAs per
// SM multiplier for work stealing (round form); chunk: pricing rounds per
// graph launch (round form).
struct TuneCfg { int threads; int grid_mult; int chunk; int persistent; };

static std::mutex g_tune_mu;
static TuneCfg g_tuned[kNumBuckets];
static bool g_tuned_ok[kNumBuckets];

static TuneCfg default_cfg(int maxV) {
    TuneCfg t;
    t.threads = maxV <= 256 ? 128 : 256;
    t.grid_mult = 1;
    t.chunk = 16;
    t.persistent = 1;
    return t;
}

static size_t instance_ws_bytes(int V, int m) {
    Ctx probe;
    size_t gb = 0;
    carve_ctx(probe, nullptr, V, m, nullptr, (int64_t*)16, nullptr, &gb);
    return al256(gb);
}

struct BatchRunner {
    DevBuf d_cost, d_sd, d_desc, d_out, d_bfs, d_pot, d_sc, d_ws, d_ctr;
    HostBuf h_cost, h_sd, h_desc, h_out, h_sc, h_ctr;
    cudaStream_t st[kNumBuckets] = {};
    // the first bucket's later staging chunks (its uploads and launches
    // overlap the packing of the next chunk)
    static constexpr int kStageChunks = 4;
    cudaStream_t cst[kStageChunks - 1] = {};
    cudaEvent_t ev_start = nullptr, ev_done = nullptr, ev_join = nullptr;
    bool init = false;
    // per call
    int count = 0;
    std::vector<int> V_of, m_of, n_of, plain_list;
    std::vector<int64_t> out_off, pot_off;   // basis cells / duals before instance k
    std::vector<int64_t> cost_off, sd_off, ws_off;
    std::vector<int> order_;                // staged instances, grouped by bucket
    int64_t total_cells = 0, total_pot = 0, total_cost = 0, total_sd = 0, total_ws = 0;
    std::vector<BatchDesc> descs;           // grouped by bucket
    int bstart[kNumBuckets + 1] = {};
    int bmaxV[kNumBuckets] = {}, bmaxM[kNumBuckets] = {};
    flock_options opt;
    const flock_instance* insts = nullptr;
    std::vector<flock_stats> plain_stats;
    std::vector<std::vector<flock_flow>> plain_flows;
    int32_t launches = 0;                   // kernels launched by the last run
    bool packed = false;                    // every bucket packed into the staging buffers
    std::vector<uint8_t> cost_bad, cost_checked;   // per instance: cost out of range / range checked

    int setup() {
        if (init) return FLOCK_OK;
        for (auto& s : st) FLOCK_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        for (auto& s : cst) FLOCK_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        FLOCK_CK(cudaEventCreate(&ev_start));
        FLOCK_CK(cudaEventCreate(&ev_done));
        FLOCK_CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
        FLOCK_CK(cudaFuncSetAttribute(k_bround, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageSmemMax));
        for (int t : {256, 512, 1024})
            FLOCK_CK(cudaFuncSetAttribute(bsolve_fn(t), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageSmemMax));
        FLOCK_CK(d_ctr.ensure((size_t)kNumBuckets * 2 * kMaxChunk * sizeof(int32_t)));
        FLOCK_CK(h_ctr.ensure((size_t)kNumBuckets * 2 * kMaxChunk * sizeof(int32_t)));
        init = true;
        return FLOCK_OK;
    }

    // Validate the instances and lay out the arenas.  Costs are packed into
    // pinned memory per bucket just before that bucket is uploaded and
    // launched (pack_bucket), so packing overlaps with the device work of the
    // buckets launched before it.
    int prepare(int cnt, const flock_instance* in, const flock_options* opt_in) {
        int rc = setup();
        if (rc) return rc;
        flock_default_options(&opt);
        if (opt_in) opt = *opt_in;
        if (opt.bfs_method == FLOCK_BFS_VOGEL_DEVICE) {
            set_error("vam_device Vogel runs on flock_solve and flock_vogel_device only");
            return FLOCK_ERR_ARG;
        }
        if (opt.pivot_method == FLOCK_PIVOT_SS) {
            set_error("the parallel stepping-stone mode runs on flock_solve only");
            return FLOCK_ERR_ARG;
        }
        insts = in;
        count = cnt;
        V_of.assign(cnt, 0); m_of.assign(cnt, 0); n_of.assign(cnt, 0);
        out_off.assign(cnt, 0); pot_off.assign(cnt, 0);
        cost_off.assign(cnt, 0); sd_off.assign(cnt, 0); ws_off.assign(cnt, 0);
        plain_list.clear();
        total_cells = total_pot = total_cost = total_sd = total_ws = 0;
        // Validation with the result validate_instance gives one instance at a
        // time: the first failing instance reports its first failing check
        // (shape, then the cost range).  Shapes are checked here; the cost
        // range of a staged instance is checked while its bucket is packed,
        // before that bucket is uploaded or launched (a bad one stops the
        // call, see cost_failure); the plain-path instances' costs here.
        std::vector<int> pre(cnt, FLOCK_OK);
        std::vector<std::string> pre_msg(cnt);
        parallel_for(cnt, [&](int k) {
            if ((pre[k] = validate_shape(&in[k], &pre_msg[k]))) return;
            m_of[k] = in[k].m; n_of[k] = in[k].n; V_of[k] = in[k].m + in[k].n;
        });
        cost_bad.assign(cnt, 0);
        cost_checked.assign(cnt, 0);
        int first_bad = cnt;
        for (int k = 0; k < cnt; k++) if (pre[k]) { first_bad = k; break; }
        parallel_for(cnt, [&](int k) {
            if (!pre[k] && (V_of[k] > kMaxStagedV || k < first_bad)) {
                if (V_of[k] > kMaxStagedV || first_bad < cnt) {
                    cost_bad[k] = !costs_in_range(in[k].cost, (size_t)m_of[k] * n_of[k]);
                    cost_checked[k] = 1;
                }
            }
        });
        for (int k = 0; k < cnt; k++) {
            if (pre[k]) { set_error(pre_msg[k]); return pre[k]; }
            if (cost_bad[k]) { set_error("cost out of range"); return FLOCK_ERR_RANGE; }
        }
        // bucket, largest first inside each bucket (work stealing starts with the long solves)
        std::vector<int> order;
        for (int k = 0; k < cnt; k++) {
            out_off[k] = total_cells; total_cells += V_of[k] - 1;
            pot_off[k] = total_pot; total_pot += V_of[k];
            if (V_of[k] <= kMaxStagedV) order.push_back(k); else plain_list.push_back(k);
        }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const int ba = bucket_of(V_of[a]), bb = bucket_of(V_of[b]);
            if (ba != bb) return ba < bb;
            return (int64_t)m_of[a] * n_of[a] > (int64_t)m_of[b] * n_of[b];
        });
        order_ = order;
        // arenas in bucket order: each bucket's costs and quantities are contiguous
        for (int k : order) {
            const int m = m_of[k], n = n_of[k], ldc = (n + 3) & ~3;
            cost_off[k] = total_cost; total_cost += (int64_t)m * ldc;
            sd_off[k] = total_sd; total_sd += m + n;
            ws_off[k] = total_ws; total_ws += (int64_t)instance_ws_bytes(m + n, m);
        }
        FLOCK_CK(h_cost.ensure((size_t)total_cost * 4 + 16));
        FLOCK_CK(h_sd.ensure((size_t)total_sd * 4 + 16));
        descs.resize(order.size());
        for (int b = 0; b <= kNumBuckets; b++) bstart[b] = 0;
        for (int b = 0; b < kNumBuckets; b++) { bmaxV[b] = 0; bmaxM[b] = 0; }
        for (size_t q = 0; q < order.size(); q++) {
            const int k = order[q];
            const int b = bucket_of(V_of[k]);
            bstart[b + 1]++;
            bmaxV[b] = std::max(bmaxV[b], V_of[k]);
            bmaxM[b] = std::max(bmaxM[b], m_of[k]);
        }
        for (int b = 0; b < kNumBuckets; b++) bstart[b + 1] += bstart[b];
        packed = false;
        return FLOCK_OK;
    }

    // Pack bucket b's costs (row pitch padded to 4) and quantities into the
    // pinned staging buffers (threads over instances), checking the cost
    // range in the same pass.  Returns false if an instance of the bucket
    // has a cost outside |c| <= 2^30 (flagged in cost_bad).
    bool pack_bucket(int b) { return pack_range(b, 0, bstart[b + 1] - bstart[b]); }
    // Pack instances [lo, hi) of bucket b (positions in its order).
    bool pack_range(int b, int lo, int hi) {
        std::atomic<int> bad{0};
        parallel_for(hi - lo, [&](int q) {
            const int k = order_[bstart[b] + lo + q];
            const int m = m_of[k], n = n_of[k], ldc = (n + 3) & ~3;
            int32_t* dst = h_cost.as<int32_t>() + cost_off[k];
            bool ok = true;
            if (ldc == n) {
                ok = copy_costs_checked(dst, insts[k].cost, m * n);
            } else {
                for (int i = 0; i < m; i++) {
                    ok &= copy_costs_checked(dst + (size_t)i * ldc, insts[k].cost + (size_t)i * n, n);
                    for (int j = n; j < ldc; j++) dst[(size_t)i * ldc + j] = 0;
                }
            }
            cost_checked[k] = 1;
            if (!ok) { cost_bad[k] = 1; bad.store(1); }
            memcpy(h_sd.as<int32_t>() + sd_off[k], insts[k].supply, (size_t)m * 4);
            memcpy(h_sd.as<int32_t>() + sd_off[k] + m, insts[k].demand, (size_t)n * 4);
        });
        return !bad.load();
    }

    // A cost range failure found while packing: wait for the buckets already
    // launched, check the instances not packed yet, and report the first
    // failing instance (validate_instance's error for it).
    int cost_failure() {
        for (auto s : st) cudaStreamSynchronize(s);
        parallel_for(count, [&](int k) {
            if (!cost_checked[k]) {
                cost_bad[k] = !costs_in_range(insts[k].cost, (size_t)m_of[k] * n_of[k]);
                cost_checked[k] = 1;
            }
        });
        packed = false;
        set_error("cost out of range");
        return FLOCK_ERR_RANGE;
    }

    // Pack and upload instances [lo, hi) of bucket b on stream s (their
    // cost and quantity ranges are contiguous in both arenas).
    int stage_range(int b, int lo, int hi, cudaStream_t s) {
        if (hi <= lo) return FLOCK_OK;
        if (!pack_range(b, lo, hi)) return cost_failure();
        const int k0 = order_[bstart[b] + lo], k1 = order_[bstart[b] + hi - 1];
        const int64_t c0 = cost_off[k0], c1 = cost_off[k1] + (int64_t)m_of[k1] * ((n_of[k1] + 3) & ~3);
        const int64_t s0 = sd_off[k0], s1 = sd_off[k1] + V_of[k1];
        FLOCK_CK(cudaMemcpyAsync(d_cost.as<int32_t>() + c0, h_cost.as<int32_t>() + c0, (size_t)(c1 - c0) * 4,
                                 cudaMemcpyHostToDevice, s));
        FLOCK_CK(cudaMemcpyAsync(d_sd.as<int32_t>() + s0, h_sd.as<int32_t>() + s0, (size_t)(s1 - s0) * 4,
                                 cudaMemcpyHostToDevice, s));
        return FLOCK_OK;
    }

    int ensure_device() {
        FLOCK_CK(d_cost.ensure((size_t)total_cost * 4 + 16));
        FLOCK_CK(d_sd.ensure((size_t)total_sd * 4 + 16));
        FLOCK_CK(d_desc.ensure(std::max<size_t>(1, descs.size()) * sizeof(BatchDesc)));
        FLOCK_CK(d_out.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(d_bfs.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(d_pot.ensure((size_t)total_pot * 8 + 16));
        FLOCK_CK(d_sc.ensure((size_t)count * sizeof(Scalars)));
        FLOCK_CK(d_ws.ensure((size_t)total_ws + 256));
        FLOCK_CK(h_desc.ensure(std::max<size_t>(1, descs.size()) * sizeof(BatchDesc)));
        FLOCK_CK(h_out.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(h_sc.ensure((size_t)count * sizeof(Scalars)));
        for (size_t q = 0; q < order_.size(); q++) {
            const int k = order_[q];
            BatchDesc& d = descs[q];
            d.m = m_of[k]; d.n = n_of[k]; d.ldc = (n_of[k] + 3) & ~3; d.index = k;
            d.cost = d_cost.as<int32_t>() + cost_off[k];
            d.sd = d_sd.as<int32_t>() + sd_off[k];
            d.ws = d_ws.as<uint8_t>() + ws_off[k];
            d.out = d_out.as<int32_t>() + 3 * out_off[k];
            d.bfs = d_bfs.as<int32_t>() + 3 * out_off[k];
            d.pot = d_pot.as<int64_t>() + pot_off[k];
            d.sc = d_sc.as<Scalars>() + k;
            d.done = nullptr;
        }
        if (!descs.empty()) memcpy(h_desc.p, descs.data(), descs.size() * sizeof(BatchDesc));
        return FLOCK_OK;
    }

    // FLOCK_BATCH_FORM=round|persistent forces the form (tests run both).
    TuneCfg cfg_for(int b) {
        TuneCfg t;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            t = g_tuned_ok[b] ? g_tuned[b] : default_cfg(bmaxV[b]);
        }
        // FLOCK_BATCH_THREADS="b:t,b:t": block size of bucket b (diagnostics).
        if (const char* bt = getenv("FLOCK_BATCH_THREADS")) {
            for (const char* p = bt; *p;) {
                int bb = -1, tt = 0, used = 0;
                if (sscanf(p, "%d:%d%n", &bb, &tt, &used) != 2) break;
                if (bb == b && (tt == 32 || tt == 64 || tt == 128 || tt == 256 || tt == 512 || tt == 1024)) t.threads = tt;
                p += used;
                if (*p == ',') p++;
            }
        }
        const char* f = getenv("FLOCK_BATCH_FORM");
        if (f && !strcmp(f, "round")) { t.persistent = 0; t.threads = std::min(std::max(t.threads, 128), 256); }
        if (f && !strcmp(f, "persistent")) t.persistent = 1;
        return t;
    }

    BatchArgs args_for(int b) {
        BatchArgs a;
        a.ph = nullptr;
        a.cost_smem = 0;
        block_pricing(a.pp);
        a.desc = d_desc.as<BatchDesc>() + bstart[b];
        a.count = bstart[b + 1] - bstart[b];
        a.next = nullptr; a.active = nullptr;
        a.maxV = bmaxV[b]; a.maxM = bmaxM[b];
        a.light = stage_light(bmaxV[b], bmaxM[b]) ? 1 : 0;
        a.bfs_method = opt.bfs_method == FLOCK_BFS_NWC ? FLOCK_BFS_NWC : FLOCK_BFS_VOGEL;
        a.mode = pivot_mode(opt);
        a.pricing = pricing_of(opt);
        a.max_rounds = opt.max_iterations > 0 ? opt.max_iterations : (1 << 30);
        return a;
    }

    int32_t* ctr(int b) { return d_ctr.as<int32_t>() + (size_t)b * 2 * kMaxChunk; }

    size_t bucket_smem(int b) { return launch_smem_bytes(bmaxV[b], bmaxM[b], stage_light(bmaxV[b], bmaxM[b])); }

    int grid_for(int b, const TuneCfg& t, size_t smem, const void* fn, int count = -1) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, t.threads, smem);
        if (per_sm < 1) per_sm = 1;
        const int nb = count >= 0 ? count : bstart[b + 1] - bstart[b];
        int g = std::max(1, std::min(nb, per_sm * num_sms() * t.grid_mult));
        // FLOCK_GRID_CAP="b:g,...": at most g blocks for bucket b (diagnostics)
        if (const char* e = getenv("FLOCK_GRID_CAP")) {
            for (const char* p = e; *p;) {
                int bb = -1, gg = 0, used = 0;
                if (sscanf(p, "%d:%d%n", &bb, &gg, &used) != 2) break;
                if (bb == b && gg >= 1) g = std::min(g, gg);
                p += used;
                if (*p == ',') p++;
            }
        }
        return g;
    }

    // Pricing rounds of bucket b as a CUDA graph: `chunk` x (zero the
    // counters, one k_bround launch).
    int capture_rounds(int b, const TuneCfg& t, cudaGraphExec_t* exec) {
        const size_t smem = bucket_smem(b);
        const int grid = grid_for(b, t, smem, (const void*)k_bround);
        cudaStream_t s = st[b];
        cudaGraph_t g;
        FLOCK_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int r = 0; r < t.chunk; r++) {
            BatchArgs a = args_for(b);
            a.next = ctr(b) + r;
            a.active = ctr(b) + kMaxChunk + r;
            cudaMemsetAsync(a.next, 0, sizeof(int32_t), s);
            cudaMemsetAsync(a.active, 0, sizeof(int32_t), s);
            k_bround<<<grid, t.threads, smem, s>>>(a);
        }
        FLOCK_CK(cudaStreamEndCapture(s, &g));
        FLOCK_CK(cudaGraphInstantiate(exec, g, 0));
        cudaGraphDestroy(g);
        return FLOCK_OK;
    }

    // Solve every staged bucket (all buckets concurrently, one stream each).
    // Inputs must already be on the device.  Returns when all are done.
    // stage: pack and upload each bucket's inputs on its stream right before
    // its launch (the descriptors must already be on the device).
    int run_device(const TuneCfg* cfg, float* ms, int only_bucket = -1, bool stage = false) {
        int rc;
        cudaStream_t s0 = st[0];
        FLOCK_CK(cudaEventRecord(ev_start, s0));
        for (int b = 1; b < kNumBuckets; b++) FLOCK_CK(cudaStreamWaitEvent(st[b], ev_start, 0));
        cudaGraphExec_t exec[kNumBuckets] = {};
        bool live[kNumBuckets] = {};
        launches = 0;
        bool chunked = false;     // the first bucket staged from the host goes in kStageChunks pieces
        // largest bucket first: its long solves start before the small ones
        for (int b = kNumBuckets - 1; b >= 0; b--) {
            const int nb = bstart[b + 1] - bstart[b];
            if (!nb || (only_bucket >= 0 && b != only_bucket)) continue;
            BatchArgs a = args_for(b);
            a.next = ctr(b);
            if (cfg[b].persistent) {
                const size_t smem = bucket_smem(b);
                const void* fn = bsolve_fn(cfg[b].threads);
                // staged from the host: the first bucket in chunks on their own
                // streams (each chunk's kernel starts once that chunk is
                // packed and uploaded); the largest instances lead
                const int K = stage && !chunked && nb >= 4 * kStageChunks ? kStageChunks : 1;
                chunked |= stage;
                for (int q = 0; q < K; q++) {
                    const int lo = (int)((int64_t)nb * q / K), hi = (int)((int64_t)nb * (q + 1) / K);
                    cudaStream_t sq = q == 0 ? st[b] : cst[q - 1];
                    if (q > 0) FLOCK_CK(cudaStreamWaitEvent(sq, ev_start, 0));
                    if (stage && (rc = stage_range(b, lo, hi, sq))) return rc;
                    BatchArgs aq = a;
                    aq.desc = a.desc + lo;
                    aq.count = hi - lo;
                    aq.next = ctr(b) + q;       // one work-stealing counter per chunk
                    FLOCK_CK(cudaMemsetAsync(aq.next, 0, sizeof(int32_t), sq));
                    void* kargs[] = {&aq};
                    FLOCK_CK(cudaLaunchKernel(fn, dim3(grid_for(b, cfg[b], smem, fn, hi - lo)), dim3(cfg[b].threads),
                                              kargs, smem, sq));
                    launches++;
                    if (q > 0) {
                        FLOCK_CK(cudaEventRecord(ev_join, sq));
                        FLOCK_CK(cudaStreamWaitEvent(st[b], ev_join, 0));
                    }
                }
                continue;
            }
            if (stage && (rc = stage_range(b, 0, nb, st[b]))) return rc;
            live[b] = true;
            FLOCK_CK(cudaMemsetAsync(a.next, 0, sizeof(int32_t), st[b]));
            k_bsetup<<<grid_for(b, cfg[b], 0, (const void*)k_bsetup), cfg[b].threads, 0, st[b]>>>(a);
            FLOCK_CK(cudaGetLastError());
            launches++;
            if ((rc = capture_rounds(b, cfg[b], &exec[b]))) return rc;
        }
        int32_t* hc = h_ctr.as<int32_t>();
        for (int guard = 0; guard < (1 << 26); guard++) {
            bool any = false;
            for (int b = 0; b < kNumBuckets; b++) {
                if (!live[b]) continue;
                any = true;
                FLOCK_CK(cudaGraphLaunch(exec[b], st[b]));
                launches += cfg[b].chunk;
                FLOCK_CK(cudaMemcpyAsync(hc + (size_t)b * 2 * kMaxChunk + kMaxChunk, ctr(b) + kMaxChunk,
                                         (size_t)cfg[b].chunk * sizeof(int32_t), cudaMemcpyDeviceToHost, st[b]));
            }
            if (!any) break;
            for (int b = 0; b < kNumBuckets; b++) {
                if (!live[b]) continue;
                FLOCK_CK(cudaStreamSynchronize(st[b]));
                if (hc[(size_t)b * 2 * kMaxChunk + kMaxChunk + cfg[b].chunk - 1] == 0) {
                    live[b] = false;
                    BatchArgs a = args_for(b);
                    a.next = ctr(b);
                    FLOCK_CK(cudaMemsetAsync(a.next, 0, sizeof(int32_t), st[b]));
                    k_bfinal<<<grid_for(b, cfg[b], 0, (const void*)k_bfinal), cfg[b].threads, 0, st[b]>>>(a);
                    FLOCK_CK(cudaGetLastError());
                    launches++;
                }
            }
        }
        for (int b = 0; b < kNumBuckets; b++) if (exec[b]) cudaGraphExecDestroy(exec[b]);
        for (int b = 1; b < kNumBuckets; b++) {
            FLOCK_CK(cudaEventRecord(ev_join, st[b]));
            FLOCK_CK(cudaStreamWaitEvent(s0, ev_join, 0));
        }
        FLOCK_CK(cudaEventRecord(ev_done, s0));
        FLOCK_CK(cudaEventSynchronize(ev_done));
        if (ms) cudaEventElapsedTime(ms, ev_start, ev_done);
        return FLOCK_OK;
    }

    // Upload every staged input (packing the buckets not packed yet).
    int upload() {
        cudaStream_t s0 = st[0];
        if (!packed) {
            bool ok = true;
            for (int b = 0; b < kNumBuckets; b++) ok &= pack_bucket(b);
            if (!ok) return cost_failure();
            packed = true;
        }
        if (total_cost) FLOCK_CK(cudaMemcpyAsync(d_cost.p, h_cost.p, (size_t)total_cost * 4, cudaMemcpyHostToDevice, s0));
        if (total_sd) FLOCK_CK(cudaMemcpyAsync(d_sd.p, h_sd.p, (size_t)total_sd * 4, cudaMemcpyHostToDevice, s0));
        if (!descs.empty())
            FLOCK_CK(cudaMemcpyAsync(d_desc.p, h_desc.p, descs.size() * sizeof(BatchDesc), cudaMemcpyHostToDevice, s0));
        return FLOCK_OK;
    }

    int download() {
        cudaStream_t s0 = st[0];
        FLOCK_CK(cudaMemcpyAsync(h_out.p, d_out.p, (size_t)total_cells * 12, cudaMemcpyDeviceToHost, s0));
        FLOCK_CK(cudaMemcpyAsync(h_sc.p, d_sc.p, (size_t)count * sizeof(Scalars), cudaMemcpyDeviceToHost, s0));
        FLOCK_CK(cudaStreamSynchronize(s0));
        return FLOCK_OK;
    }

    // Whole solve: upload, device rounds, download, then the large instances
    // on the plain path.  Blocking.
    float last_ms = 0;
    int solve_all() {
        int rc = ensure_device();
        if (rc) return rc;
        TuneCfg cfg[kNumBuckets];
        for (int b = 0; b < kNumBuckets; b++) cfg[b] = cfg_for(b);
        if (packed) {
            if ((rc = upload())) return rc;
            if ((rc = run_device(cfg, &last_ms))) return rc;
        } else {
            // descriptors first, then each bucket packed, uploaded and
            // launched in turn (largest first) so host packing overlaps with
            // the device work already launched
            if (!descs.empty())
                FLOCK_CK(cudaMemcpyAsync(d_desc.p, h_desc.p, descs.size() * sizeof(BatchDesc), cudaMemcpyHostToDevice,
                                         st[0]));
            if ((rc = run_device(cfg, &last_ms, -1, true))) return rc;
            packed = true;
        }
        if ((rc = download())) return rc;
        plain_stats.assign(plain_list.size(), flock_stats{});
        plain_flows.assign(plain_list.size(), {});
        for (size_t q = 0; q < plain_list.size(); q++) {
            const int k = plain_list[q];
            plain_flows[q].resize((size_t)V_of[k] - 1);
            rc = solve_plain(&insts[k], &opt, plain_flows[q].data(), nullptr, nullptr, &plain_stats[q]);
            if (rc && rc != FLOCK_ERR_NOT_OPTIMAL) return rc;
        }
        return FLOCK_OK;
    }

    // Device-resident rerun for the benchmark: inputs stay where they are.
    int rerun_device_only(float* ms) {
        TuneCfg cfg[kNumBuckets];
        for (int b = 0; b < kNumBuckets; b++) cfg[b] = cfg_for(b);
        return run_device(cfg, ms);
    }

    void collect(int k, flock_flow* flows, flock_stats* st_out) const {
        if (V_of[k] > kMaxStagedV) {
            for (size_t q = 0; q < plain_list.size(); q++)
                if (plain_list[q] == k) {
                    if (flows) memcpy(flows, plain_flows[q].data(), plain_flows[q].size() * sizeof(flock_flow));
                    if (st_out) *st_out = plain_stats[q];
                }
            return;
        }
        const Scalars& S = h_sc.as<Scalars>()[k];
        const int V = V_of[k];
        const int32_t* src = h_out.as<int32_t>() + 3 * out_off[k];
        const int32_t* dst = src + (V - 1);
        const int32_t* qty = src + 2 * (V - 1);
        const bool broken = S.status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE);
        if (flows && !broken) fill_flows_from_basis(V, src, dst, qty, flows);
        if (st_out) {
            int status = S.status & kFailMask;
            if (opt.verify && S.cert) status |= ST_CERT_FAIL;
            st_out->notes = (S.status & ~kFailMask) | (S.fail_site << 8);
            st_out->objective = S.objective;
            st_out->iterations = S.rounds;
            st_out->pivots = S.pivots;
            st_out->active_flows = broken ? 0 : S.active;
            st_out->status = status;
            st_out->certified = (!broken && S.cert == 0) ? 1 : 0;
            st_out->vogel_events = S.events;
            st_out->ms_total = 0; st_out->ms_bfs = 0; st_out->ms_simplex = 0;
            st_out->ms_dual = st_out->ms_sweep = st_out->ms_pivot = 0;
            st_out->ms_cycle = st_out->ms_resolve = st_out->ms_adjust = 0;
        }
    }

    // Autotune each bucket with enough instances: the bucket alone is solved
    // once per candidate configuration (inputs resident) and the fastest wins;
    // then the block sizes are refined with all buckets running together.
    // Candidates: the persistent form at three block sizes scaled to the
    // bucket's largest instance, and the round form at 128/256 threads.
    int autotune() {
        bool need = false;
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            for (int b = 0; b < kNumBuckets; b++)
                if (!g_tuned_ok[b] && bstart[b + 1] - bstart[b] >= 32) need = true;
        }
        if (!need) return FLOCK_OK;
        int rc = ensure_device();
        if (rc) return rc;
        if ((rc = upload())) return rc;
        FLOCK_CK(cudaStreamSynchronize(st[0]));
        for (int b = 0; b < kNumBuckets; b++) {
            const int nb = bstart[b + 1] - bstart[b];
            {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                if (g_tuned_ok[b] || nb < 32) continue;
            }
            std::vector<TuneCfg> cands;
            // persistent form: three block sizes around the bucket's size
            const int V = bmaxV[b];
            const int t0 = V <= 128 ? 32 : V <= 256 ? 64 : V <= 512 ? 128 : 256;
            for (int t = t0; t <= 4 * t0; t *= 2) cands.push_back(TuneCfg{t, 1, 16, 1});
            // round form (graph-captured chunks of k_bround)
            const int thr[2] = {128, 256};
            for (int ti = 0; ti < 2; ti++) {
                if (thr[ti] == 128 && bmaxV[b] > 256) continue;
                for (int gm = 1; gm <= 2; gm++)
                    for (int ch : {8, 32}) cands.push_back(TuneCfg{thr[ti], gm, ch, 0});
            }
            float best_ms = 1e30f;
            TuneCfg best = default_cfg(bmaxV[b]);
            for (const TuneCfg& t : cands) {
                TuneCfg cfg[kNumBuckets];
                for (int x = 0; x < kNumBuckets; x++) cfg[x] = t;
                float ms = 0;
                if ((rc = run_device(cfg, &ms, b))) return rc;
                if (getenv("FLOCK_TUNE_LOG"))
                    fprintf(stderr, "  bucket %d candidate %s threads=%d grid_mult=%d chunk=%d: %.3f ms\n", b,
                            t.persistent ? "persistent" : "rounds", t.threads, t.grid_mult, t.chunk, ms);
                if (ms < best_ms) { best_ms = ms; best = t; }
            }
            if (getenv("FLOCK_TUNE_LOG"))
                fprintf(stderr, "flock autotune: bucket %d (%d instances, V <= %d): %s threads=%d grid_mult=%d chunk=%d  %.3f ms\n",
                        b, nb, bmaxV[b], best.persistent ? "persistent" : "rounds", best.threads, best.grid_mult,
                        best.chunk, best_ms);
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned[b] = best;
            g_tuned_ok[b] = true;
        }
        return tune_jointly();
    }

    // Second stage: the buckets share the GPU in a real solve, where a block
    // size that is fastest for a bucket alone (its longest instance finishes
    // first) can cost throughput.  One coordinate-descent pass over the
    // buckets, largest first, tries each persistent bucket's block sizes with
    // every bucket running; a change is kept when the whole batch gets at
    // least 2 % faster.
    int tune_jointly() {
        TuneCfg cur[kNumBuckets];
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            for (int b = 0; b < kNumBuckets; b++) cur[b] = g_tuned_ok[b] ? g_tuned[b] : default_cfg(bmaxV[b]);
        }
        int rc;
        float best_ms = 0;
        if ((rc = run_device(cur, &best_ms))) return rc;
        if ((rc = run_device(cur, &best_ms))) return rc;
        for (int b = kNumBuckets - 1; b >= 0; b--) {
            const int nb = bstart[b + 1] - bstart[b];
            if (nb < 32 || !cur[b].persistent) continue;
            const int V = bmaxV[b];
            const int t0 = V <= 128 ? 32 : V <= 256 ? 64 : V <= 512 ? 128 : 256;
            for (int t = t0; t <= 4 * t0; t *= 2) {
                if (t == cur[b].threads) continue;
                TuneCfg trial[kNumBuckets];
                for (int x = 0; x < kNumBuckets; x++) trial[x] = cur[x];
                trial[b].threads = t;
                float ms = 0;
                if ((rc = run_device(trial, &ms))) return rc;
                if (getenv("FLOCK_TUNE_LOG"))
                    fprintf(stderr, "  joint: bucket %d threads=%d: %.3f ms (current %.3f ms)\n", b, t, ms, best_ms);
                if (ms < 0.98f * best_ms) { best_ms = ms; cur[b] = trial[b]; }
            }
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        for (int b = 0; b < kNumBuckets; b++)
            if (g_tuned_ok[b]) g_tuned[b] = cur[b];
        if (getenv("FLOCK_TUNE_LOG"))
            for (int b = 0; b < kNumBuckets; b++)
                if (g_tuned_ok[b])
                    fprintf(stderr, "flock autotune (joint): bucket %d: %s threads=%d\n", b,
                            cur[b].persistent ? "persistent" : "rounds", cur[b].threads);
        return FLOCK_OK;
    }
};

// ------------------------------------------------------------ served form ---
// Helpers for the served form (serve.cu): a request's device region, the
// launch of one admission group, and its result.
ServeLayout serve_layout(int m, int n) {
    const int V = m + n, ldc = (n + 3) & ~3;
    ServeLayout L;
    size_t o = 0;
    L.cost = o; o = al256(o + (size_t)m * ldc * 4);
    L.sd = o;   o = al256(o + (size_t)V * 4);
    L.ws = o;   o = al256(o + instance_ws_bytes(V, m));
    L.out = o;  o = al256(o + (size_t)3 * (V - 1) * 4);
    L.bfs = o;  o = al256(o + (size_t)3 * (V - 1) * 4);
    L.pot = o;  o = al256(o + (size_t)V * 8);
    L.sc = o;   o = al256(o + sizeof(Scalars));
    L.total = o;
    return L;
}

int serve_init() {
    for (int t : {256, 512, 1024})
        FLOCK_CK(cudaFuncSetAttribute(bsolve_fn(t), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kStageSmemMax));
    return FLOCK_OK;
}

// Block size of a served launch by its largest instance, latency first: the
// one-launch plain solver's sizes (FLOCK_SERVE_THREADS=64..1024, a multiple
// of 32, overrides it, for tuning).
static int serve_threads(int maxV) {
    if (const char* e = getenv("FLOCK_SERVE_THREADS")) {
        const int t = atoi(e);
        if (t >= 64 && t <= 1024 && t % 32 == 0) return t;
    }
    return maxV <= 128 ? 128 : maxV <= 512 ? 256 : 1024;
}

int serve_launch(const BatchDesc* d_desc, int count, int maxV, int maxM, const flock_options& opt, int32_t* d_next,
                 cudaStream_t s) {
    if (count < 1 || maxV > kMaxStagedV) return FLOCK_ERR_ARG;
    BatchArgs a;
    a.ph = nullptr;
    a.cost_smem = 0;
    block_pricing(a.pp);
    a.desc = d_desc;
    a.count = count;
    a.next = d_next;
    a.active = nullptr;
    a.maxV = maxV; a.maxM = maxM;
    a.bfs_method = opt.bfs_method == FLOCK_BFS_NWC ? FLOCK_BFS_NWC : FLOCK_BFS_VOGEL;
    a.mode = pivot_mode(opt);
    a.pricing = pricing_of(opt);
    a.max_rounds = opt.max_iterations > 0 ? opt.max_iterations : (1 << 30);
    a.light = stage_light(maxV, maxM) ? 1 : 0;
    const size_t smem = launch_smem_bytes(maxV, maxM, a.light != 0);
    const int threads = serve_threads(maxV);
    const void* fn = bsolve_fn(threads);
    int per_sm = 0;
    FLOCK_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem));
    const int grid = std::max(1, std::min(count, std::max(1, per_sm) * num_sms()));
    void* kargs[] = {&a};
    FLOCK_CK(cudaLaunchKernel(fn, dim3(grid), dim3(threads), kargs, smem, s));
    return FLOCK_OK;
}

void serve_collect(const Scalars& S, int V, const int32_t* out3, flock_flow* flows, flock_stats* st) {
    const bool broken = S.status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE);
    if (flows && !broken) fill_flows_from_basis(V, out3, out3 + (V - 1), out3 + 2 * (V - 1), flows);
    if (st) {
        memset(st, 0, sizeof(*st));
        st->notes = (S.status & ~kFailMask) | (S.fail_site << 8);
        st->objective = S.objective;
        st->iterations = S.rounds;
        st->pivots = S.pivots;
        st->active_flows = broken ? 0 : S.active;
        st->status = (S.status & kFailMask) | (S.cert ? ST_CERT_FAIL : 0);
        st->certified = (!broken && S.cert == 0) ? 1 : 0;
        st->vogel_events = S.events;
    }
}

static std::mutex g_batch_mu;
static BatchRunner* g_batch = nullptr;

static int batch_solve(int cnt, const flock_instance* insts, const flock_options* opt, flock_flow* flows,
                       const int64_t* flow_offset, flock_stats* stats) {
    if (cnt < 0 || (cnt > 0 && !insts)) return FLOCK_ERR_ARG;
    if (cnt == 0) return FLOCK_OK;
    const auto t0 = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (!g_batch) g_batch = new BatchRunner();
    BatchRunner& R = *g_batch;
    int rc = R.prepare(cnt, insts, opt);
    if (rc) return rc;
    const auto t1 = std::chrono::steady_clock::now();
    const char* at = getenv("FLOCK_AUTOTUNE");
    if (!at || strcmp(at, "0") != 0) { if ((rc = R.autotune())) return rc; }
    const auto t2 = std::chrono::steady_clock::now();
    if ((rc = R.solve_all())) return rc;
    const auto t3 = std::chrono::steady_clock::now();
    const float ms = R.last_ms;
    std::vector<int64_t> off(cnt);
    int64_t o = 0;
    for (int k = 0; k < cnt; k++) { off[k] = flow_offset ? flow_offset[k] : o; o += R.V_of[k] - 1; }
    std::atomic<int> bad{0};
    const double total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    parallel_for(cnt, [&](int k) {
        flock_stats s;
        R.collect(k, flows ? flows + off[k] : nullptr, &s);
        s.ms_total = total;
        s.ms_simplex = ms;
        if (stats) stats[k] = s;
        if (s.status) bad.store(1);
    });
    if (getenv("FLOCK_TIMING")) {
        auto ms_ = [](std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
            return std::chrono::duration<double, std::milli>(b - a).count();
        };
        fprintf(stderr, "flock_batch_solve: validate+layout %.2f ms, autotune %.2f ms, stage+solve+download %.2f ms "
                        "(device %.2f ms), collect %.2f ms\n", ms_(t0, t1), ms_(t1, t2), ms_(t2, t3), ms, 
                ms_(t3, std::chrono::steady_clock::now()));
    }
    return bad.load() ? FLOCK_ERR_NOT_OPTIMAL : FLOCK_OK;
}

// Benchmark hook: cost cells priced by the CTA sweeps of the last batch
// (every instance solved by the batched kernels).
int batch_cells(int64_t* cells) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (!g_batch || !cells) return FLOCK_ERR_ARG;
    int64_t t = 0;
    for (int k = 0; k < g_batch->count; k++)
        if (g_batch->V_of[k] <= kMaxStagedV) t += g_batch->h_sc.as<Scalars>()[k].cells;
    *cells = t;
    return FLOCK_OK;
}

// Device-only timing hook for the benchmark: solve the last staged batch
// again with its inputs already resident.  Returns the kernel time in ms.
int batch_rerun_device(float* ms, int32_t* launches) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (!g_batch) return FLOCK_ERR_ARG;
    const int rc = g_batch->rerun_device_only(ms);
    if (launches) *launches = g_batch->launches;
    return rc;
}

}  // namespace flock

// ================================================================ C ABI ===
extern "C" {

void flock_default_options(flock_options* opt) {
    if (!opt) return;
    opt->bfs_method = FLOCK_BFS_VOGEL;
    opt->pivot_method = FLOCK_PIVOT_SWITCH;
    opt->max_iterations = 0;
    opt->verify = 1;
    opt->pricing = FLOCK_PRICING_PARTIAL;
}

const char* flock_last_error(void) { return flock::g_err.c_str(); }
const char* flock_version(void) { return "flock-gb300 0.1 (sm_103a)"; }

int flock_vogel(const flock_instance* inst, flock_flow* flows, int32_t* events) {
    if (!flows) return FLOCK_ERR_ARG;
    return flock::vogel_plain(inst, flows, events);
}

int flock_vogel_device(const flock_instance* inst, flock_flow* flows, int32_t* events) {
    if (!flows) return FLOCK_ERR_ARG;
    return flock::vogel_plain(inst, flows, events, true);
}

int flock_solve(const flock_instance* inst, const flock_options* opt, flock_flow* flows,
                int64_t* duals_u, int64_t* duals_v, flock_stats* stats) {
    return flock::solve_plain(inst, opt, flows, duals_u, duals_v, stats);
}

int flock_batch_solve(int32_t count, const flock_instance* insts, const flock_options* opt,
                      flock_flow* flows, const int64_t* flow_offset, flock_stats* stats) {
    return flock::batch_solve(count, insts, opt, flows, flow_offset, stats);
}

/* Benchmark hook (not part of the public header): rerun the last batch with
 * its inputs resident on the device and report the device time. */
int flock_bench_batch_rerun(float* ms, int32_t* launches) { return flock::batch_rerun_device(ms, launches); }

/* Benchmark hook: cost cells priced by the batched kernels' sweeps in the last
 * batch (after a re-solve, the re-solve's count). */
int flock_bench_batch_cells(int64_t* cells) { return flock::batch_cells(cells); }

// Benchmark hook: CTAs of the grid path's cluster rounds on this device (0:
// the six-kernel rounds only).
int flock_bench_cluster_ctas(int32_t* ctas) {
    if (!ctas) return FLOCK_ERR_ARG;
    flock::PlainSolver& P = flock::plain();
    std::lock_guard<std::mutex> lk(P.mu);
    const int rc = P.setup();
    if (rc) return rc;
    *ctas = P.cluster_ctas;
    return FLOCK_OK;
}

/* Benchmark hook: average device time of the fused reduced-cost sweep on an
 * m x n matrix (random costs and duals, inputs resident). */
int flock_bench_sweep(int32_t m, int32_t n, int32_t iters, float* avg_ms, int32_t* tile) {
    return flock::bench_sweep(m, n, iters, avg_ms, tile);
}

/* Benchmark hook: average device time of an L2 read-bandwidth kernel making
 * `passes` passes over a buffer of `bytes` per launch. */
int flock_bench_l2(int64_t bytes, int32_t passes, int32_t iters, float* avg_ms) {
    return flock::bench_l2(bytes, passes, iters, avg_ms);
}

/* Test hook: partial pricing's candidate-row selection over host row keys
 * (prow needs room for the returned pp_rows entries). */
int flock_test_select_rows(int32_t m, const uint64_t* keys, uint64_t* keys_out, int32_t* prow, int32_t* pn,
                           int32_t* pp_rows, uint64_t* best, int32_t threads) {
    return flock::test_select_rows(m, keys, keys_out, prow, pn, pp_rows, best, threads);
}

/* Test hook (host only, no CUDA call): the batch call's parallel loop over
 * count items, each adding 1 to hits[item]. */
int flock_test_parallel_for(int32_t count, int32_t* hits) {
    if (count < 0 || (count > 0 && !hits)) return FLOCK_ERR_ARG;
    flock::parallel_for(count, [&](int k) { hits[k]++; });
    return FLOCK_OK;
}

/* Test hook: one reduced-cost sweep over host costs and duals, row keys back
 * (cta_form 0: the bulk sweep; > 0: the one-block sweep with `threads`;
 * < 0: the bulk sweep on the 16-bit copy of the costs). */
int flock_test_sweep(int32_t m, int32_t n, const int32_t* cost, const int64_t* pot, uint64_t* keys,
                     int32_t cta_form, int32_t threads) {
    return flock::test_sweep(m, n, cost, pot, keys, cta_form, threads);
}

}  // extern "C"

// ======================================================= static scratch ===
// flock_vogel_static: Vogel's approximation on the GPU without any
// allocation.  Every device array of the call (the padded cost
// matrix, supplies/demands, the Vogel working set, the packed flow list and
// the status scalars) is carved from one file-scope __device__ array of fixed
// size, so a call makes no cudaMalloc/cudaFree, no pinned-host allocation and
// no stream or event creation.  The device code is the same vogel_cta that
// flock_vogel runs; results are identical.
//
// Limits: m + n <= FLOCK_VOGEL_STATIC_MAX_V and m * ceil4(n) <=
// FLOCK_VOGEL_STATIC_MAX_CELLS (include/flock.h); larger instances are
// rejected with FLOCK_ERR_RANGE before any CUDA call.
//
// Set-up: the first call on a device resolves the scratch array's device
// address with cudaGetSymbolAddress, with that device current, and caches it
// for the device together with the id of the CUDA context it belongs to.  A
// per-device lock makes the set-up safe when several host threads make their
// first call at once.  A later call in a different context of that device
// (after cudaDeviceReset the runtime makes a new primary context, where the
// array may lie elsewhere) repeats the set-up.  The first call on a device
// loads the module and should come before any stream capture.
//
// Concurrency: every call on one device uses the same scratch, so calls that
// overlap in time (several host threads, or a caller reusing the stream while
// a call is in flight) race on it.  Callers serialise.

namespace flock {
namespace {

constexpr size_t kStaticBytes = size_t(6) << 20;   // 6 MiB per device
static __device__ __align__(256) unsigned char g_vogel_scratch[kStaticBytes];

constexpr int kMaxDevices = 64;
// Per-device cache of the scratch array's address, valid in the context
// whose id it records; guarded by its lock.
struct ScratchSlot {
    std::mutex mu;
    void* ptr = nullptr;
    unsigned long long ctx_id = 0;
};
ScratchSlot g_scratch_slot[kMaxDevices];

size_t al(size_t x) { return (x + 255) & ~size_t(255); }

int cuda_err(const char* what, cudaError_t e) {
    set_error(std::string("flock_vogel_static: ") + what + ": " + cudaGetErrorString(e));
    return FLOCK_ERR_CUDA;
}

// The driver's cuCtxGetCurrent and cuCtxGetId, fetched through the runtime
// (no link against the driver library).  Signatures of CUDA 12.0.
typedef int (*CtxGetCurrentFn)(void** ctx);
typedef int (*CtxGetIdFn)(void* ctx, unsigned long long* id);
struct CtxFns {
    CtxGetCurrentFn get_current = nullptr;
    CtxGetIdFn get_id = nullptr;
};
const CtxFns& ctx_fns() {
    static CtxFns f;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.get_current = (CtxGetCurrentFn)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            f.get_id = (CtxGetIdFn)p;
    });
    return f;
}

// Id of the context current on this thread; 0 when none is current yet or
// the driver does not say.
unsigned long long current_ctx_id() {
    const CtxFns& f = ctx_fns();
    if (!f.get_current || !f.get_id) return 0;
    void* ctx = nullptr;
    if (f.get_current(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    return f.get_id(ctx, &id) == 0 ? id : 0;
}

// Device address of the scratch array on device `dev` (current), from the
// device's cache when it was resolved in the current context.
int scratch_address(int dev, unsigned char** out) {
    ScratchSlot& slot = g_scratch_slot[dev];
    std::lock_guard<std::mutex> lk(slot.mu);
    unsigned long long id = current_ctx_id();
    if (slot.ptr && id != 0 && id == slot.ctx_id) {
        *out = (unsigned char*)slot.ptr;
        return FLOCK_OK;
    }
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_vogel_scratch);   // binds the context if none was
    if (e != cudaSuccess) return cuda_err("cudaGetSymbolAddress", e);
    if (id == 0) id = current_ctx_id();
    slot.ptr = p;
    slot.ctx_id = id;
    *out = (unsigned char*)p;
    return FLOCK_OK;
}

// Byte offsets of the regions inside the scratch array for one instance.
struct Layout {
    size_t cost, sd, ws, flows, sc, end;
};
Layout layout_for(int m, int n) {
    const int V = m + n, ldc = (n + 3) & ~3;
    Layout L;
    L.cost = 0;
    L.sd = al(L.cost + (size_t)m * ldc * 4);
    L.ws = al(L.sd + (size_t)V * 4);
    size_t gbytes = 0;
    Ctx probe;
    carve_ctx(probe, nullptr, V, m, nullptr, nullptr, nullptr, &gbytes);
    L.flows = al(L.ws + gbytes);
    L.sc = al(L.flows + (size_t)(V - 1) * sizeof(flock_flow));
    L.end = L.sc + sizeof(Scalars);
    return L;
}

// The largest admitted shapes both fit: m+n at the vertex limit with the cell
// limit spent on few rows, and the cell limit with a square matrix.
bool fits(int m, int n) { return layout_for(m, n).end <= kStaticBytes; }

}  // namespace

// Variant of k_vogel_only that also packs the allocation list into the
// caller's flow layout, so one device-to-host copy returns it.
__global__ void __launch_bounds__(1024) k_vogel_static(Ctx c, flock_flow* out) {
    __shared__ BlockScratch bs;
    vogel_cta(c, bs);
    const int V = c.I.m + c.I.n;
    for (int k = threadIdx.x; k < V - 1; k += blockDim.x) out[k] = {c.bfs_src[k], c.bfs_dst[k], c.bfs_qty[k]};
}

static int vogel_static(const flock_instance* I, flock_flow* flows, int32_t* events) {
    int rc = validate_instance(I);
    if (rc) return rc;
    const int m = I->m, n = I->n, V = m + n, ldc = (n + 3) & ~3;
    if (V > FLOCK_VOGEL_STATIC_MAX_V || (int64_t)m * ldc > FLOCK_VOGEL_STATIC_MAX_CELLS || !fits(m, n)) {
        set_error("flock_vogel_static: instance exceeds the static scratch (m + n <= " +
                  std::to_string(FLOCK_VOGEL_STATIC_MAX_V) + " and m * ceil4(n) <= " +
                  std::to_string(FLOCK_VOGEL_STATIC_MAX_CELLS) + " required)");
        return FLOCK_ERR_RANGE;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_err("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) { set_error("flock_vogel_static: device ordinal out of range"); return FLOCK_ERR_ARG; }
    unsigned char* base = nullptr;
    if ((rc = scratch_address(dev, &base))) return rc;
    const Layout L = layout_for(m, n);
    cudaStream_t s = cudaStreamPerThread;

    Ctx c;
    carve_ctx(c, base + L.ws, V, m, nullptr, nullptr);
    c.I.m = m; c.I.n = n; c.I.ldc = ldc;
    c.I.cost = (const int32_t*)(base + L.cost);
    c.I.supply = (const int32_t*)(base + L.sd);
    c.I.demand = (const int32_t*)(base + L.sd) + m;
    c.sc = (Scalars*)(base + L.sc);
    flock_flow* dflows = (flock_flow*)(base + L.flows);

    // Inputs.  The padding columns of the cost rows are never read.
    e = cudaMemcpy2DAsync(base + L.cost, (size_t)ldc * 4, I->cost, (size_t)n * 4, (size_t)n * 4, m,
                          cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_err("cost upload", e);
    e = cudaMemcpyAsync(base + L.sd, I->supply, (size_t)m * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_err("supply upload", e);
    e = cudaMemcpyAsync(base + L.sd + (size_t)m * 4, I->demand, (size_t)n * 4, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_err("demand upload", e);
    // The status scalars (events, status, fail site) must start at zero; the
    // Vogel working arrays are initialised by the kernel itself.
    e = cudaMemsetAsync(c.sc, 0, sizeof(Scalars), s);
    if (e != cudaSuccess) return cuda_err("scalar reset", e);

    const int nt = std::max(128, std::min(1024, ((V + 31) / 32) * 32));
    k_vogel_static<<<1, nt, 0, s>>>(c, dflows);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err("k_vogel_static launch", e);

    Scalars hs;
    e = cudaMemcpyAsync(flows, dflows, (size_t)(V - 1) * sizeof(flock_flow), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_err("flow download", e);
    e = cudaMemcpyAsync(&hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_err("scalar download", e);
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err("k_vogel_static", e);
    if ((rc = vogel_status_check(hs, "flock_vogel_static"))) return rc;
    if (events) *events = hs.events;
    return FLOCK_OK;
}

}  // namespace flock

extern "C" int flock_vogel_static(const flock_instance* inst, flock_flow* flows, int32_t* events) {
    if (!flows) return FLOCK_ERR_ARG;
    return flock::vogel_static(inst, flows, events);
}
