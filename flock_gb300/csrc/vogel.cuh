// vogel.cuh -- Vogel's approximation on the device with the exact semantics of
// the reference's sequential host routine (find_vogel_bfs_sequencial,
// src/parallel_simplex_method/IBFS_vogel.cu:546-769):
//
//  * penalties are refreshed for ALL rows only after a step that covered a row,
//    for ALL columns only after a step that covered a column (both at the
//    start); otherwise the stored values stay stale (:570,:588-642);
//  * penalty = second-cheapest - cheapest uncovered crossing cost, computed in
//    float and converted to int as x86 does (one uncovered cell: float(2^31)-c,
//    which is INT_MIN when it rounds to 2^31; none: 0); covered lines -1;
//  * the chosen line is the LAST index with the maximal penalty over
//    [rows, columns] (:651-659);
//  * in that line the FIRST cheapest uncovered crossing cell is used
//    (:671-676, :721-727); if there is none the reference reuses the previous
//    step's index, which is reproduced (and counted) while it is in range;
//  * min(residual supply, residual demand) is allocated; a tie covers the
//    column (:691, :739).
//
// Instead of rescanning every uncovered line per refresh (O(V*m*n) in the
// reference), each line caches its two cheapest uncovered crossing cells.  A
// cache stays exact until one of those two crossing lines is covered; only
// then is the line rescanned, with a warp-shuffle (or block-wide) top-2
// reduction.  The penalties written at each refresh are therefore identical
// to a full recomputation.
#pragma once
#include "device.cuh"

namespace flock {

__device__ __forceinline__ int32_t vogel_penalty(int4 t) {
    long long c1 = t.z >= 0 ? (long long)t.x : 2147483648LL;
    long long c2 = t.w >= 0 ? (long long)t.y : 2147483648LL;
    // float(c2) - float(c1) is exact-then-rounded for |c| <= 2^24.
    return f2i_x86(__ll2float_rn(c2 - c1));
}

__device__ __forceinline__ int4 top2_from_keys(uint64_t a1, uint64_t a2) {
    int4 t;
    t.x = a1 == kNoKey ? 0 : key_val(a1);
    t.y = a2 == kNoKey ? 0 : key_val(a2);
    t.z = a1 == kNoKey ? -1 : (int32_t)key_idx(a1);
    t.w = a2 == kNoKey ? -1 : (int32_t)key_idx(a2);
    return t;
}

// crossing line of line L at crossing index x
__device__ __forceinline__ int crossing_vertex(int L, int x, int m) { return L < m ? m + x : x; }

__device__ __forceinline__ bool top2_valid(const Ctx& c, int L, int4 t) {
    const int m = c.I.m;
    if (t.z == -2) return false;                  // never built
    if (t.z < 0) return true;                     // nothing uncovered: stays so
    if (c.covered[crossing_vertex(L, t.z, m)]) return false;
    if (t.w >= 0 && c.covered[crossing_vertex(L, t.w, m)]) return false;
    return true;
}

// This thread's share (crossing indices first, first + step, ...) of line
// L's two cheapest uncovered crossing cells.  kWide (instances whose line
// state is in global memory): eight (four along a column read row by row)
// crossings' loads issued together, and a
// column read from the column-major copy costT (n rows of ceil4(m)) when
// there is one, instead of one row per element.
template <bool kWide>
__device__ __forceinline__ void vogel_scan(const Ctx& c, int L, int first, int step, const int32_t* costT,
                                           uint64_t& a1, uint64_t& a2) {
    const InstDev& I = c.I;
    a1 = kNoKey; a2 = kNoKey;
    const int32_t* line = nullptr;
    const uint8_t* cov = nullptr;
    int len = 0;
    if (L < I.m) { line = I.cost + (size_t)L * I.ldc; cov = c.covered + I.m; len = I.n; }
    else if (kWide && costT) { line = costT + (size_t)(L - I.m) * ((I.m + 3) & ~3); cov = c.covered; len = I.m; }
    if (line) {
        if (kWide) {
            // eight crossings' loads in flight (a rescan's stride leaves a lane
            // about len / (32 g) crossings: one or two batches at 8000)
            int x = first;
            for (; x + 7 * step < len; x += 8 * step) {
                int32_t cv[8];
                uint8_t cc[8];
                #pragma unroll
                for (int u = 0; u < 8; u++) { cv[u] = line[x + u * step]; cc[u] = cov[x + u * step]; }
                #pragma unroll
                for (int u = 0; u < 8; u++)
                    if (!cc[u]) top2_insert(a1, a2, pack_i32(cv[u], (uint32_t)(x + u * step)));
            }
            for (; x < len; x += step)
                if (!cov[x]) top2_insert(a1, a2, pack_i32(line[x], (uint32_t)x));
        } else {
            for (int x = first; x < len; x += step)
                if (!cov[x]) top2_insert(a1, a2, pack_i32(line[x], (uint32_t)x));
        }
    } else {
        const int j = L - I.m;
        if (kWide) {
            int i = first;
            for (; i + 3 * step < I.m; i += 4 * step) {
                int32_t cv[4];
                uint8_t cc[4];
                #pragma unroll
                for (int u = 0; u < 4; u++) { cv[u] = cost_of(I, i + u * step, j); cc[u] = c.covered[i + u * step]; }
                #pragma unroll
                for (int u = 0; u < 4; u++)
                    if (!cc[u]) top2_insert(a1, a2, pack_i32(cv[u], (uint32_t)(i + u * step)));
            }
            for (; i < I.m; i += step)
                if (!c.covered[i]) top2_insert(a1, a2, pack_i32(cost_of(I, i, j), (uint32_t)i));
        } else {
            for (int i = first; i < I.m; i += step)
                if (!c.covered[i]) top2_insert(a1, a2, pack_i32(cost_of(I, i, j), (uint32_t)i));
        }
    }
}

// one warp rebuilds the cache of line L
template <bool kWide>
__device__ void vogel_rescan_warp(const Ctx& c, int L, const int32_t* costT) {
    const int lane = threadIdx.x & 31;
    uint64_t a1, a2;
    vogel_scan<kWide>(c, L, lane, 32, costT, a1, a2);
    warp_top2(a1, a2);
    if (lane == 0) c.top2[L] = top2_from_keys(a1, a2);
}

// the whole block rebuilds the cache of line L (block-uniform call)
template <bool kWide>
__device__ void vogel_rescan_block(const Ctx& c, int L, BlockScratch& bs, const int32_t* costT) {
    uint64_t a1, a2;
    vogel_scan<kWide>(c, L, threadIdx.x, blockDim.x, costT, a1, a2);
    warp_top2(a1, a2);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) { bs.red[w] = a1; bs.red2[w] = a2; }
    __syncthreads();
    if (w == 0) {
        uint64_t b1 = l < nw ? bs.red[l] : kNoKey, b2 = l < nw ? bs.red2[l] : kNoKey;
        warp_top2(b1, b2);
        if (l == 0) c.top2[L] = top2_from_keys(b1, b2);
    }
    __syncthreads();
}

// Refresh the stored penalties of lines [lo, hi) (all rows or all columns)
// and return the largest (penalty, line) key among them.  A line whose cache
// lost a crossing is rescanned first: one warp per line when there are at
// least as many such lines as warps, else the warps split them (warp w scans
// every g-th 32-wide slice of line w mod k, g = warps / k) and warp 0 merges
// the partial top-2 pairs inside the final reduction.  That reduction also
// settles the step's choice: `best` = the larger of the half's key and
// `other` (the other half's largest key), and `stale` = whether the chosen
// line's cache must be rebuilt, decided by one thread before the last
// barrier (afterwards thread 0's allocation may change covered[]).  The
// rescan count bs.i[ctr] must be 0 on entry and is 0 again on return (rows
// and columns use different counters).  Three barriers.
template <bool kWide>
__device__ uint64_t vogel_refresh_max(const Ctx& c, int lo, int hi, int ctr, uint64_t other, uint64_t& best,
                                      int& stale, BlockScratch& bs, const int32_t* costT) {
    uint64_t mx = 0;
    if (kWide) {    // four lines' loads issued together (their latency is a global-memory round trip)
        const int bd = blockDim.x;
        for (int base = lo + threadIdx.x; base < hi; base += 4 * bd) {
            uint8_t cv[4];
            int4 t[4];
            int32_t d[4];
            #pragma unroll
            for (int u = 0; u < 4; u++) {
                const int v = base + u * bd;
                if (v < hi) { cv[u] = c.covered[v]; t[u] = c.top2[v]; d[u] = c.diff[v]; }
            }
            #pragma unroll
            for (int u = 0; u < 4; u++) {
                const int v = base + u * bd;
                if (v >= hi) continue;
                if (cv[u]) {
                    c.diff[v] = -1;
                    const uint64_t k = pack_i32(-1, (uint32_t)v);
                    mx = k > mx ? k : mx;
                } else if (!top2_valid(c, v, t[u])) {
                    c.rescan[atomicAdd(&bs.i[ctr], 1)] = v;
                } else {
                    const uint64_t k = pack_i32(d[u], (uint32_t)v);
                    mx = k > mx ? k : mx;
                }
            }
        }
    } else {
        for (int v = lo + threadIdx.x; v < hi; v += blockDim.x) {
            if (c.covered[v]) {
                c.diff[v] = -1;
                const uint64_t k = pack_i32(-1, (uint32_t)v);
                mx = k > mx ? k : mx;
                continue;
            }
            const int4 t = c.top2[v];
            if (!top2_valid(c, v, t)) { c.rescan[atomicAdd(&bs.i[ctr], 1)] = v; continue; }
            // a valid cache's penalty is the stored one: every cache rebuild
            // stores its penalty with it
            const uint64_t k = pack_i32(c.diff[v], (uint32_t)v);
            mx = k > mx ? k : mx;
        }
    }
    __syncthreads();
    const int k = bs.i[ctr];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (k >= nw) {
        for (int q = w; q < k; q += nw) {
            const int L = c.rescan[q];
            vogel_rescan_warp<kWide>(c, L, costT);
            if (l == 0) {
                const int32_t p = vogel_penalty(c.top2[L]);
                c.diff[L] = p;
                const uint64_t key = pack_i32(p, (uint32_t)L);
                mx = key > mx ? key : mx;
            }
        }
    } else if (k > 0) {
        const int g = nw / k;
        if (w < g * k) {
            const int L = c.rescan[w % k], s = w / k;
            uint64_t a1, a2;
            vogel_scan<kWide>(c, L, 32 * s + l, 32 * g, costT, a1, a2);
            warp_top2(a1, a2);
            if (l == 0) { bs.part1[w] = a1; bs.part2[w] = a2; }
        }
    }
    mx = warp_max_u64(mx);
    if (l == 0) bs.red[w] = mx;        // every read of bs.red before this refresh preceded its first barrier
    __syncthreads();
    if (w == 0) {
        uint64_t x = l < nw ? bs.red[l] : 0ull;
        if (k > 0 && k < nw && l < k) {
            const int g = nw / k;
            uint64_t a1 = kNoKey, a2 = kNoKey;
            for (int s = 0; s < g; s++) top2_merge(a1, a2, bs.part1[l + s * k], bs.part2[l + s * k]);
            const int L = c.rescan[l];
            const int4 t = top2_from_keys(a1, a2);
            c.top2[L] = t;
            const int32_t p = vogel_penalty(t);
            c.diff[L] = p;
            const uint64_t key = pack_i32(p, (uint32_t)L);
            x = key > x ? key : x;
        }
        __syncwarp();                  // the merged caches are visible to lane 0 below
        x = warp_max_u64(x);
        if (l == 0) {
            const uint64_t all = x > other ? x : other;
            const int L = (int)key_idx(all);
            bs.red[0] = x;
            bs.red2[0] = all;
            // an uncovered line of the half just refreshed has an exact cache
            // (checked or rebuilt above): the wide form reads the cache only
            // for a line of the other half or a covered one (penalty -1)
            const bool check = !kWide || other > x || key_val(all) == -1;
            bs.i[9] = check && !top2_valid(c, L, c.top2[L]) ? 1 : 0;
            bs.i[ctr] = 0;                   // every thread read it before the barrier above
        }
    }
    __syncthreads();
    best = bs.red2[0];
    stale = bs.i[9];
    return bs.red[0];
}

// Vogel's approximation.  Writes the V-1 allocations to c.bfs_* in allocation
// order and the event count to c.sc->events (-1: the reference's behaviour is
// undefined from the step written as (-1,-1,0) on).
//
// A step covers exactly one line, so only that line's half (rows or
// columns) has its penalties refreshed in the next step; the other half's
// penalties stay as stored (the reference's staleness rule), and so does
// its largest key, kept in bs.red4[0] (rows) / bs.red4[1] (columns).
// kWide: the form for instances whose line state is in global memory (the
// plain solver's setup, flock_vogel): loads batched, columns read from costT
// when given.  The staged forms (line state in shared memory) keep the
// leaner loops and their registers.
template <bool kWide = false>
__device__ void vogel_cta(const Ctx& c, BlockScratch& bs, const int32_t* costT = nullptr) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        c.covered[v] = 0;
        c.res[v] = v < m ? I.supply[v] : I.demand[v - m];
    }
    // initial caches: rows one warp per row (coalesced), columns one thread
    // per column walking down the rows (coalesced across the warp)
    const int nw = blockDim.x >> 5;
    // (each cache is stored with its penalty: a refresh reuses the penalty
    // of every line whose cache stayed valid)
    for (int i = threadIdx.x >> 5; i < m; i += nw) {
        const int32_t* row = I.cost + (size_t)i * I.ldc;
        uint64_t a1 = kNoKey, a2 = kNoKey;
        for (int j = threadIdx.x & 31; j < n; j += 32) top2_insert(a1, a2, pack_i32(row[j], (uint32_t)j));
        warp_top2(a1, a2);
        if ((threadIdx.x & 31) == 0) {
            const int4 t = top2_from_keys(a1, a2);
            c.top2[i] = t;
            c.diff[i] = vogel_penalty(t);
        }
    }
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        uint64_t a1 = kNoKey, a2 = kNoKey;
        for (int i = 0; i < m; i++) top2_insert(a1, a2, pack_i32(cost_of(I, i, j), (uint32_t)i));
        const int4 t = top2_from_keys(a1, a2);
        c.top2[m + j] = t;
        c.diff[m + j] = vogel_penalty(t);
    }
    if (threadIdx.x == 0) {
        bs.i[0] = 1; bs.i[1] = 1;   // refresh rows / columns in the next step
        bs.i[2] = 0; bs.i[3] = 0;   // covered rows / columns (counters)
        bs.i[4] = 0;                // stale min-cost index
        bs.i[5] = 0;                // events
        bs.i[6] = 0; bs.i[8] = 0;   // rescan list lengths (rows, columns)
        bs.red4[0] = 0; bs.red4[1] = 0;
        bs.i[7] = 0;                // stop
    }
    __syncthreads();
    for (int step = 0; step < V - 1; step++) {
        const int cr = bs.i[2], cc = bs.i[3];
        if (cr + cc >= V - 1 || bs.i[7]) break;
        const int pr = bs.i[0], pc = bs.i[1];
        uint64_t mrow = bs.red4[0], mcol = bs.red4[1], best = 0;
        int stale = 0;
        if (pr) mrow = vogel_refresh_max<kWide>(c, 0, m, 6, pc ? 0ull : mcol, best, stale, bs, costT);
        if (pc) mcol = vogel_refresh_max<kWide>(c, m, V, 8, mrow, best, stale, bs, costT);
        const int L = (int)key_idx(best);
        if (stale) vogel_rescan_block<kWide>(c, L, bs, costT);
        if (threadIdx.x == 0) {
            bs.red4[0] = mrow;
            bs.red4[1] = mcol;
            bs.i[0] = 0;
            bs.i[1] = 0;
            const int4 t = c.top2[L];
            // a rebuilt cache keeps its penalty with it; the stored penalty
            // only matters at the next refresh of L's half (stale until then)
            if (stale) c.diff[L] = vogel_penalty(t);
            const bool found = t.z >= 0;
            const int cross = found ? t.z : bs.i[4];
            if (!found) bs.i[5]++;
            int row, col;
            bool undefined;
            if (L >= m) { col = L - m; row = cross; undefined = row < 0 || row >= m; }
            else        { row = L; col = cross; undefined = col < 0 || col >= n; }
            const int counter = cr + cc;
            if (undefined) {
                bs.i[5] = -1;
                bs.i[7] = 1;
                for (int k = counter; k < V - 1; k++) { c.bfs_src[k] = -1; c.bfs_dst[k] = -1; c.bfs_qty[k] = 0; }
            } else {
                const int32_t rs = c.res[row], rd = c.res[m + col];
                int32_t q;
                if (rd > rs) {
                    q = rs; c.res[m + col] = rd - rs; c.res[row] = 0; c.covered[row] = 1;
                    bs.i[0] = 1; bs.i[2] = cr + 1;
                } else {
                    q = rd; c.res[row] = rs - rd; c.res[m + col] = 0; c.covered[m + col] = 1;
                    bs.i[1] = 1; bs.i[3] = cc + 1;
                }
                c.bfs_src[counter] = row; c.bfs_dst[counter] = col; c.bfs_qty[counter] = q;
                if (found) bs.i[4] = cross;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) c.sc->events = bs.i[5];
    __syncthreads();
}

// North-west corner rule (IBFS_nwc.cu:3-33), thread 0 only; caller syncs.
__device__ void nwc_thread0(const Ctx& c) {
    const InstDev& I = c.I;
    int r = 0, k = 0, cnt = 0;
    int32_t cd = I.demand[0], cs = I.supply[0];
    while (r < I.m && k < I.n && cnt < I.m + I.n - 1) {
        if (cd >= cs) {
            c.bfs_src[cnt] = r; c.bfs_dst[cnt] = k; c.bfs_qty[cnt] = cs;
            cd -= cs; r++; cs = r < I.m ? I.supply[r] : 0;
        } else {
            c.bfs_src[cnt] = r; c.bfs_dst[cnt] = k; c.bfs_qty[cnt] = cd;
            cs -= cd; k++; cd = k < I.n ? I.demand[k] : 0;
        }
        cnt++;
    }
    for (; cnt < I.m + I.n - 1; cnt++) { c.bfs_src[cnt] = -1; c.bfs_dst[cnt] = -1; c.bfs_qty[cnt] = 0; }
}

// ---------------------------------------------------------------------------
// Vogel as the reference's device variant find_vogel_bfs_parallel
// (IBFS_vogel.cu:3-543, BFS_METHOD "vam_device"): regrets from positions into
// per-line cost-sorted books; a different BFS from vogel_cta (other tie rules:
// the first largest regret, no stale penalties).

// Ascending floats -> ascending unsigned keys (no -0.0 arises from int costs).
__device__ __forceinline__ uint32_t float_order_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_from_order_bits(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Book entries per line of the other kind's count plus the two sentinels.
__host__ __device__ __forceinline__ size_t book_entries(int m, int n) {
    return (size_t)m * (n + 2) + (size_t)n * (m + 2);
}

// The book of one line (IBFS_vogel.cu:126-350): its len cells and two
// sentinels (index len and len + 1, cost 32767.0f) ordered by (float cost,
// index) -- the order the reference's two stable sorts give, equal costs in
// index order -- then the entry at position len + 1 lowered by 1.0f
// (override_row_sorts / override_col_sorts).  line < m: row `line`, else
// column line - m.  sk: P >= len + 2 shared keys (P a power of two); out:
// len + 2 entries (index, float bits of the cost).
__device__ void book_line_cta(const InstDev& I, int line, uint64_t* sk, int P, int2* out) {
    const int m = I.m;
    const bool row = line < m;
    const int len = row ? I.n : m;
    for (int k = threadIdx.x; k < P; k += blockDim.x) {
        uint64_t key = kNoKey;
        if (k < len + 2) {
            const float cf = k < len ? (float)(row ? cost_of(I, line, k) : cost_of(I, k, line - m)) : 32767.0f;
            key = ((uint64_t)float_order_bits(cf) << 32) | (uint32_t)k;
        }
        sk[k] = key;
    }
    __syncthreads();
    // bitonic sort, ascending (keys are distinct: the index is in the low word)
    for (int size = 2; size <= P; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < (P >> 1); t += blockDim.x) {
                const int lo = 2 * t - (t & (stride - 1)), hi = lo + stride;
                const uint64_t a = sk[lo], b = sk[hi];
                if ((a > b) == ((lo & size) == 0)) { sk[lo] = b; sk[hi] = a; }
            }
            __syncthreads();
        }
    for (int k = threadIdx.x; k < len + 2; k += blockDim.x) {
        const uint64_t key = sk[k];
        float cf = float_from_order_bits((uint32_t)(key >> 32));
        if (k == len + 1) cf = cf - 1.0f;
        out[k] = make_int2((int)(uint32_t)key, __float_as_int(cf));
    }
    __syncthreads();
}

// The step loop (IBFS_vogel.cu:417-537) over books built by book_line_cta
// (rbook: m rows of n + 2 entries, cbook: n columns of m + 2).  Line state in
// c.top2 (position il1, position il2, entry index, float bits of the regret;
// initially 0, 1, 0, 0.0f as the reference's vogelDifference defaults);
// residuals in c.res.  A step refreshes the lines of the kind not eliminated
// last (both at the first step, rows first: computeDifferences, :3-122),
// takes the first largest regret over [rows, columns] (thrust::max_element),
// allocates min(residuals) -- the column is eliminated on a tie -- and resets
// the eliminated line to (count of the other kind, +1, -1, -1.0f).  Writes
// m+n-1 allocations to c.bfs_*; c.sc->events = -1 where the reference would
// index past its arrays (its flows from there on are written as (-1,-1,0)).
__device__ void vogel_books_cta(const Ctx& c, const int2* rbook, const int2* cbook, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    int4* st = c.top2;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        st[v] = make_int4(0, 1, 0, 0);
        c.res[v] = v < m ? I.supply[v] : I.demand[v - m];
    }
    // bs.i[0]: last eliminated line; bs.i[1]: stop (undefined), written by
    // thread 0 only; bs.i[2]: a refresh left the book (read by thread 0)
    if (threadIdx.x == 0) { bs.i[0] = -1; bs.i[1] = 0; bs.i[2] = 0; }
    __syncthreads();
    for (int counter = 0; counter < V - 1; counter++) {
        const int prev = bs.i[0];
        for (int pass = 0; pass < (counter == 0 ? 2 : 1); pass++) {
            const int p = counter == 0 ? (pass == 0 ? V : -1) : prev;
            const bool rows = p >= m;
            const int lo = rows ? 0 : m, hi = rows ? m : V;
            const int len = rows ? n : m;        // real entries of this kind's books
            const int own = rows ? m : n;        // a line of the other kind is covered when its il1 >= own
            const int obase = rows ? m : 0;      // first line of the other kind
            const int reject = rows ? p - m : p;
            int bad = 0;
            for (int v = lo + threadIdx.x; v < hi; v += blockDim.x) {
                const int2* book = rows ? rbook + (size_t)v * (n + 2) : cbook + (size_t)(v - m) * (m + 2);
                int4 e = st[v];
                int2 l1 = book[e.x], l2 = book[e.y];
                if (l1.x == reject || l2.x == reject) {
                    if (l1.x == reject) { e.x = e.y; l1 = l2; }
                    while (e.y < len - 1) {
                        e.y++;
                        const int x = book[e.y].x;
                        if (x < 0 || x >= len) { bad = 1; break; }
                        if (st[obase + x].x < own) break;
                    }
                    l2 = book[e.y];
                }
                e.z = l1.x;
                e.w = __float_as_int(__int_as_float(l2.y) - __int_as_float(l1.y));
                st[v] = e;
            }
            if (bad) bs.i[2] = 1;
            __syncthreads();
        }
        // first largest regret: the smallest (inverted regret, line) key
        uint64_t key = kNoKey;
        for (int v = threadIdx.x; v < V; v += blockDim.x) {
            const uint64_t k2 = ((uint64_t)(~float_order_bits(__int_as_float(st[v].w))) << 32) | (uint32_t)v;
            key = k2 < key ? k2 : key;
        }
        key = block_min_u64(key, bs);
        if (threadIdx.x == 0) {
            const int L = (int)(uint32_t)key;
            const int cross = st[L].z;
            int row, col;
            if (L >= m) { col = L - m; row = cross; } else { row = L; col = cross; }
            if (bs.i[2] || row < 0 || row >= m || col < 0 || col >= n) {
                bs.i[1] = 1;
                for (int k = counter; k < V - 1; k++) { c.bfs_src[k] = -1; c.bfs_dst[k] = -1; c.bfs_qty[k] = 0; }
            } else {
                const int32_t rs = c.res[row], rd = c.res[m + col];
                int32_t q;
                if (rd > rs) {
                    q = rs; c.res[m + col] = rd - rs; c.res[row] = 0; bs.i[0] = row;
                    st[row] = make_int4(n, n + 1, -1, __float_as_int(-1.0f));
                } else {
                    q = rd; c.res[row] = rs - rd; c.res[m + col] = 0; bs.i[0] = m + col;
                    st[m + col] = make_int4(m, m + 1, -1, __float_as_int(-1.0f));
                }
                c.bfs_src[counter] = row; c.bfs_dst[counter] = col; c.bfs_qty[counter] = q;
            }
        }
        __syncthreads();
        if (bs.i[1]) break;
    }
    if (threadIdx.x == 0) c.sc->events = bs.i[1] ? -1 : 0;
    __syncthreads();
}

}  // namespace flock
