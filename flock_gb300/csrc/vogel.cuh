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

// The writes of a Vogel step that other threads may still be reading when it
// ends: the line it covered and its two residuals.  Thread 0 stores them
// after the next step's barrier; until the barrier after that makes them
// visible, every reader takes them from this copy, which every thread holds
// in registers (all threads decide each step's allocation themselves).
struct VogelPending {
    int jc1 = -1, jc2 = -1;   // lines covered by the previous step and the step before it
    int r0 = -1, r1 = -1;     // vertices whose residuals the previous step changed ...
    int32_t q0 = 0, q1 = 0;   // ... and their new values
    __device__ __forceinline__ bool covered(const Ctx& c, int v) const {
        return v == jc1 || v == jc2 || c.covered[v];
    }
    __device__ __forceinline__ int32_t res(const Ctx& c, int v) const {
        return v == r0 ? q0 : v == r1 ? q1 : c.res[v];
    }
    // thread 0, after the step's barrier: the previous step's writes
    __device__ __forceinline__ void apply(const Ctx& c) const {
        if (jc1 >= 0) c.covered[jc1] = 1;
        if (r0 >= 0) c.res[r0] = q0;
        if (r1 >= 0) c.res[r1] = q1;
    }
};

__device__ __forceinline__ bool top2_valid(const Ctx& c, int L, int4 t, const VogelPending& pd) {
    const int m = c.I.m;
    if (t.z == -2) return false;                  // never built
    if (t.z < 0) return true;                     // nothing uncovered: stays so
    if (pd.covered(c, crossing_vertex(L, t.z, m))) return false;
    if (t.w >= 0 && pd.covered(c, crossing_vertex(L, t.w, m))) return false;
    return true;
}

// This thread's share of line L's two cheapest uncovered crossing cells:
// crossing indices first, first + step, ...
__device__ __forceinline__ void vogel_scan_part(const Ctx& c, int L, int first, int step, const VogelPending& pd,
                                                uint64_t& a1, uint64_t& a2) {
    const InstDev& I = c.I;
    a1 = kNoKey; a2 = kNoKey;
    if (L < I.m) {
        const int32_t* row = I.cost + (size_t)L * I.ldc;
        for (int j = first; j < I.n; j += step)
            if (!pd.covered(c, I.m + j)) top2_insert(a1, a2, pack_i32(row[j], (uint32_t)j));
    } else {
        const int j = L - I.m;
        for (int i = first; i < I.m; i += step)
            if (!pd.covered(c, i)) top2_insert(a1, a2, pack_i32(cost_of(I, i, j), (uint32_t)i));
    }
}

// Refresh the stored penalties of lines [lo, hi) (all rows or all columns)
// and return the largest (penalty, line) key among them, in every thread.
// Thread t takes lines lo + t + k * blockDim, kVogelUnroll of them with their
// loads issued together; a line whose cache lost a crossing goes to the
// rescan list (list[], count *cnt, which is 0 on entry and again on return).
// After the first barrier the listed lines are rebuilt: one warp per line
// when there are at least as many lines as warps or the lines are short,
// else the warps split them (warp w scans every g-th 32-wide slice of line
// w mod k, g = warps / k) and every warp merges the partial top-2 pairs
// after the second barrier (warp 0 stores them, then a third barrier makes
// them visible).  Two barriers otherwise; the warp maxima go to slot[].
// Thread 0 applies the previous step's pending writes after the first
// barrier when `apply` is set.  Callers alternate two counters, so that the
// reset of one refresh's counter (after its second barrier) cannot meet the
// next refresh's additions.
constexpr int kVogelUnroll = 4;
constexpr int kVogelSplitLen = 512;   // lines of more crossings are split over warps
__device__ uint64_t vogel_refresh(const Ctx& c, int lo, int hi, int32_t* list, int* cnt, uint64_t* slot,
                                  BlockScratch& bs, const VogelPending& pd, bool apply) {
    const InstDev& I = c.I;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int bd = blockDim.x;
    uint64_t mx = 0;
    for (int base = lo + threadIdx.x; base < hi; base += kVogelUnroll * bd) {
        uint8_t cv[kVogelUnroll];
        int4 t[kVogelUnroll];
        int32_t d[kVogelUnroll];
        #pragma unroll
        for (int u = 0; u < kVogelUnroll; u++) {
            const int v = base + u * bd;
            if (v < hi) { cv[u] = c.covered[v]; t[u] = c.top2[v]; d[u] = c.diff[v]; }
        }
        #pragma unroll
        for (int u = 0; u < kVogelUnroll; u++) {
            const int v = base + u * bd;
            if (v >= hi) continue;
            if (cv[u] || v == pd.jc1 || v == pd.jc2) {
                c.diff[v] = -1;
                const uint64_t k = pack_i32(-1, (uint32_t)v);
                mx = k > mx ? k : mx;
            } else if (!top2_valid(c, v, t[u], pd)) {
                list[atomicAdd(cnt, 1)] = v;
            } else {
                // a valid cache's penalty is the stored one: every cache
                // rebuild stores its penalty with it
                const uint64_t k = pack_i32(d[u], (uint32_t)v);
                mx = k > mx ? k : mx;
            }
        }
    }
    __syncthreads();
    if (apply && threadIdx.x == 0) pd.apply(c);
    const int k = *cnt;
    const bool split = k > 0 && k < nw && (lo == 0 ? I.n : I.m) > kVogelSplitLen;   // block-uniform
    const int mine = split && lane < k ? list[lane] : -1;   // the split lines, kept past the second barrier
    if (!split) {
        for (int q = w; q < k; q += nw) {
            const int L = list[q];
            uint64_t a1, a2;
            vogel_scan_part(c, L, lane, 32, pd, a1, a2);
            warp_top2(a1, a2);
            const int4 tt = top2_from_keys(a1, a2);
            const int32_t pen = vogel_penalty(tt);
            if (lane == 0) { c.top2[L] = tt; c.diff[L] = pen; }
            const uint64_t key = pack_i32(pen, (uint32_t)L);
            mx = key > mx ? key : mx;
        }
    } else {
        const int g = nw / k;
        if (w < g * k) {
            uint64_t a1, a2;
            vogel_scan_part(c, list[w % k], 32 * (w / k) + lane, 32 * g, pd, a1, a2);
            warp_top2(a1, a2);
            if (lane == 0) { bs.part1[w] = a1; bs.part2[w] = a2; }
        }
    }
    mx = warp_max_u64(mx);
    if (lane == 0) slot[w] = mx;
    __syncthreads();
    if (threadIdx.x == 0) *cnt = 0;                    // every thread read it before the barrier above
    uint64_t x = lane < nw ? slot[lane] : 0ull;
    if (split) {
        if (lane < k) {
            const int g = nw / k;
            uint64_t a1 = kNoKey, a2 = kNoKey;
            for (int q = 0; q < g; q++) top2_merge(a1, a2, bs.part1[lane + q * k], bs.part2[lane + q * k]);
            const int4 tt = top2_from_keys(a1, a2);
            const int32_t pen = vogel_penalty(tt);
            if (w == 0) { c.top2[mine] = tt; c.diff[mine] = pen; }
            const uint64_t key = pack_i32(pen, (uint32_t)mine);
            x = key > x ? key : x;
        }
        __syncthreads();      // the rebuilt caches are visible to every reader after the refresh
    }
    return warp_max_u64(x);
}

// Vogel's approximation.  Writes the V-1 allocations to c.bfs_* in allocation
// order and the event count to c.sc->events (-1: the reference's behaviour is
// undefined from the step written as (-1,-1,0) on).
//
// A step covers exactly one line, so only that line's half (rows or
// columns) has its penalties refreshed in the next step; the other half's
// penalties stay as stored (the reference's staleness rule), and so does
// its largest key.  Every thread runs the step's decisions on the same values
// (the halves' largest keys, the chosen line's cache, the residuals), so a
// step needs only the refresh's barriers (two, three when long lines are
// rebuilt split over warps), plus one when the chosen line's cache must be
// rebuilt (a line of the stale half can have lost a crossing since its last
// refresh).
__device__ void vogel_cta(const Ctx& c, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        c.covered[v] = 0;
        c.res[v] = v < m ? I.supply[v] : I.demand[v - m];
    }
    // initial caches: rows one warp per row (coalesced), columns one thread
    // per column walking down the rows (coalesced across the warp)
    const int nw = blockDim.x >> 5, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    // (each cache is stored with its penalty: a refresh reuses the penalty
    // of every line whose cache stayed valid)
    for (int i = w; i < m; i += nw) {
        const int32_t* row = I.cost + (size_t)i * I.ldc;
        uint64_t a1 = kNoKey, a2 = kNoKey;
        for (int j = lane; j < n; j += 32) top2_insert(a1, a2, pack_i32(row[j], (uint32_t)j));
        warp_top2(a1, a2);
        if (lane == 0) {
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
    __syncthreads();
    VogelPending pd;
    bool pr = true, pc = true, stop = false;   // refresh rows / columns in this step
    int cr = 0, cc = 0;                        // covered rows / columns
    int prev = 0;                              // the reference's stale min-cost index
    int events = 0;
    uint64_t mrow = 0, mcol = 0;
    unsigned nref = 0;
    if (threadIdx.x == 0) { bs.i[0] = 0; bs.i[1] = 0; }
    __syncthreads();
    while (cr + cc < V - 1 && !stop) {
        // rows list their rescans in rescan[0, m), columns in rescan[m, V)
        if (pr) { mrow = vogel_refresh(c, 0, m, c.rescan, &bs.i[nref & 1], bs.red, bs, pd, true); nref++; }
        if (pc) { mcol = vogel_refresh(c, m, V, c.rescan + m, &bs.i[nref & 1], bs.red, bs, pd, !pr); nref++; }
        const uint64_t best = mrow > mcol ? mrow : mcol;
        const int L = (int)key_idx(best);
        int4 t = c.top2[L];
        const bool stale = !top2_valid(c, L, t, pd);
        if (stale) {      // block-uniform: the whole block rebuilds L's cache
            uint64_t a1, a2;
            vogel_scan_part(c, L, threadIdx.x, blockDim.x, pd, a1, a2);
            warp_top2(a1, a2);
            if (lane == 0) { bs.red3[w] = a1; bs.red4[w] = a2; }
            __syncthreads();
            uint64_t b1 = lane < nw ? bs.red3[lane] : kNoKey, b2 = lane < nw ? bs.red4[lane] : kNoKey;
            warp_top2(b1, b2);
            t = top2_from_keys(b1, b2);
        }
        const bool found = t.z >= 0;
        const int cross = found ? t.z : prev;
        if (!found) events++;
        int row, col;
        bool undefined;
        if (L >= m) { col = L - m; row = cross; undefined = row < 0 || row >= m; }
        else        { row = L; col = cross; undefined = col < 0 || col >= n; }
        const int counter = cr + cc;
        if (undefined) {
            events = -1;
            stop = true;
            if (threadIdx.x == 0)
                for (int k = counter; k < V - 1; k++) { c.bfs_src[k] = -1; c.bfs_dst[k] = -1; c.bfs_qty[k] = 0; }
            break;
        }
        const int32_t rs = pd.res(c, row), rd = pd.res(c, m + col);
        int32_t q, nrs, nrd;
        int cov;
        if (rd > rs) { q = rs; nrs = 0; nrd = rd - rs; cov = row; }
        else         { q = rd; nrs = rs - rd; nrd = 0; cov = m + col; }
        if (threadIdx.x == 0) {
            c.bfs_src[counter] = row; c.bfs_dst[counter] = col; c.bfs_qty[counter] = q;
            // a rebuilt cache keeps its penalty with it; the stored penalty
            // only matters at the next refresh of L's half (stale until
            // then; no thread reads L's cache before the next barrier: the
            // next step refreshes the other half)
            if (stale && cov != L) { c.top2[L] = t; c.diff[L] = vogel_penalty(t); }
        }
        pr = cov < m;
        pc = !pr;
        if (pr) cr++; else cc++;
        if (found) prev = cross;
        pd.jc2 = pd.jc1; pd.jc1 = cov;
        pd.r0 = row; pd.q0 = nrs; pd.r1 = m + col; pd.q1 = nrd;
    }
    __syncthreads();      // every read of this step's state is done
    if (threadIdx.x == 0) {
        pd.apply(c);
        c.sc->events = events;
    }
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
