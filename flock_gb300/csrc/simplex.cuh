// simplex.cuh -- exact int64 transportation simplex on a rooted basis tree.
//
// Reference path being replaced: the u-v method of uvModel_parallel::execute
// (src/parallel_simplex_method/parallel_uv_method/uv_model_parallel.cu:227-395)
// and the parallel stepping-stone round of SS_METHOD::perform_a_parallel_pivot
// (src/parallel_simplex_method/parallel_ss_method/PIVOT_ss.cu:294-454).
//
// Design (all integer, no floating point):
//  * The tree is rooted at a column rho and stored as parent[], depth[] and
//    flow[] (flow on the edge to the parent).  Duals pot[] satisfy
//    u_i + v_j = c_ij on tree edges with v_rho = 0.
//  * Anti-cycling: pivoting runs on the perturbed right-hand side
//    s'_i = M s_i + 1, d'_j = M d_j - 1 (j != rho), d'_rho = M d_rho + V'-1,
//    M = 2V'+1.  Every basis of this problem is nondegenerate, so each pivot
//    strictly lowers the perturbed objective and no basis repeats (this is
//    Cunningham's strongly feasible tree rule in exact arithmetic).  The
//    original flows are recovered as round(flow / M) at the end.
//  * The start tree keeps every positive flow of the initial solution (Vogel
//    or NW corner) and re-chooses the zero-flow basic cells so that the tree
//    is strongly feasible (each non-root column has a positive edge to its
//    parent).  Zero-demand columns can carry no flow and are kept out of the
//    pivoting tree; they are attached at the end with v_j = min_i c_ij - u_i.
//  * A round: duals by pointer jumping (O(log depth) steps), a sweep that keeps
//    the best reduced cost per row, then every negative row-best candidate
//    walks its cycle with parent/depth LCA steps, claims its edges with
//    atomicMin on a (reduced cost, row) priority, and the candidates that own
//    all their edges (an edge-disjoint set, always containing the best one)
//    are applied together.  Edge-disjoint pivots commute, so the round equals
//    applying them one after another.  Sequential mode applies only the best
//    candidate (Dantzig's rule with the reference's row-major first-minimum
//    tie-break, uv_model_parallel.cu:178-200).
#pragma once
#include "vogel.cuh"

namespace flock {

__device__ __forceinline__ int32_t block_exclusive_scan_i32(int32_t* a, int n, BlockScratch& bs) {
    // in-place exclusive scan of a[0..n), returns the total
    const int T = blockDim.x;
    const int chunk = (n + T - 1) / T;
    const int lo = threadIdx.x * chunk, hi = min(n, lo + chunk);
    int32_t s = 0;
    for (int k = lo; k < hi; k++) s += a[k];
    // warp inclusive scan of per-thread sums
    int32_t x = s;
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5, nw = T >> 5;
    #pragma unroll
    for (int o = 1; o < 32; o <<= 1) { int32_t y = __shfl_up_sync(0xffffffffu, x, o); if (l >= o) x += y; }
    __syncthreads();
    if (l == 31) bs.red[w] = (uint64_t)(int64_t)x;
    __syncthreads();
    if (w == 0) {
        int32_t t = l < nw ? (int32_t)(int64_t)bs.red[l] : 0;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) { int32_t y = __shfl_up_sync(0xffffffffu, t, o); if (l >= o) t += y; }
        bs.red2[l] = (uint64_t)(int64_t)t;
    }
    __syncthreads();
    int32_t base = (w > 0 ? (int32_t)(int64_t)bs.red2[w - 1] : 0) + x - s;
    for (int k = lo; k < hi; k++) { int32_t v = a[k]; a[k] = base; base += v; }
    const int32_t total = (int32_t)(int64_t)bs.red2[nw - 1];
    __syncthreads();
    return total;
}

__device__ __forceinline__ int uf_find(int32_t* uf, int x) {
    while (uf[x] != x) { uf[x] = uf[uf[x]]; x = uf[x]; }
    return x;
}

// ------------------------------------------------------------ start tree ---
// Warp 0 (all its lanes) extends the tree from the queued vertices
// order[qh, qt): level by level, each lane takes one queued vertex and claims
// its positive-cell neighbours that no vertex has claimed yet (parent -2 ->
// the vertex, by compare-and-swap), appending them to the queue; every
// parent precedes its children in the queue.  On a forest each vertex is
// claimed once; a second path to a vertex (a cycle among the positive cells)
// shows as fewer claims than positive cells, which the caller checks.
// Returns the new tail; *claims (lane 0) grows by the claims made.
__device__ __forceinline__ int warp_extend(const Ctx& c, int qh, int qt, int* s_tail, int* claims) {
    const int V = c.I.m + c.I.n;
    const int lane = threadIdx.x & 31;
    int mine = 0;
    while (qh < qt) {                                 // warp-uniform
        const int end = qt;
        if (lane == 0) *s_tail = end;
        __syncwarp();
        for (int b0 = qh; b0 < end; b0 += 32) {
            const int idx = b0 + lane;
            if (idx >= end) continue;
            const int p = c.order[idx];
            if (!FLOCK_IN(p, V)) { fail_check(c.sc, 31); continue; }
            const int dp = c.depth[p];
            const int e1 = c.csr_start[p + 1];
            for (int e = c.csr_start[p]; e < e1; e++) {
                const int ch = c.csr_adj[e];
                if (!FLOCK_IN(ch, V)) { fail_check(c.sc, 31); break; }
                if (atomicCAS(&c.parent[ch], -2, p) != -2) continue;
                c.depth[ch] = dp + 1;
                const int slot = atomicAdd(s_tail, 1);
                if (slot >= V) { fail_check(c.sc, 34); break; }
                c.order[slot] = ch;
                mine++;
            }
        }
        __syncwarp();
        qh = end;
        qt = min(*s_tail, V);
        __syncwarp();                                 // every lane read the tail before lane 0 resets it
    }
    mine = (int)__reduce_add_sync(0xffffffffu, (unsigned)mine);
    if (lane == 0) *claims += mine;
    return qt;
}

// Builds the strongly feasible start tree from the allocation list c.bfs_*.
// If the list is not a feasible solution whose positive cells form a forest
// (the reference's undefined Vogel case), the NW-corner solution is used:
// a list that does not balance the supplies and demands is replaced before
// the tree is built; a cycle among the positive cells shows after the
// traversal (fewer claims than positive cells) and the build restarts from
// the NW-corner list.
__device__ void sf_init_cta(const Ctx& c, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int v = threadIdx.x; v < V; v += blockDim.x) c.bsum[v] = 0;
    if (threadIdx.x == 0) bs.i[0] = 0;
    __syncthreads();
    for (int k = threadIdx.x; k < V - 1; k += blockDim.x) {
        const int a = c.bfs_src[k], b = c.bfs_dst[k], q = c.bfs_qty[k];
        if (a < 0 || a >= m || b < 0 || b >= n || q < 0) { bs.i[0] = 1; continue; }
        atomicAdd((unsigned long long*)&c.bsum[a], (unsigned long long)(int64_t)q);
        atomicAdd((unsigned long long*)&c.bsum[m + b], (unsigned long long)(int64_t)q);
    }
    __syncthreads();
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int64_t want = v < m ? I.supply[v] : I.demand[v - m];
        if (c.bsum[v] != want) bs.i[0] = 1;
    }
    __syncthreads();
    if (bs.i[0]) {
        if (threadIdx.x == 0) { nwc_thread0(c); c.sc->status |= ST_START_REPAIRED; }
        __syncthreads();
    }

    // root: the column with the largest demand (lowest index on ties)
    uint64_t rk = 0;
    int32_t alive_cols = 0;
    int64_t S = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const uint32_t dj = (uint32_t)I.demand[j];
        uint64_t k = ((uint64_t)dj << 32) | (uint64_t)(0xffffffffu - (uint32_t)j);
        rk = k > rk ? k : rk;
        alive_cols += I.demand[j] > 0;
    }
    for (int i = threadIdx.x; i < m; i += blockDim.x) S += I.supply[i];
    rk = block_max_u64(rk, bs);
    const int root = m + (int)(0xffffffffu - (uint32_t)rk);
    const int64_t nalive = block_sum_i64(alive_cols, bs) + (I.demand[root - m] == 0 ? 1 : 0);
    S = block_sum_i64(S, bs);
    const int v_alive = m + (int)nalive;
    const int64_t M = 2 * (int64_t)v_alive + 1;
    if (threadIdx.x == 0) {
        c.sc->root = root;
        c.sc->v_alive = v_alive;
        c.sc->M = M;
        if (M > ((int64_t)1 << 62) / (S + 2)) c.sc->status |= ST_RANGE;
    }

    for (int attempt = 0; attempt < 2; attempt++) {
        // CSR of positive cells (order[] holds degrees, then cursors)
        for (int v = threadIdx.x; v < V; v += blockDim.x) c.order[v] = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < V - 1; k += blockDim.x) {
            if (c.bfs_qty[k] <= 0 || c.bfs_src[k] < 0) continue;
            atomicAdd(&c.order[c.bfs_src[k]], 1);
            atomicAdd(&c.order[m + c.bfs_dst[k]], 1);
        }
        __syncthreads();
        for (int v = threadIdx.x; v < V; v += blockDim.x) c.csr_start[v] = c.order[v];
        __syncthreads();
        const int32_t tot = block_exclusive_scan_i32(c.csr_start, V, bs);
        if (threadIdx.x == 0) c.csr_start[V] = tot;
        for (int v = threadIdx.x; v < V; v += blockDim.x) c.order[v] = c.csr_start[v];
        __syncthreads();
        for (int k = threadIdx.x; k < V - 1; k += blockDim.x) {
            if (c.bfs_qty[k] <= 0 || c.bfs_src[k] < 0) continue;
            const int a = c.bfs_src[k], b = m + c.bfs_dst[k];
            c.csr_adj[atomicAdd(&c.order[a], 1)] = b;
            c.csr_adj[atomicAdd(&c.order[b], 1)] = a;
        }
        for (int v = threadIdx.x; v < V; v += blockDim.x) { c.parent[v] = -2; c.depth[v] = 0; }
        __syncthreads();

        // components of the positive cells, attached to the tree built so far
        if (warp == 0) {
            if (lane == 0) {
                c.parent[root] = -1;
                c.depth[root] = 0;
                c.order[0] = root;
                bs.i[1] = 0;   // scan pointer
                bs.i[6] = 0;   // claims
            }
            __syncwarp();
            const int qt = warp_extend(c, 0, 1, &bs.i[5], &bs.i[6]);
            if (lane == 0) bs.i[2] = qt;   // queue tail
        }
        __syncthreads();
        for (int guard = 0; guard <= V; guard++) {
            if (threadIdx.x == 0) {
                int w = bs.i[1];
                while (w < V && (c.parent[w] != -2 || w == root || (w >= m && I.demand[w - m] == 0))) w++;
                bs.i[1] = w;
                int rc = -1;
                if (w < V) {
                    if (w < m) rc = w;
                    else {
                        for (int e = c.csr_start[w]; e < c.csr_start[w + 1]; e++) {
                            const int x = c.csr_adj[e];
                            if (x < m && (rc < 0 || x < rc)) rc = x;
                        }
                    }
                }
                bs.i[3] = rc;
            }
            __syncthreads();
            const int rc = bs.i[3];
            if (rc < 0) break;
            uint64_t best = kNoKey;
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                if (c.parent[m + j] != -2) {
                    const uint64_t k = pack_i32(cost_of(I, rc, j), (uint32_t)j);
                    best = k < best ? k : best;
                }
            best = block_min_u64(best, bs);
            const bool ok = !(best == kNoKey || !FLOCK_IN(rc, m) || bs.i[2] >= V);   // block-uniform
            if (threadIdx.x == 0 && !ok) fail_check(c.sc, 33);
            if (ok && warp == 0) {
                const int qt0 = bs.i[2];
                if (lane == 0) {
                    const int js = m + (int)key_idx(best);
                    c.parent[rc] = js;
                    c.depth[rc] = c.depth[js] + 1;
                    c.order[qt0] = rc;
                }
                __syncwarp();
                const int qt = warp_extend(c, qt0, qt0 + 1, &bs.i[5], &bs.i[6]);
                if (lane == 0) bs.i[2] = qt;
            }
            __syncthreads();
            if (!ok) break;
        }
        // a forest has as many claims (vertices reached through positive
        // cells) as positive cells; more cells means a cycle among them
        const bool cycle = bs.i[6] != tot / 2;       // block-uniform: read after the barrier above
        __syncthreads();
        if (!cycle || attempt == 1) break;
        if (threadIdx.x == 0) { nwc_thread0(c); c.sc->status |= ST_START_REPAIRED; }
        __syncthreads();
    }

    // perturbed flows, children before parents (reverse BFS order)
    const int qt = bs.i[2];
    for (int q = threadIdx.x; q < qt; q += blockDim.x) {
        const int v = c.order[q];
        int64_t b;
        if (v < m) b = M * I.supply[v] + 1;
        else if (v != root) b = -(M * I.demand[v - m] - 1);
        else b = -(M * I.demand[v - m] + (v_alive - 1));
        c.bsum[v] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (qt != v_alive) c.sc->status |= ST_SF_FAIL;
        for (int q = qt - 1; q >= 1; q--) {
            const int v = c.order[q];
            const int p = c.parent[v];
            const int64_t f = v < m ? c.bsum[v] : -c.bsum[v];
            c.flow[v] = f;
            if (f <= 0) c.sc->status |= ST_SF_FAIL;
            c.bsum[p] += c.bsum[v];
        }
        c.flow[root] = 0;
        if (c.sc->status & (ST_SF_FAIL | ST_RANGE)) c.sc->done = 1;
    }
    __syncthreads();
}

// --------------------------------------------------------------- duals ------
// depth[] and pot[] from parent[] by pointer jumping: pot[v] = acc + (-1)^len pot[anc].
// Also the int32 column duals and the count of those outside the window.
template <int J = kJump>
__device__ void tree_recompute_cta(const Ctx& c, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int V = I.m + I.n;
    const int root = c.sc->root;
    int32_t* aA = c.anc0;
    int32_t* aB = c.anc1;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int p = c.parent[v];
        if (p == -2) { aA[v] = -2; c.len0[v] = 0; c.acc0[v] = kDeadPot; }
        else if (v == root) { aA[v] = v; c.len0[v] = 0; c.acc0[v] = 0; }
        else if (!FLOCK_IN(p, V) || (p < I.m) == (v < I.m)) { fail_check(c.sc, 20); aA[v] = root; c.len0[v] = 0; c.acc0[v] = 0; }
        else { aA[v] = p; c.len0[v] = 1; c.acc0[v] = edge_cost(I, v, p); }
    }
    int32_t* lA = c.len0; int32_t* lB = c.len1;
    int64_t* xA = c.acc0; int64_t* xB = c.acc1;
    int pending = 1;
    __syncthreads();
    for (int it = 0; it < 40 && pending; it++) {
        int mine = 0;
        // J vertices per thread per step with their loads interleaved
        // (a thread's vertices are independent chains): when V exceeds the
        // block, one dependent-load latency covers all of them.
        for (int base = threadIdx.x; base < V; base += J * blockDim.x) {
            int vv[J], a[J], kind[J], aa[J], la[J], lb[J];
            int64_t xa[J], xb[J];
            #pragma unroll
            for (int u = 0; u < J; u++) {
                vv[u] = base + u * blockDim.x;
                a[u] = vv[u] < V ? aA[vv[u]] : 0;
            }
            #pragma unroll
            for (int u = 0; u < J; u++) {
                const int v = vv[u], x = a[u];
                // 0: no vertex, 1: at the root or dead, 2: bad ancestor, 3: jump
                kind[u] = v >= V ? 0 : (x < 0 || x == root) ? 1 : !FLOCK_IN(x, V) ? 2 : 3;
                la[u] = kind[u] == 1 || kind[u] == 3 ? lA[v] : 0;
                xa[u] = kind[u] == 1 || kind[u] == 3 ? xA[v] : 0;
                aa[u] = kind[u] == 3 ? aA[x] : 0;
                lb[u] = kind[u] == 3 ? lA[x] : 0;
                xb[u] = kind[u] == 3 ? xA[x] : 0;
            }
            #pragma unroll
            for (int u = 0; u < J; u++) {
                const int v = vv[u];
                if (kind[u] == 1) { aB[v] = a[u]; lB[v] = la[u]; xB[v] = xa[u]; }
                else if (kind[u] == 2 || (kind[u] == 3 && !FLOCK_IN(aa[u], V))) {
                    fail_check(c.sc, kind[u] == 2 ? 21 : 22);
                    aB[v] = root; lB[v] = 0; xB[v] = 0;
                } else if (kind[u] == 3) {
                    aB[v] = aa[u];
                    lB[v] = la[u] + lb[u];
                    xB[v] = xa[u] + ((la[u] & 1) ? -xb[u] : xb[u]);
                    mine |= (aa[u] != root);
                }
            }
        }
        pending = __syncthreads_or(mine);
        int32_t* t1 = aA; aA = aB; aB = t1;
        int32_t* t2 = lA; lA = lB; lB = t2;
        int64_t* t3 = xA; xA = xB; xB = t3;
    }
    int64_t wide = 0;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int64_t p = xA[v];
        c.depth[v] = lA[v];
        c.pot[v] = p;
        if (v >= I.m) { int w = 0; c.v32[v - I.m] = narrow_dual(p, w); wide += w; }
    }
    wide = block_sum_i64(wide, bs);
    if (threadIdx.x == 0) {
        c.sc->nwide = (int32_t)wide;
        c.sc->narrow = wide == 0;
        if (pending) { c.sc->status |= ST_TREE_CORRUPT; c.sc->done = 1; }
    }
    __syncthreads();
}

// Preorder intervals of the tree from parent[] (into the first half of iv,
// sc->ivp = 0).  Euler tour: for each non-root tree vertex v the arc 2v
// enters v from its parent and the arc 2v+1 leaves it; after entering v the
// tour takes v's first child (or leaves v), after leaving v it enters v's
// next sibling (or leaves the parent; the root's last child ends the tour).
// Pointer jumping gives each arc the number of entering arcs from it to the
// end of the tour, S(a); with T = S(first arc) = tree vertices - 1:
//   pre(v) = T - S(2v) + 1,   size(v) = S(2v) - S(2v+1),   root: (0, T + 1).
// Children lists (first child / next sibling) live in claim[]; the two arc
// buffers in the pointer-jumping scratch.  Sibling order does not matter:
// any preorder gives the same ancestor relation.
template <int J = kJump>
__device__ void euler_intervals_cta(const Ctx& c, BlockScratch& bs) {
    const int V = c.I.m + c.I.n;
    const int root = c.sc->root;
    int32_t* fc = (int32_t*)c.claim;          // first child
    int32_t* ns = fc + V;                      // next sibling
    for (int v = threadIdx.x; v < V; v += blockDim.x) fc[v] = -1;
    __syncthreads();
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int p = c.parent[v];
        if (FLOCK_IN(p, V)) ns[v] = atomicExch(&fc[p], v);
    }
    __syncthreads();
    // arc word: (successor arc + 1) << 32 | entering arcs counted so far (0: end)
    uint64_t* X = (uint64_t*)c.anc0;
    uint64_t* Y = (uint64_t*)c.acc0;
    const int A = 2 * V;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int p = c.parent[v];
        uint64_t d = 0, u = 0;
        if (FLOCK_IN(p, V)) {
            const int f = fc[v], sb = ns[v];
            const int sd = f >= 0 ? 2 * f : 2 * v + 1;
            const int su = sb >= 0 ? 2 * sb : (p == root ? -1 : 2 * p + 1);
            d = ((uint64_t)(uint32_t)(sd + 1) << 32) | 1u;
            u = (uint64_t)(uint32_t)(su + 1) << 32;
        }
        X[2 * v] = d;
        X[2 * v + 1] = u;
    }
    int pending = 1;
    __syncthreads();
    for (int it = 0; it < 40 && pending; it++) {
        int mine = 0, bad = 0;
        for (int base = threadIdx.x; base < A; base += J * blockDim.x) {
            uint64_t x[J], y[J];
            int sa[J];
            #pragma unroll
            for (int u = 0; u < J; u++) {
                const int a = base + u * blockDim.x;
                x[u] = a < A ? X[a] : 0;
                sa[u] = (int)(x[u] >> 32) - 1;
                if (sa[u] >= A) { bad = 1; sa[u] = -1; }
            }
            #pragma unroll
            for (int u = 0; u < J; u++) y[u] = sa[u] >= 0 ? X[sa[u]] : 0;
            #pragma unroll
            for (int u = 0; u < J; u++) {
                const int a = base + u * blockDim.x;
                if (a >= A) continue;
                if (sa[u] < 0) { Y[a] = x[u] & 0xffffffffull; continue; }
                Y[a] = (y[u] & 0xffffffff00000000ull) | (uint32_t)((uint32_t)x[u] + (uint32_t)y[u]);
                mine |= (y[u] >> 32) != 0;
            }
        }
        if (bad) fail_check(c.sc, 23);
        pending = __syncthreads_or(mine);
        uint64_t* t = X; X = Y; Y = t;
    }
    const int f0 = fc[root];
    const int T = FLOCK_IN(f0, V) ? (int)(uint32_t)X[2 * f0] : 0;
    int2* iv = c.iv;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int p = c.parent[v];
        int2 w = make_int2(0, 0);
        if (v == root) w = make_int2(0, T + 1);
        else if (FLOCK_IN(p, V)) {
            const int sd = (int)(uint32_t)X[2 * v], su = (int)(uint32_t)X[2 * v + 1];
            w = make_int2(T - sd + 1, sd - su);
        }
        iv[v] = w;
    }
    if (threadIdx.x == 0) {
        c.sc->ivp = 0;
        if (pending || T + 1 != c.sc->v_alive) fail_check(c.sc, 23);
    }
    __syncthreads();
}

// Full rebuild of the tree's derived state from parent[] and flow[]:
// depths, duals, int32 duals, preorder intervals.
template <int J = kJump>
__device__ void tree_build_cta(const Ctx& c, BlockScratch& bs) {
    tree_recompute_cta<J>(c, bs);
    if (c.sc->done) return;
    euler_intervals_cta<J>(c, bs);
    if (threadIdx.x == 0) c.sc->stale = 0;
    __syncthreads();
}

// ---------------------------------------------------------------- sweep -----
// Row best key with per-element int64 reduced costs over columns [j0, j1):
// min over j of (clamp32(c_ij - u_i - v_j), j).  One warp, all lanes return it.
// (row: the row's costs, vp: the column duals.)  Plain arguments keep the
// rarely taken call from forcing the caller's context into local memory.
__device__ __noinline__ uint64_t row_best_exact(const int32_t* row, int64_t u, const int64_t* vp, int j0, int j1) {
    uint64_t best = kNoKey;
    for (int j = j0 + (int)(threadIdx.x & 31); j < j1; j += 32) {
        const int64_t r = (int64_t)row[j] - u - vp[j];
        const uint64_t k = pack_i32(clamp32(r), (uint32_t)j);
        best = k < best ? k : best;
    }
    return warp_min_u64(best);
}

// Narrow form: t = c_ij - v_j in int32 (exact while sc->narrow), running
// minimum with the first column among equal values.
__device__ __forceinline__ void min4(int32_t& bv, int32_t& bj, const int4 cv, const int4 vv, int j) {
    int32_t t;
    t = cv.x - vv.x; if (t < bv) { bv = t; bj = j; }
    t = cv.y - vv.y; if (t < bv) { bv = t; bj = j + 1; }
    t = cv.z - vv.z; if (t < bv) { bv = t; bj = j + 2; }
    t = cv.w - vv.w; if (t < bv) { bv = t; bj = j + 3; }
}

// Eight 16-bit costs (one 16-byte vector) against their eight int32 duals.
__device__ __forceinline__ void min8(int32_t& bv, int32_t& bj, const int4 cv, const int4 va, const int4 vb, int j) {
    const uint32_t w[4] = {(uint32_t)cv.x, (uint32_t)cv.y, (uint32_t)cv.z, (uint32_t)cv.w};
    const int32_t v[8] = {va.x, va.y, va.z, va.w, vb.x, vb.y, vb.z, vb.w};
    #pragma unroll
    for (int k = 0; k < 8; k++) {
        const int32_t c = (int32_t)(int16_t)(uint16_t)(w[k >> 1] >> (16 * (k & 1)));
        const int32_t t = c - v[k];
        if (t < bv) { bv = t; bj = j + k; }
    }
}

// Turn the warp's narrow minimum over columns [j0, j1) of row i into the
// row key.  The key equals row_best_exact's unless the winning column is a
// zero-demand one or the reduced cost is below INT32_MIN; those rows are
// recomputed exactly (all lanes agree on the branch).
__device__ __forceinline__ uint64_t narrow_row_key(const Ctx& c, int i, int j0, int j1, int32_t bv, int32_t bj) {
    const uint64_t kk = warp_min_u64(pack_i32(bv, (uint32_t)bj));
    const int jw = (int)key_idx(kk);
    const int64_t r = (int64_t)key_val(kk) - c.pot[i];
    if (c.v32[jw] == kDead32 || r < INT32_MIN)
        return row_best_exact(c.I.cost + (size_t)i * c.I.ldc, c.pot[i], c.pot + c.I.m, j0, j1);
    return pack_i32(clamp32(r), (uint32_t)jw);
}

// CTA-local sweep of the rows list[0..cnt) (all rows 0..cnt-1 when list is
// null): best (reduced cost, column) of each into row_best[].  Rows are
// int4-vectorised (row pitch a multiple of 4, 16-byte aligned); a warp takes
// two rows per pass for more loads in flight.  A listed row outside the
// instance is an internal error (recorded, skipped).
__device__ void sweep_rows_cta(const Ctx& c, const int32_t* list, int cnt) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n;
    const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) c.sc->cells += (int64_t)cnt * n;
    if (!c.sc->narrow) {
        for (int t = threadIdx.x >> 5; t < cnt; t += nw) {
            const int i = list ? list[t] : t;
            if (!FLOCK_IN(i, m)) { if (lane == 0) fail_check(c.sc, 19); continue; }
            const uint64_t k = row_best_exact(I.cost + (size_t)i * I.ldc, c.pot[i], c.pot + m, 0, n);
            if (lane == 0) c.row_best[i] = k;
        }
        __syncthreads();
        return;
    }
    const int4* v4 = reinterpret_cast<const int4*>(c.v32);
    const int nfull = n >> 2, tail = n & 3;
    for (int t = threadIdx.x >> 5; t < cnt; t += 2 * nw) {
        const int t2 = t + nw;
        const int i = list ? list[t] : t;
        int i2 = t2 < cnt ? (list ? list[t2] : t2) : i;
        if (!FLOCK_IN(i, m) || !FLOCK_IN(i2, m)) { if (lane == 0) fail_check(c.sc, 19); continue; }
        const bool two = t2 < cnt;
        const int4* ra = reinterpret_cast<const int4*>(I.cost + (size_t)i * I.ldc);
        const int4* rb = reinterpret_cast<const int4*>(I.cost + (size_t)i2 * I.ldc);
        int32_t av = INT32_MAX, aj = INT32_MAX, bv = INT32_MAX, bj = INT32_MAX;
        int q = lane;
        for (; q + 32 < nfull; q += 64) {
            const int4 a0 = ra[q], a1 = ra[q + 32], b0 = rb[q], b1 = rb[q + 32];
            const int4 w0 = v4[q], w1 = v4[q + 32];
            min4(av, aj, a0, w0, 4 * q);
            min4(av, aj, a1, w1, 4 * (q + 32));
            min4(bv, bj, b0, w0, 4 * q);
            min4(bv, bj, b1, w1, 4 * (q + 32));
        }
        if (q < nfull) {
            const int4 a0 = ra[q], b0 = rb[q], w0 = v4[q];
            min4(av, aj, a0, w0, 4 * q);
            min4(bv, bj, b0, w0, 4 * q);
        }
        if (lane < tail) {
            const int j = 4 * nfull + lane;
            const int32_t vj = c.v32[j];
            const int32_t ta = I.cost[(size_t)i * I.ldc + j] - vj;
            if (ta < av) { av = ta; aj = j; }
            if (two) {
                const int32_t tb = I.cost[(size_t)i2 * I.ldc + j] - vj;
                if (tb < bv) { bv = tb; bj = j; }
            }
        }
        const uint64_t ka = narrow_row_key(c, i, 0, n, av, aj);
        if (lane == 0) c.row_best[i] = ka;
        if (two) {      // warp-uniform
            const uint64_t kb = narrow_row_key(c, i2, 0, n, bv, bj);
            if (lane == 0) c.row_best[i2] = kb;
        }
    }
    __syncthreads();
}

__device__ void sweep_cta(const Ctx& c) { sweep_rows_cta(c, nullptr, c.I.m); }

// After a full sweep: keep the sc->pp_rows rows with the most negative keys in
// prow[] (32-bin histogram threshold, then row order: value-determined),
// optionally clearing every other row's key; resets the partial-pricing age.
// Returns the smallest (reduced cost, row) pair among the kept rows (kNoKey:
// none), i.e. the sequential rule's entering row over the keys that remain:
// when the first histogram bin alone holds more than pp_rows rows, the rows
// past pp_rows in row order are dropped, possibly the overall best one.  All
// threads of the block; uses cand[] as scratch.
__device__ uint64_t select_candidate_rows(const Ctx& c, BlockScratch& bs, bool clear_others) {
    const int m = c.I.m;
    const int cap = min(max(c.sc->pp_rows, 1), kPPRows);
    int32_t rmin = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) rmin = min(rmin, key_val(c.row_best[i]));
    rmin = key_val(block_min_u64(pack_i32(rmin, 0u), bs));
    const int64_t span = rmin < 0 ? -(int64_t)rmin : 1;
    int last = -1;                                             // highest histogram bin kept
    if (rmin < 0) {
        if (threadIdx.x < 32) bs.red2[threadIdx.x] = 0;
        __syncthreads();
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const int32_t v = key_val(c.row_best[i]);
            if (v < 0) atomicAdd((unsigned long long*)&bs.red2[((int64_t)v - rmin) * 32 / span], 1ull);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t cum = bs.red2[0];
            int l = 0;
            for (int b = 1; b < 32 && cum + bs.red2[b] <= (uint64_t)cap; b++) { cum += bs.red2[b]; l = b; }
            bs.i[1] = l;
        }
        __syncthreads();
        last = bs.i[1];
    }
    // candidates in row order: exclusive scan of the selection flags
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int32_t v = key_val(c.row_best[i]);
        c.cand[i] = (v < 0 && ((int64_t)v - rmin) * 32 / span <= last) ? 1 : 0;
    }
    __syncthreads();
    const int32_t total = block_exclusive_scan_i32(c.cand, m, bs);   // ends with a barrier
    uint64_t bestp = kNoKey;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        const int32_t v = key_val(c.row_best[i]);
        const bool sel = v < 0 && ((int64_t)v - rmin) * 32 / span <= last;
        const int slot = c.cand[i];
        if (sel && slot < cap) {
            c.prow[slot] = i;
            const uint64_t P = pack_i32(v, (uint32_t)i);
            bestp = P < bestp ? P : bestp;
        } else if (clear_others) {
            c.row_best[i] = kNoKey;
        }
    }
    if (threadIdx.x == 0) { c.sc->pp_n = min(total, cap); c.sc->pp_age = 0; }
    return block_min_u64(bestp, bs);                           // its barriers order the writes above
}

// Partial pricing (candidate rows).  A full sweep keeps the pp_rows rows
// with the most negative best reduced costs in prow[] (chosen by a 32-bin
// histogram threshold and then by row index, so the set depends only on the
// values) and clears every other row's key; the next rounds re-price only
// those rows.  Every reader of the keys in a partial-pricing round looks at
// the listed rows only (row_best need not survive between rounds: the round
// form stages it afresh in every launch).  A full sweep runs again when the
// candidates hold no negative reduced cost any more or after pp_refresh
// rounds, so a round without a negative key (optimality) is always a full
// sweep.  Returns the smallest (reduced cost, row) pair among the negative
// keys (kNoKey: none): the sequential rule's entering row, already reduced
// over the block.  The caller's end-of-round barrier orders pp_age.
__device__ uint64_t sweep_partial_cta(const Ctx& c, BlockScratch& bs) {
    const int m = c.I.m;
    const int pn = c.sc->pp_n, age = c.sc->pp_age;
    const bool full = pn <= 0 || pn > kPPRows || age >= max(c.sc->pp_refresh, 1);
    uint64_t best = kNoKey;
    if (!full) {
        sweep_rows_cta(c, c.prow, pn);
        for (int t = threadIdx.x; t < pn; t += blockDim.x) {
            const int i = c.prow[t];
            if (!FLOCK_IN(i, m)) continue;                     // recorded by the sweep
            const int32_t v = key_val(c.row_best[i]);
            if (v < 0) { const uint64_t P = pack_i32(v, (uint32_t)i); best = P < best ? P : best; }
        }
        best = block_min_u64(best, bs);
    }
    if (full || best == kNoKey) {
        sweep_rows_cta(c, nullptr, m);
        best = select_candidate_rows(c, bs, true);
    }
    if (threadIdx.x == 0) c.sc->pp_age++;
    return best;
}

// ---------------------------------------------------------------- pivots ----
struct CycleResult {
    int64_t theta;
    int32_t q;        // leaving edge (child vertex)
    int32_t lside;    // 1: leaving edge on the column (l) side
    int32_t ok;
};

// Visit every tree edge on the path between vertices k and l: f(v, side)
// for the edge whose child is v, side 0 on k's branch (in order from k
// upward), 1 on l's branch (from l upward).  The endpoint depths are read
// once: the deeper side climbs to equal depth, then both sides step
// together, so a step costs one parent load per side and the two chains
// overlap.  f returns false to stop.  Result: 0 done, 1 stopped by f,
// -1 the parent/depth arrays are inconsistent.
template <class F>
__device__ __forceinline__ int walk_path(const Ctx& c, int k, int l, int V, F&& f) {
    int x = k, y = l;
    int dx = c.depth[x], dy = c.depth[y];
    if ((unsigned)dx > (unsigned)V || (unsigned)dy > (unsigned)V) return -1;
    for (; dx > dy; dx--) {
        if (!f(x, 0)) return 1;
        x = c.parent[x];
        if (!FLOCK_IN(x, V)) return -1;
    }
    for (; dy > dx; dy--) {
        if (!f(y, 1)) return 1;
        y = c.parent[y];
        if (!FLOCK_IN(y, V)) return -1;
    }
    for (int s = 0; x != y; s++) {
        if (s > V) return -1;
        if (!f(x, 0) || !f(y, 1)) return 1;
        x = c.parent[x];
        y = c.parent[y];
        if (!FLOCK_IN(x, V) || !FLOCK_IN(y, V)) return -1;
    }
    return 0;
}

// Walk the cycle of entering cell (row k, column vertex l).  Edges on the
// k side decrease when their child is a row, on the l side when the child is
// a column.  Ties (impossible with the perturbation) resolve as Cunningham's
// rule: the l side first, highest edge there; else the lowest k-side edge.
// If P != kNoKey every edge is claimed with atomicMin(claim, P).
__device__ __forceinline__ CycleResult cycle_walk(const Ctx& c, int k, int l, uint64_t P, int V) {
    const int m = c.I.m;
    int64_t bk = INT64_MAX, bl = INT64_MAX;
    int qk = -1, ql = -1;
    CycleResult res;
    res.ok = 1;
    const int w = walk_path(c, k, l, V, [&](int v, int side) {
        if (side == 0) {
            if (v < m) { const int64_t f = c.flow[v]; if (f < bk) { bk = f; qk = v; } }
        } else {
            if (v >= m) { const int64_t f = c.flow[v]; if (f <= bl) { bl = f; ql = v; } }
        }
        if (P != kNoKey) atomicMin((unsigned long long*)&c.claim[v], (unsigned long long)P);
        return true;
    });
    if (w < 0) { res.ok = 0; fail_check(c.sc, 11); }
    if (bl <= bk) { res.theta = bl; res.q = ql; res.lside = 1; }
    else          { res.theta = bk; res.q = qk; res.lside = 0; }
    if (res.q < 0) res.ok = 0;
    return res;
}

__device__ __forceinline__ bool cycle_owned(const Ctx& c, int k, int l, uint64_t P, int V) {
    const int w = walk_path(c, k, l, V, [&](int v, int) { return c.claim[v] == P; });
    if (w < 0) fail_check(c.sc, 12);
    return w == 0;
}

__device__ __forceinline__ void cycle_apply(const Ctx& c, int k, int l, const CycleResult& cr, int V) {
    const int m = c.I.m;
    const int64_t th = cr.theta;
    const int w = walk_path(c, k, l, V, [&](int v, int side) {
        c.flow[v] += (side == 0) == (v < m) ? -th : th;
        return true;
    });
    if (w < 0) { fail_check(c.sc, 13); return; }
    // re-hang the subtree below the leaving edge at the entering cell
    int v = cr.lside ? l : k;
    int prev = cr.lside ? k : l;
    int64_t pf = th;
    for (int s = 0; s <= V; s++) {
        if (!FLOCK_IN(v, V)) { fail_check(c.sc, 14); return; }
        const int nxt = c.parent[v];
        const int64_t f = c.flow[v];
        c.parent[v] = prev;
        c.flow[v] = pf;
        if (v == cr.q) break;
        prev = v; pf = f; v = nxt;
        if (s == V) fail_check(c.sc, 15);
    }
}

// int64 -> uint64 preserving order (for unsigned block reductions).
__device__ __forceinline__ uint64_t oflow(int64_t f) { return (uint64_t)f ^ 0x8000000000000000ull; }

// One pivot of entering cell (row k, column vertex l), every step done by the
// whole CTA in parallel on the preorder intervals, and the tree's derived
// state updated in place of a rebuild.
//
// Cycle: a tree edge (child v) is on the cycle iff v's subtree holds exactly
// one of k and l; the k side is the chain from k up to the apex, the l side
// the chain from l.  The leaving edge and theta follow cycle_walk's rule
// exactly: on the k side the decreasing edges are row children and ties go
// to the deepest, on the l side column children, ties to the shallowest; the
// l side wins ties between the sides.  One reduction of two (flow, tie key)
// pairs gives both sides' candidates.  The same pass records both chains by
// distance from their endpoint, with their flows (path[i] / pflow[i] for the
// k side, path[V-1-i] / pflow[V-1-i] for the l side: the cycle has fewer
// than V edges, so they never meet).
//
// Update: let q be the leaving edge's child, e the entering endpoint below
// it (S = subtree of q holds e) and other the endpoint outside S.  The path
// e = p_0, ..., p_t = q (the start of e's chain) is reversed (p_i's new
// parent is p_(i-1), e's is other, with the flow of the edge it replaces
// after the cycle update) and S is re-hung below other; the other cycle
// edges change by -/+theta.  For x in S whose deepest path ancestor is p_i:
// depth' = depth(other) + 1 + i + (depth(x) - depth(p_i)), and every dual in
// S shifts by the entering cell's reduced cost r (rows on e's side of the
// bipartition by +r, the others by -r), so that the new tree edge has zero
// reduced cost.  Intervals: S's block is cut out and re-inserted right after
// other; inside it the branches of p_0, p_1, ... follow one another (branch
// i = subtree(p_i) minus subtree(p_(i-1)), old order kept), so that each
// subtree' is contiguous; sizes change on the path and on the old and new
// ancestors of S.  Old intervals are read from one buffer of iv and the new
// ones written to the other.  Two passes over the vertices, four barriers.
// Returns 1 if the pivot was applied (block-uniform).
template <int J = kJump>
__device__ int single_pivot_iv(const Ctx& c, BlockScratch& bs, int k, int l, int V, PhaseScope* ps = nullptr) {
    const int m = c.I.m;
    const int par = c.sc->ivp;
    const int2* ivA = c.iv + (par ? V : 0);
    int2* ivB = c.iv + (par ? 0 : V);
    const int pk = ivA[k].x, pl = ivA[l].x;
    const int dk = c.depth[k], dl = c.depth[l];
    // the entering cell's reduced cost (exact): read here, before any dual
    // changes, like everything the update reads of other vertices (after the
    // reduction other warps may already be rewriting depths, parents, duals)
    const int64_t r = (int64_t)cost_of(c.I, k, l - m) - c.pot[k] - c.pot[l];
    int32_t* path = c.path;
    int64_t* pflow = c.pflow;
    // (order-preserving flow, tie key): k side ties to the largest (depth, v),
    // so its key is complemented; l side to the smallest
    uint64_t kf = kNoKey, kt = kNoKey, lf = kNoKey, lt = kNoKey;
    int bad = 0;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        if (c.parent[v] < 0) continue;
        const int2 w = ivA[v];
        const bool on_k = iv_in(w, pk), on_l = iv_in(w, pl);
        if (on_k == on_l) continue;
        const int dv = c.depth[v];
        const int64_t f = c.flow[v];
        const int i = on_k ? dk - dv : dl - dv;
        if (!FLOCK_IN(i, V)) { bad = 1; continue; }
        const int slot = on_k ? i : V - 1 - i;
        path[slot] = v;
        pflow[slot] = f;
        const uint64_t tie = ((uint64_t)(uint32_t)dv << 32) | (uint32_t)v;
        if (on_k && v < m) pair_min_into(kf, kt, oflow(f), ~tie);
        if (on_l && v >= m) pair_min_into(lf, lt, oflow(f), tie);
    }
    if (bad) { kf = 0; kt = 0; }                           // no real pair is (0, 0): it carries the failure
    if (threadIdx.x == 0) bs.i[4] = 0;                     // ordered by the reduction's barriers
    block_min_pairs(kf, kt, lf, lt, bs);
    if (kf == 0 && kt == 0) {                              // block-uniform
        if (threadIdx.x == 0) fail_check(c.sc, 17);
        __syncthreads();
        return 0;
    }
    const bool lside = lf <= kf;                           // uniform
    const uint64_t fmin = lside ? lf : kf;
    const uint64_t qkey = lside ? lt : ~kt;                // (depth << 32) | child of the leaving edge
    const int q = (int)(uint32_t)qkey;
    const int e = lside ? l : k, other = lside ? k : l;
    const int de = lside ? dl : dk;
    const int t = de - (int)(uint32_t)(qkey >> 32);
    const int base = lside ? V - 1 : 0, dir = lside ? -1 : 1;   // e's chain entry i at path[base + dir * i]
    if (fmin == kNoKey || !FLOCK_IN(q, V) || !FLOCK_IN(t, V) || path[base + dir * t] != q) {   // uniform
        if (threadIdx.x == 0) fail_check(c.sc, 16);
        __syncthreads();
        return 0;
    }
    if (ps) ps->mark(PH_ADJUST);                          // cycle known; leaving edge chosen by the reduction
    const int64_t th = (int64_t)(fmin ^ 0x8000000000000000ull);
    const int eside = lside ? 2 : 1;
    const int dother = lside ? dk : dl;
    const int2 Q = ivA[q], O = ivA[other];
    const int P = Q.x, s = Q.y;
    const int ins = O.x - (O.x >= P + s ? s : 0) + 1;   // S's new first position
    const int dnew = dother + 1 - de;                  // depth' = dnew + 2 i + depth
    const bool erow = e < m;
    int dwide = 0;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int pv0 = c.parent[v];
        if (pv0 == -2) continue;                       // not in the tree
        const int2 w = ivA[v];
        int side = 0;
        if (pv0 >= 0) {
            const bool on_k = iv_in(w, pk), on_l = iv_in(w, pl);
            side = on_k != on_l ? (on_k ? 1 : 2) : 0;
        }
        int2 nw;
        if (iv_in(Q, w.x)) {
            // deepest path vertex above v: smallest i whose subtree holds v
            int lo = 0, hi = t;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                const int pv = path[base + dir * mid];
                if (!FLOCK_IN(pv, V)) { bad = 1; break; }
                if (iv_in(ivA[pv], w.x)) hi = mid; else lo = mid + 1;
            }
            const int i = lo;
            const int pi = path[base + dir * i];
            if (!FLOCK_IN(pi, V)) { bad = 1; continue; }
            const int2 Pi = ivA[pi];
            int off = 0, rank = w.x - Pi.x;
            int pc = -1;
            if (i > 0) {
                pc = path[base + dir * (i - 1)];
                if (!FLOCK_IN(pc, V)) { bad = 1; continue; }
                const int2 Pc = ivA[pc];
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
    if (dwide) atomicAdd(&bs.i[4], dwide);
    bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        if (bad) fail_check(c.sc, 24);
        c.sc->ivp = par ^ 1;
        c.sc->nwide += bs.i[4];
        c.sc->narrow = c.sc->nwide == 0;
    }
    return bad ? 0 : 1;
}

// ------------------------------------------------- parallel stepping stone --
// -a parallel_ss (ss_model_parallel.cu:128-246, PIVOT_ss.cu:294-571,
// parallel_kernels.cu:396-660): every cell with a negative cycle cost is a
// candidate; candidates are taken most negative first (ties in row-major
// order) and one is accepted unless its cycle shares a tree edge with a
// cycle accepted before it; all accepted cycles pivot in the same round.
// The reference computes each cell's cycle cost from per-row tree searches
// (alternating sums of the path costs, no duals); along any tree path those
// sums telescope to u_i + v_j, so the cycle cost of cell (i, j) is exactly
// c_ij - u_i - v_j in integer arithmetic, which the round reads from the
// full sweep's duals.  Candidates: the negative cells below a 32-bin
// histogram threshold over [min, 0), at most kSSCap (and m) of them, in
// row-major order -- the most negative ones, so the accepted set is the
// reference's greedy choice restricted to them.  Selection: rounds of edge
// claims (atomicMin of the candidate's priority (cost, slot)) among the
// undecided candidates; one that owns every edge of its cycle is accepted
// and marks its edges taken, one whose cycle holds a taken edge is
// rejected.  Each selection round accepts at least the best undecided
// candidate, and the result is the lexicographically first independent set
// by priority: the sequential greedy's.
constexpr int kSSCap = 1024;

// Candidate s of an ss round: row cand[s], column uf[s], priority row_best[s],
// theta cand_theta[s], leaving edge cand_q[s], cand_info[s]: bit 0 leaving
// edge on the column side, bit 1 accepted, bit 2 rejected, bit 3 walk failed.
__device__ __forceinline__ int64_t cell_reduced(const Ctx& c, int i, int j) {
    return (int64_t)cost_of(c.I, i, j) - c.pot[i] - c.pot[c.I.m + j];
}

template <int J = kJump>
__device__ void ss_round_cta(const Ctx& c, BlockScratch& bs, PhaseScope* ps) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int cap = min(kSSCap, m);
    // the most negative cycle cost (the full sweep's row keys)
    int32_t rmin = 0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) rmin = min(rmin, key_val(c.row_best[i]));
    rmin = key_val(block_min_u64(pack_i32(rmin, 0u), bs));
    if (rmin >= 0) {
        if (threadIdx.x == 0) { c.sc->done = 1; c.sc->ncand = 0; }
        return;
    }
    const int64_t span = -(int64_t)rmin;
    // histogram of every negative cell
    if (threadIdx.x < 32) bs.red2[threadIdx.x] = 0;
    __syncthreads();
    for (int i = warp; i < m; i += nw)
        for (int j = lane; j < n; j += 32) {
            const int64_t r = cell_reduced(c, i, j);
            if (r < 0) atomicAdd((unsigned long long*)&bs.red2[((int64_t)clamp32(r) - rmin) * 32 / span], 1ull);
        }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t cum = bs.red2[0];
        int last = 0;
        for (int b = 1; b < 32 && cum + bs.red2[b] <= (uint64_t)cap; b++) { cum += bs.red2[b]; last = b; }
        bs.i[1] = last;
    }
    __syncthreads();
    const int last = bs.i[1];
    auto chosen = [&](int64_t r) { return r < 0 && ((int64_t)clamp32(r) - rmin) * 32 / span <= last; };
    // per-row counts, their exclusive scan, then each row's cells in column order
    for (int i = warp; i < m; i += nw) {
        int cnt = 0;
        for (int j = lane; j < n; j += 32) cnt += chosen(cell_reduced(c, i, j)) ? 1 : 0;
        cnt = (int)__reduce_add_sync(0xffffffffu, (unsigned)cnt);
        if (lane == 0) c.cand_info[i] = cnt;
    }
    __syncthreads();
    const int total = block_exclusive_scan_i32(c.cand_info, m, bs);
    const int ncand = min(total, cap);
    for (int i = warp; i < m; i += nw) {
        int pos = c.cand_info[i];
        if (pos >= ncand) continue;
        for (int j0 = 0; j0 < n && pos < ncand; j0 += 32) {
            const int j = j0 + lane;
            const int64_t r = j < n ? cell_reduced(c, i, j) : 0;
            const bool sel = j < n && chosen(r);
            const unsigned mask = __ballot_sync(0xffffffffu, sel);
            const int slot = pos + __popc(mask & ((1u << lane) - 1u));
            if (sel && slot < ncand) {
                c.cand[slot] = i;
                c.uf[slot] = j;
                c.row_best[slot] = pack_i32(clamp32(r), (uint32_t)slot);
            }
            pos += __popc(mask);
        }
    }
    for (int v = threadIdx.x; v < V; v += blockDim.x) { c.claim[v] = kNoKey; c.side[v] = 0; }
    __syncthreads();
    for (int t = threadIdx.x; t < ncand; t += blockDim.x) c.cand_info[t] = 0;
    if (ps) ps->mark(PH_RESOLVE);
    // selection rounds (each accepts the best undecided candidate at least)
    int bad = 0;
    for (int it = 0; it <= ncand; it++) {
        // claims of the undecided candidates; theta and the leaving edge on the first walk
        for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
            if (c.cand_info[t] & 14) continue;
            const int k = c.cand[t], l = m + c.uf[t];
            const uint64_t P = c.row_best[t];
            bool taken = false;
            const int w = walk_path(c, k, l, V, [&](int v, int) {
                if (c.side[v]) { taken = true; return false; }
                return true;
            });
            if (w < 0) { c.cand_info[t] |= 8; bad = 1; continue; }
            if (taken) { c.cand_info[t] |= 4; continue; }
            if (it == 0) {
                const CycleResult cr = cycle_walk(c, k, l, P, V);
                if (!cr.ok) { c.cand_info[t] |= 8; bad = 1; continue; }
                c.cand_theta[t] = cr.theta;
                c.cand_q[t] = cr.q;
                c.cand_info[t] |= cr.lside;
            } else {
                walk_path(c, k, l, V, [&](int v, int) {
                    atomicMin((unsigned long long*)&c.claim[v], (unsigned long long)P);
                    return true;
                });
            }
        }
        __syncthreads();
        int undecided = 0;
        for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
            if (c.cand_info[t] & 14) continue;
            if (cycle_owned(c, c.cand[t], m + c.uf[t], c.row_best[t], V)) c.cand_info[t] |= 2 | 16;   // 16: new this round
            else undecided++;
        }
        __syncthreads();
        // the new winners mark their edges taken; every claim is reset
        for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
            if (!(c.cand_info[t] & 16)) continue;
            c.cand_info[t] &= ~16;
            walk_path(c, c.cand[t], m + c.uf[t], V, [&](int v, int) { c.side[v] = 1; return true; });
        }
        for (int v = threadIdx.x; v < V; v += blockDim.x) c.claim[v] = kNoKey;
        undecided = (int)block_sum_i64(undecided, bs);     // its barriers order the marks and resets
        if (undecided == 0) break;
    }
    if (ps) ps->mark(PH_ADJUST);
    // the accepted cycles are edge-disjoint: they pivot together
    int wins = 0;
    for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
        if ((c.cand_info[t] & 2) == 0) continue;
        CycleResult cr;
        cr.theta = c.cand_theta[t]; cr.q = c.cand_q[t]; cr.lside = c.cand_info[t] & 1; cr.ok = 1;
        cycle_apply(c, c.cand[t], m + c.uf[t], cr, V);
        wins++;
    }
    const int64_t w = block_sum_i64(wins, bs);
    const int any_bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        c.sc->pivots += (int32_t)w;
        c.sc->ncand = ncand;
        c.sc->last_winners = (int32_t)w;
        c.sc->stale = 1;
        if (any_bad || w == 0) { c.sc->status |= ST_TREE_CORRUPT; c.sc->done = 1; }
    }
    __syncthreads();
}

// Parallel mode: candidates walked per round (the rest wait for later rounds).
constexpr int kMaxCand = 32;
// Switch mode: a parallel round applying fewer pivots than this switches the
// instance to sequential rounds (switch/switch_model_parallel.cu:182-184).
constexpr int kSwitchPivots = 10;

// One pricing round after sweep: choose candidates, claim, apply.
// have_best: the sweep already reduced the sequential rule's entering row
// (pre_best, kNoKey: none).  With partial pricing only the listed candidate
// rows hold keys this round, and only they are read.
// kSS: the parallel stepping-stone mode (Scalars::mode 3) is compiled in
// (the plain solver's round kernel); the persistent kernels leave it out and
// keep their registers.
template <int J = kJump, bool kSS = false>
__device__ void pivot_round_cta(const Ctx& c, BlockScratch& bs, bool have_best = false, uint64_t pre_best = kNoKey,
                                PhaseScope* ps = nullptr) {
    const InstDev& I = c.I;
    const int m = I.m, V = m + I.n;
    const int mode = c.sc->mode;
    if (kSS && mode == 3) {   // parallel stepping stone (full pricing: every row key is current)
        if (ps) ps->mark(PH_CYCLE);
        ss_round_cta<J>(c, bs, ps);
        return;
    }
    // a candidate key whose column is outside the instance is an internal
    // error: recorded, never used as an index
    const uint32_t ncols = (uint32_t)I.n;
    const bool plist = c.sc->pricing != 0;
    const int nrows = plist ? min(max(c.sc->pp_n, 0), kPPRows) : m;
    int ncand = 0, first = 0;
    if (mode == 0 && have_best) {
        ncand = pre_best != kNoKey ? 1 : 0;
        first = (int)key_idx(pre_best);
        if (ncand && (!FLOCK_IN(first, m) || key_idx(c.row_best[first]) >= ncols)) {   // block-uniform
            if (threadIdx.x == 0) fail_check(c.sc, 18);
            return;
        }
    } else {
    if (threadIdx.x == 0) bs.i[0] = 0;
    __syncthreads();
    if (mode == 0) {
        uint64_t best = kNoKey;
        for (int t = threadIdx.x; t < nrows; t += blockDim.x) {
            const int i = plist ? c.prow[t] : t;
            if (!FLOCK_IN(i, m)) continue;
            const uint64_t k = c.row_best[i];
            if (k != kNoKey && key_val(k) < 0 && key_idx(k) >= ncols) { fail_check(c.sc, 18); continue; }
            if (k != kNoKey && key_val(k) < 0) {
                const uint64_t P = pack_i32(key_val(k), (uint32_t)i);
                best = P < best ? P : best;
            }
        }
        best = block_min_u64(best, bs);
        if (threadIdx.x == 0 && best != kNoKey) { c.cand[0] = (int32_t)key_idx(best); bs.i[0] = 1; }
    } else {
        // Candidates: the rows with the most negative best reduced costs, at
        // most kMaxCand (plus ties of the boundary bin when the first bin
        // alone exceeds it).  A 32-bin histogram over [rmin, 0) picks the
        // threshold, so the set depends only on the values.  A candidate is
        // applied only if no better candidate's cycle shares an edge with it,
        // so leaving out weaker rows changes no decision among the rest; the
        // cap bounds the cycle walks of a round.
        int32_t rmin = 0;
        for (int t = threadIdx.x; t < nrows; t += blockDim.x) {
            const int i = plist ? c.prow[t] : t;
            if (!FLOCK_IN(i, m)) continue;
            const uint64_t k = c.row_best[i];
            if (k != kNoKey && key_val(k) < 0 && key_idx(k) >= ncols) { fail_check(c.sc, 18); continue; }
            if (k != kNoKey) rmin = min(rmin, key_val(k));
        }
        rmin = key_val(block_min_u64(pack_i32(rmin, 0u), bs));
        if (rmin < 0) {
            const int64_t span = -(int64_t)rmin;
            if (threadIdx.x < 32) bs.red2[threadIdx.x] = 0;
            __syncthreads();
            for (int t = threadIdx.x; t < nrows; t += blockDim.x) {
                const int i = plist ? c.prow[t] : t;
                if (!FLOCK_IN(i, m)) continue;
                const uint64_t k = c.row_best[i];
                if (k != kNoKey && key_val(k) < 0 && key_idx(k) < ncols)
                    atomicAdd((unsigned long long*)&bs.red2[((int64_t)key_val(k) - rmin) * 32 / span], 1ull);
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                uint64_t cum = bs.red2[0];
                int last = 0;
                for (int b = 1; b < 32 && cum + bs.red2[b] <= (uint64_t)kMaxCand; b++) { cum += bs.red2[b]; last = b; }
                bs.i[1] = last;
            }
            __syncthreads();
            const int last = bs.i[1];
            for (int t = threadIdx.x; t < nrows; t += blockDim.x) {
                const int i = plist ? c.prow[t] : t;
                if (!FLOCK_IN(i, m)) continue;
                const uint64_t k = c.row_best[i];
                if (k != kNoKey && key_val(k) < 0 && key_idx(k) < ncols &&
                    ((int64_t)key_val(k) - rmin) * 32 / span <= last)
                    c.cand[atomicAdd(&bs.i[0], 1)] = i;
            }
        }
    }
    __syncthreads();
    ncand = bs.i[0];
    first = c.cand[0];
    }
    // The two outcomes below end with thread 0 writing the scalars; every
    // caller follows with its own thread-0 update and a barrier before the
    // scalars are read again.
    if (ncand == 0) {
        if (threadIdx.x == 0) { c.sc->done = 1; c.sc->ncand = 0; }
        return;
    }
    if (ps) ps->mark(PH_CYCLE);
    if (ncand == 1) {
        const int ok = single_pivot_iv<J>(c, bs, first, m + (int)key_idx(c.row_best[first]), V, ps);
        if (threadIdx.x == 0) {
            c.sc->pivots += ok;
            c.sc->ncand = 1;
            c.sc->last_winners = ok;
            if (!ok) { c.sc->status |= ST_TREE_CORRUPT; c.sc->done = 1; }
            if (mode == 2) c.sc->mode = 0;
        }
        return;
    }
    // Several candidates: claims, ownership, then the owners applied; the
    // tree's derived state is rebuilt before the next sweep.
    for (int v = threadIdx.x; v < V; v += blockDim.x) c.claim[v] = kNoKey;
    __syncthreads();
    int bad = 0;
    for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
        const int i = c.cand[t];
        const uint64_t key = c.row_best[i];
        const int l = m + (int)key_idx(key);
        const uint64_t P = pack_i32(key_val(key), (uint32_t)i);
        const CycleResult cr = cycle_walk(c, i, l, P, V);
        c.cand_theta[t] = cr.theta;
        c.cand_q[t] = cr.q;
        c.cand_info[t] = cr.lside | (cr.ok ? 0 : 4);
        bad |= !cr.ok;
    }
    __syncthreads();
    if (ps) ps->mark(PH_RESOLVE);
    int wins = 0;
    for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
        if (c.cand_info[t] & 4) continue;
        const int i = c.cand[t];
        const uint64_t key = c.row_best[i];
        const int l = m + (int)key_idx(key);
        const uint64_t P = pack_i32(key_val(key), (uint32_t)i);
        if (cycle_owned(c, i, l, P, V)) { c.cand_info[t] |= 2; wins++; }
    }
    __syncthreads();
    if (ps) ps->mark(PH_ADJUST);
    for (int t = threadIdx.x; t < ncand; t += blockDim.x) {
        if (!(c.cand_info[t] & 2)) continue;
        const int i = c.cand[t];
        const int l = m + (int)key_idx(c.row_best[i]);
        CycleResult cr;
        cr.theta = c.cand_theta[t]; cr.q = c.cand_q[t]; cr.lside = c.cand_info[t] & 1; cr.ok = 1;
        cycle_apply(c, i, l, cr, V);
    }
    const int64_t w = block_sum_i64(wins, bs);
    const int any_bad = __syncthreads_or(bad);
    if (threadIdx.x == 0) {
        c.sc->pivots += (int32_t)w;
        c.sc->ncand = ncand;
        c.sc->last_winners = (int32_t)w;
        c.sc->stale = 1;
        if (any_bad || w == 0) { c.sc->status |= ST_TREE_CORRUPT; c.sc->done = 1; }
        if (mode == 2 && w < kSwitchPivots) c.sc->mode = 0;
    }
    __syncthreads();
}

// -------------------------------------------------------------- finalize ----
// Attach zero-demand columns, recover original flows, write the basis and the
// objective.  Dual of a zero-demand column: min_i (c_ij - u_i).
__device__ void finalize_cta(const Ctx& c, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    const int root = c.sc->root;
    const int64_t M = c.sc->M;
    const int64_t half = (M - 1) / 2;
    for (int j = 0; j < n; j++) {
        if (c.parent[m + j] != -2) continue;      // uniform: all threads read the same
        uint64_t best = kNoKey;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const int64_t val = (int64_t)cost_of(I, i, j) - c.pot[i];
            const uint64_t k = (uint64_t)val ^ 0x8000000000000000ull;
            best = k < best ? k : best;
        }
        best = block_min_u64(best, bs);
        const int64_t vmin = (int64_t)(best ^ 0x8000000000000000ull);
        uint64_t who = kNoKey;
        for (int i = threadIdx.x; i < m; i += blockDim.x)
            if ((int64_t)cost_of(I, i, j) - c.pot[i] == vmin) who = (uint64_t)i < who ? (uint64_t)i : who;
        who = block_min_u64(who, bs);
        if (threadIdx.x == 0) { c.parent[m + j] = (int)who; c.pot[m + j] = vmin; c.flow[m + j] = 0; }
        __syncthreads();
    }
    int64_t obj = 0;
    int32_t act = 0;
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        if (v == root) continue;
        const int k = v < root ? v : v - 1;
        const int p = c.parent[v];
        if (!FLOCK_IN(p, V) || (p < m) == (v < m)) { fail_check(c.sc, 41); continue; }
        const int row = v < m ? v : p, col = v < m ? p - m : v - m;
        const int64_t x = (c.flow[v] + half) / M;   // flow = M x + t, |t| <= V'-1 < M/2
        c.out_src[k] = row; c.out_dst[k] = col; c.out_qty[k] = (int32_t)x;
        obj += x * (int64_t)cost_of(I, row, col);
        act += x > 0;
    }
    obj = block_sum_i64(obj, bs);
    const int64_t a = block_sum_i64(act, bs);
    if (threadIdx.x == 0) { c.sc->objective = obj; c.sc->active = (int32_t)a; }
    __syncthreads();
}

// ----------------------------------------------------------- certificate ----
// Independent exact check of the result: quantities >= 0, row/column sums,
// every reduced cost >= 0 (full pass over the matrix), complementary slackness.
__device__ void certify_flows_cta(const Ctx& c, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n, V = m + n;
    for (int v = threadIdx.x; v < V; v += blockDim.x) c.bsum[v] = 0;
    if (threadIdx.x == 0) bs.i[0] = 0;
    __syncthreads();
    int bits = 0;
    for (int k = threadIdx.x; k < V - 1; k += blockDim.x) {
        const int a = c.out_src[k], b = c.out_dst[k], q = c.out_qty[k];
        if (a < 0 || a >= m || b < 0 || b >= n || q < 0) { bits |= 1; continue; }
        atomicAdd((unsigned long long*)&c.bsum[a], (unsigned long long)(int64_t)q);
        atomicAdd((unsigned long long*)&c.bsum[m + b], (unsigned long long)(int64_t)q);
        const int64_t r = (int64_t)cost_of(I, a, b) - c.pot[a] - c.pot[m + b];
        if (q > 0 && r != 0) bits |= 16;
    }
    __syncthreads();
    for (int v = threadIdx.x; v < V; v += blockDim.x) {
        const int64_t want = v < m ? I.supply[v] : I.demand[v - m];
        if (c.bsum[v] != want) bits |= v < m ? 2 : 4;
    }
    atomicOr(&bs.i[0], bits);
    __syncthreads();
    if (threadIdx.x == 0) c.sc->cert |= bs.i[0];
    __syncthreads();
}

__device__ void certify_cells_cta(const Ctx& c, BlockScratch& bs) {
    const InstDev& I = c.I;
    const int m = I.m, n = I.n;
    int64_t neg = 0;
    for (int i = threadIdx.x >> 5; i < m; i += blockDim.x >> 5) {
        const int64_t u = c.pot[i];
        for (int j = threadIdx.x & 31; j < n; j += 32)
            neg += ((int64_t)cost_of(I, i, j) - u - c.pot[m + j]) < 0;
    }
    neg = block_sum_i64(neg, bs);
    if (threadIdx.x == 0) { c.sc->neg_cells = neg; if (neg) c.sc->cert |= 8; }
    __syncthreads();
}

}  // namespace flock
