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
// Batched path: k_batch, one CTA per instance with work stealing over a
// size-sorted queue; one launch (stream) per size bucket.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/flock.h"
#include "simplex.cuh"
#include "internal.h"

namespace flock {

// ------------------------------------------------------------ kernels ------
__global__ void __launch_bounds__(1024) k_setup(Ctx c, int bfs_method) {
    __shared__ BlockScratch bs;
    if (bfs_method == FLOCK_BFS_VOGEL) {
        vogel_cta(c, bs);
    } else {
        if (threadIdx.x == 0) { nwc_thread0(c); c.sc->events = 0; }
        __syncthreads();
    }
    if (threadIdx.x == 0 && c.sc->events < 0) c.sc->status |= ST_VOGEL_UNDEF;
    sf_init_cta(c, bs);
    if (!c.sc->done) tree_recompute_cta(c, bs);
    for (int i = threadIdx.x; i < c.I.m; i += blockDim.x) c.row_best[i] = kNoKey;
}

__global__ void __launch_bounds__(1024) k_vogel_only(Ctx c) {
    __shared__ BlockScratch bs;
    vogel_cta(c, bs);
}

// Grid-wide sweep.  blockIdx.x = tile + ntile * row_group.  Each warp owns
// one row segment of `tile` columns; lanes read 16-byte vectors.
__global__ void __launch_bounds__(256) k_sweep(Ctx c, int tile, int ntile) {
    if (c.sc->done) return;
    extern __shared__ int64_t vt[];
    const InstDev& I = c.I;
    const int m = I.m, n = I.n;
    const int t = blockIdx.x % ntile, rg = blockIdx.x / ntile, nrg = gridDim.x / ntile;
    const int j0 = t * tile;
    const int jn = min(tile, n - j0);
    for (int jj = threadIdx.x; jj < jn; jj += blockDim.x) vt[jj] = c.pot[m + j0 + jj];
    __syncthreads();
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5, warp = threadIdx.x >> 5;
    const int nq = (jn + 3) >> 2;
    for (int i = rg * wpb + warp; i < m; i += nrg * wpb) {
        const int4* row = reinterpret_cast<const int4*>(I.cost + (size_t)i * I.ldc + j0);
        const int64_t u = c.pot[i];
        uint64_t best = kNoKey;
        #pragma unroll 4
        for (int q = lane; q < nq; q += 32) {
            const int4 cv = __ldcs(row + q);   // streamed once per round: do not keep in L1
            const int jl = q * 4;
            const int32_t cc[4] = {cv.x, cv.y, cv.z, cv.w};
            #pragma unroll
            for (int e = 0; e < 4; e++) {
                if (jl + e < jn) {
                    const int64_t r = (int64_t)cc[e] - u - vt[jl + e];
                    const uint64_t k = pack_i32(clamp32(r), (uint32_t)(j0 + jl + e));
                    best = k < best ? k : best;
                }
            }
        }
        best = warp_min_u64(best);
        if (lane == 0) {
            if (ntile == 1) c.row_best[i] = best;
            else atomicMin((unsigned long long*)&c.row_best[i], (unsigned long long)best);
        }
    }
}

__global__ void __launch_bounds__(1024) k_pivot(Ctx c) {
    __shared__ BlockScratch bs;
    if (c.sc->done) return;
    pivot_round_cta(c, bs);
    if (threadIdx.x == 0) {
        c.sc->rounds++;
        if (!c.sc->done && c.sc->rounds >= c.sc->max_rounds) { c.sc->status |= ST_ITER_CAP; c.sc->done = 1; }
    }
    __syncthreads();
    if (!c.sc->done) tree_recompute_cta(c, bs);
    for (int i = threadIdx.x; i < c.I.m; i += blockDim.x) c.row_best[i] = kNoKey;
}

__global__ void __launch_bounds__(1024) k_finalize(Ctx c) {
    __shared__ BlockScratch bs;
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


__global__ void k_fill_bench(int32_t* cost, size_t cells, int64_t* pot, int V) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < cells; k += (size_t)gridDim.x * blockDim.x)
        cost[k] = (int32_t)((k * 2654435761u) % 1414u);
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < (size_t)V; k += (size_t)gridDim.x * blockDim.x)
        pot[k] = (int64_t)((k * 40503u) % 700u);
}

// ------------------------------------------------------- batched kernel ----
__global__ void __launch_bounds__(512) k_batch(BatchArgs a) {
    __shared__ BlockScratch bs;
    __shared__ int s_idx;
    extern __shared__ __align__(16) unsigned char smem[];
    uint8_t* scratch = a.scratch + (size_t)blockIdx.x * a.scratch_per_cta;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(a.next, 1);
        __syncthreads();
        const int idx = s_idx;
        __syncthreads();
        if (idx >= a.count) break;
        const BatchDesc d = a.desc[idx];
        if (d.m < 1 || d.n < 1 || d.m + d.n > a.maxV || d.m > a.maxM || d.ldc < d.n || (d.ldc & 3) ||
            (d.cost_off & 3)) {
            if (threadIdx.x == 0) {
                a.sc[d.index].status = ST_TREE_CORRUPT;
                a.sc[d.index].fail_site = 1;
            }
            continue;
        }
        Ctx c;
        c.I.m = d.m; c.I.n = d.n; c.I.ldc = d.ldc;
        c.I.cost = a.cost + d.cost_off;
        c.I.supply = a.sd + d.sd_off;
        c.I.demand = a.sd + d.sd_off + d.m;
        c.sc = a.sc + d.index;
        const int V = d.m + d.n;
        c.out_src = a.out_src + d.out_off; c.out_dst = a.out_dst + d.out_off; c.out_qty = a.out_qty + d.out_off;
        int64_t* pot_global = a.pot_out + d.pot_off;
        carve_ctx(c, scratch, a.maxV, a.maxM, a.smem_mode ? smem : nullptr, pot_global);
        if (threadIdx.x == 0) {
            Scalars z;
            memset(&z, 0, sizeof(z));
            z.max_rounds = a.max_rounds;
            z.mode = a.mode;
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
        // the start list is needed later only for the Vogel output: keep it
        for (int k = threadIdx.x; k < V - 1; k += blockDim.x) {
            a.bfs_out[3 * (d.out_off + k) + 0] = c.bfs_src[k];
            a.bfs_out[3 * (d.out_off + k) + 1] = c.bfs_dst[k];
            a.bfs_out[3 * (d.out_off + k) + 2] = c.bfs_qty[k];
        }
        __syncthreads();
        sf_init_cta(c, bs);
        if (!c.sc->done) tree_recompute_cta(c, bs);
        for (int guard = 0; guard < (1 << 30); guard++) {
            if (c.sc->done) break;
            sweep_cta(c);
            pivot_round_cta(c, bs);
            if (threadIdx.x == 0) {
                c.sc->rounds++;
                if (!c.sc->done && c.sc->rounds >= c.sc->max_rounds) { c.sc->status |= ST_ITER_CAP; c.sc->done = 1; }
            }
            __syncthreads();
            if (c.sc->done) break;
            tree_recompute_cta(c, bs);
        }
        if (!(c.sc->status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE))) {
            finalize_cta(c, bs);
            certify_flows_cta(c, bs);
            certify_cells_cta(c, bs);
        }
        if (a.smem_mode)
            for (int v = threadIdx.x; v < V; v += blockDim.x) pot_global[v] = c.pot[v];
        __syncthreads();
    }
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

int validate_instance(const flock_instance* I) {
    if (!I || !I->supply || !I->demand || !I->cost || I->m < 1 || I->n < 1) { set_error("invalid instance"); return FLOCK_ERR_ARG; }
    if ((int64_t)I->m + I->n > (1 << 28) || (int64_t)I->m * I->n > ((int64_t)1 << 34)) { set_error("instance too large"); return FLOCK_ERR_RANGE; }
    int64_t S = 0, D = 0;
    for (int i = 0; i < I->m; i++) { if (I->supply[i] < 0) { set_error("negative supply"); return FLOCK_ERR_ARG; } S += I->supply[i]; }
    for (int j = 0; j < I->n; j++) { if (I->demand[j] < 0) { set_error("negative demand"); return FLOCK_ERR_ARG; } D += I->demand[j]; }
    if (S != D) { set_error("unbalanced instance"); return FLOCK_ERR_UNBALANCED; }
    const size_t mn = (size_t)I->m * I->n;
    for (size_t k = 0; k < mn; k++) {
        const int32_t c = I->cost[k];
        if (c > (1 << 30) || c < -(1 << 30)) { set_error("cost out of range"); return FLOCK_ERR_RANGE; }
    }
    return FLOCK_OK;
}

static int threads_for(int V) {
    int t = ((V + 31) / 32) * 32;
    return std::max(128, std::min(1024, t));
}

// --------------------------------------------------------- plain solver ----
struct PlainSolver {
    std::mutex mu;
    DevBuf ws, cost, sd;
    HostBuf h_sc;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    bool init = false;

    int setup() {
        if (init) return FLOCK_OK;
        FLOCK_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        for (auto& e : ev) FLOCK_CK(cudaEventCreate(&e));
        FLOCK_CK(h_sc.ensure(sizeof(Scalars)));
        FLOCK_CK(cudaFuncSetAttribute(k_sweep, cudaFuncAttributeMaxDynamicSharedMemorySize, 8192 * 8));
        init = true;
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
        FLOCK_CK(ws.ensure(extra_off + out_bytes + al256(sizeof(Scalars))));
        carve_ctx(c, ws.as<uint8_t>(), V, m, nullptr, nullptr);
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

    int reset_scalars(Scalars* dsc, int mode, int max_rounds) {
        Scalars z;
        memset(&z, 0, sizeof(z));
        z.mode = mode;
        z.max_rounds = max_rounds;
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

static int solve_plain(const flock_instance* I, const flock_options* opt_in, flock_flow* flows,
                       int64_t* du, int64_t* dv, flock_stats* st) {
    const auto t0 = std::chrono::steady_clock::now();
    int rc = validate_instance(I);
    if (rc) return rc;
    flock_options opt;
    flock_default_options(&opt);
    if (opt_in) opt = *opt_in;
    const int max_rounds = opt.max_iterations > 0 ? opt.max_iterations : (1 << 30);
    PlainSolver& P = plain();
    std::lock_guard<std::mutex> lk(P.mu);
    if ((rc = P.setup())) return rc;
    const int m = I->m, n = I->n, V = m + n;
    Ctx c;
    int32_t* out3 = nullptr;
    if ((rc = P.prepare(I, c, &out3))) return rc;
    if ((rc = P.reset_scalars(c.sc, opt.pivot_method == FLOCK_PIVOT_SEQUENTIAL ? 0 : 1, max_rounds))) return rc;
    const int nt = threads_for(V);
    FLOCK_CK(cudaEventRecord(P.ev[0], P.stream));
    k_setup<<<1, nt, 0, P.stream>>>(c, opt.bfs_method == FLOCK_BFS_NWC ? FLOCK_BFS_NWC : FLOCK_BFS_VOGEL);
    FLOCK_CK(cudaGetLastError());
    FLOCK_CK(cudaEventRecord(P.ev[1], P.stream));
    // sweep launch shape
    const int tile = std::min((n + 3) & ~3, 8192);
    const int ntile = (n + tile - 1) / tile;
    const int nrg = std::max(1, std::min((m + 7) / 8, (4 * num_sms()) / ntile));
    const int grid = ntile * nrg;
    const size_t smem = (size_t)tile * 8;
    // pivot loop: chunks of rounds captured once as a CUDA graph
    int chunk = 8;
    cudaGraphExec_t exec = nullptr;
    int exec_chunk = 0;
    Scalars* hs = P.h_sc.as<Scalars>();
    for (;;) {
        if (exec_chunk != chunk) {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
            cudaGraph_t g;
            FLOCK_CK(cudaStreamBeginCapture(P.stream, cudaStreamCaptureModeThreadLocal));
            for (int r = 0; r < chunk; r++) {
                k_sweep<<<grid, 256, smem, P.stream>>>(c, tile, ntile);
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
        st->ms_bfs = ms_bfs;
        st->ms_simplex = ms_loop;
        st->ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    return status ? FLOCK_ERR_NOT_OPTIMAL : FLOCK_OK;
}

static int vogel_plain(const flock_instance* I, flock_flow* flows, int32_t* events) {
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
    k_vogel_only<<<1, threads_for(V), 0, P.stream>>>(c);
    FLOCK_CK(cudaGetLastError());
    std::vector<int32_t> a((size_t)V), b((size_t)V), q((size_t)V);
    FLOCK_CK(cudaMemcpyAsync(a.data(), c.bfs_src, (size_t)(V - 1) * 4, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(b.data(), c.bfs_dst, (size_t)(V - 1) * 4, cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaMemcpyAsync(q.data(), c.bfs_qty, (size_t)(V - 1) * 4, cudaMemcpyDeviceToHost, P.stream));
    Scalars* hs = P.h_sc.as<Scalars>();
    FLOCK_CK(cudaMemcpyAsync(hs, c.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, P.stream));
    FLOCK_CK(cudaStreamSynchronize(P.stream));
    for (int k = 0; k < V - 1; k++) flows[k] = {a[k], b[k], q[k]};
    if (events) *events = hs->events;
    return FLOCK_OK;
}



// Benchmark hook: time `iters` launches of the fused sweep on an m x n matrix
// with random costs and duals already resident (no pivots).  Writes the
// average launch time (CUDA events on the launching stream).
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
    const int tile = std::min(ldc, 8192);
    const int ntile = (n + tile - 1) / tile;
    const int nrg = std::max(1, std::min((m + 7) / 8, (4 * num_sms()) / ntile));
    const size_t smem = (size_t)tile * 8;
    for (int w = 0; w < 3; w++) k_sweep<<<ntile * nrg, 256, smem, P.stream>>>(c, tile, ntile);
    FLOCK_CK(cudaEventRecord(P.ev[0], P.stream));
    for (int k = 0; k < iters; k++) k_sweep<<<ntile * nrg, 256, smem, P.stream>>>(c, tile, ntile);
    FLOCK_CK(cudaEventRecord(P.ev[1], P.stream));
    FLOCK_CK(cudaEventSynchronize(P.ev[1]));
    float ms = 0;
    cudaEventElapsedTime(&ms, P.ev[0], P.ev[1]);
    *avg_ms = ms / iters;
    if (tile_out) *tile_out = tile;
    return FLOCK_OK;
}

// -------------------------------------------------------- batched solver ---
static const int kBucketEdges[] = {64, 128, 256, 512, 1024, 2048, 4096, 1 << 30};
static const int kNumBuckets = 8;

static int bucket_of(int V) {
    int b = 0;
    while (V > kBucketEdges[b]) b++;
    return b;
}

struct TuneCfg { int threads; int smem; };

static std::mutex g_tune_mu;
static TuneCfg g_tuned[kNumBuckets];
static bool g_tuned_ok[kNumBuckets];

static size_t batch_smem_bytes(int maxV, int maxM) {
    Ctx probe;
    size_t sb = 0;
    carve_ctx(probe, nullptr, maxV, maxM, (unsigned char*)16, nullptr, &sb, nullptr);
    return (sb + 15) & ~size_t(15);
}
static size_t batch_global_bytes(int maxV, int maxM, bool smem) {
    Ctx probe;
    size_t gb = 0;
    carve_ctx(probe, nullptr, maxV, maxM, smem ? (unsigned char*)16 : nullptr, (int64_t*)16, nullptr, &gb);
    return al256(gb);
}

static TuneCfg heuristic_cfg(int maxV, int maxM) {
    TuneCfg t;
    t.threads = maxV <= 256 ? 128 : (maxV <= 1024 ? 256 : 512);
    t.smem = batch_smem_bytes(maxV, maxM) <= 100 * 1024 ? 1 : 0;
    return t;
}

struct BatchRunner {
    DevBuf d_cost, d_sd, d_desc, d_out, d_bfs, d_pot, d_sc, d_next, d_scratch;
    HostBuf h_cost, h_sd, h_desc, h_out, h_bfs, h_pot, h_sc;
    cudaStream_t st[kNumBuckets] = {};
    cudaEvent_t ev_start = nullptr, ev_done = nullptr;
    bool init = false;
    // per call
    int count = 0;
    std::vector<int> V_of, m_of, n_of;
    std::vector<int64_t> out_off, pot_off;
    int64_t total_cells = 0, total_pot = 0, total_cost = 0, total_sd = 0;
    std::vector<BatchDesc> descs;           // grouped by bucket
    int bstart[kNumBuckets + 1] = {};
    int bmaxV[kNumBuckets] = {}, bmaxM[kNumBuckets] = {};
    flock_options opt;

    int setup() {
        if (init) return FLOCK_OK;
        for (auto& s : st) FLOCK_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        FLOCK_CK(cudaEventCreate(&ev_start));
        FLOCK_CK(cudaEventCreate(&ev_done));
        FLOCK_CK(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
        FLOCK_CK(d_next.ensure(kNumBuckets * sizeof(int32_t) * 32));
        init = true;
        return FLOCK_OK;
    }

    // Validate and stage the instances into pinned host memory.
    int prepare(int cnt, const flock_instance* insts, const flock_options* opt_in) {
        int rc = setup();
        if (rc) return rc;
        flock_default_options(&opt);
        if (opt_in) opt = *opt_in;
        count = cnt;
        V_of.assign(cnt, 0); m_of.assign(cnt, 0); n_of.assign(cnt, 0);
        out_off.assign(cnt, 0); pot_off.assign(cnt, 0);
        total_cells = total_pot = total_cost = total_sd = 0;
        std::vector<int64_t> cost_off(cnt), sd_off(cnt);
        for (int k = 0; k < cnt; k++) {
            if ((rc = validate_instance(&insts[k]))) return rc;
            const int m = insts[k].m, n = insts[k].n;
            m_of[k] = m; n_of[k] = n; V_of[k] = m + n;
            const int ldc = (n + 3) & ~3;
            cost_off[k] = total_cost; total_cost += (int64_t)m * ldc;
            sd_off[k] = total_sd; total_sd += m + n;
            out_off[k] = total_cells; total_cells += m + n - 1;
            pot_off[k] = total_pot; total_pot += m + n;
        }
        FLOCK_CK(h_cost.ensure((size_t)total_cost * 4 + 16));
        FLOCK_CK(h_sd.ensure((size_t)total_sd * 4 + 16));
        for (int k = 0; k < cnt; k++) {
            const int m = m_of[k], n = n_of[k], ldc = (n + 3) & ~3;
            int32_t* dst = h_cost.as<int32_t>() + cost_off[k];
            if (ldc == n) memcpy(dst, insts[k].cost, (size_t)m * n * 4);
            else for (int i = 0; i < m; i++) {
                memcpy(dst + (size_t)i * ldc, insts[k].cost + (size_t)i * n, (size_t)n * 4);
                memset(dst + (size_t)i * ldc + n, 0, (size_t)(ldc - n) * 4);
            }
            memcpy(h_sd.as<int32_t>() + sd_off[k], insts[k].supply, (size_t)m * 4);
            memcpy(h_sd.as<int32_t>() + sd_off[k] + m, insts[k].demand, (size_t)n * 4);
        }
        // bucket, largest first inside each bucket
        std::vector<int> order(cnt);
        for (int k = 0; k < cnt; k++) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            const int ba = bucket_of(V_of[a]), bb = bucket_of(V_of[b]);
            if (ba != bb) return ba < bb;
            return (int64_t)m_of[a] * n_of[a] > (int64_t)m_of[b] * n_of[b];
        });
        descs.resize(cnt);
        for (int b = 0; b <= kNumBuckets; b++) bstart[b] = 0;
        for (int b = 0; b < kNumBuckets; b++) { bmaxV[b] = 0; bmaxM[b] = 0; }
        for (int q = 0; q < cnt; q++) {
            const int k = order[q];
            BatchDesc d;
            d.m = m_of[k]; d.n = n_of[k]; d.ldc = (n_of[k] + 3) & ~3; d.index = k;
            d.cost_off = cost_off[k]; d.sd_off = sd_off[k]; d.out_off = out_off[k]; d.pot_off = pot_off[k];
            descs[q] = d;
            const int b = bucket_of(V_of[k]);
            bstart[b + 1]++;
            bmaxV[b] = std::max(bmaxV[b], V_of[k]);
            bmaxM[b] = std::max(bmaxM[b], m_of[k]);
        }
        for (int b = 0; b < kNumBuckets; b++) bstart[b + 1] += bstart[b];
        return FLOCK_OK;
    }

    int ensure_device() {
        FLOCK_CK(d_cost.ensure((size_t)total_cost * 4 + 16));
        FLOCK_CK(d_sd.ensure((size_t)total_sd * 4 + 16));
        FLOCK_CK(d_desc.ensure((size_t)count * sizeof(BatchDesc)));
        FLOCK_CK(d_out.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(d_bfs.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(d_pot.ensure((size_t)total_pot * 8 + 16));
        FLOCK_CK(d_sc.ensure((size_t)count * sizeof(Scalars)));
        FLOCK_CK(h_desc.ensure((size_t)count * sizeof(BatchDesc)));
        FLOCK_CK(h_out.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(h_bfs.ensure((size_t)total_cells * 12 + 16));
        FLOCK_CK(h_pot.ensure((size_t)total_pot * 8 + 16));
        FLOCK_CK(h_sc.ensure((size_t)count * sizeof(Scalars)));
        memcpy(h_desc.p, descs.data(), (size_t)count * sizeof(BatchDesc));
        return FLOCK_OK;
    }

    TuneCfg cfg_for(int b) {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (g_tuned_ok[b]) {
            TuneCfg t = g_tuned[b];
            if (t.smem && batch_smem_bytes(bmaxV[b], bmaxM[b]) > 200 * 1024) t.smem = 0;
            return t;
        }
        return heuristic_cfg(bmaxV[b], bmaxM[b]);
    }

    // Launch the bucket [q0, q1) of descs on stream s with config t.
    int launch_bucket(int b, int q0, int q1, TuneCfg t, cudaStream_t s, int32_t* next) {
        if (q1 <= q0) return FLOCK_OK;
        const int maxV = bmaxV[b], maxM = bmaxM[b];
        const size_t smem = t.smem ? batch_smem_bytes(maxV, maxM) : 0;
        int per_sm = 0;
        FLOCK_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, t.threads, smem));
        if (per_sm < 1) per_sm = 1;
        const int grid = std::max(1, std::min(q1 - q0, per_sm * num_sms()));
        const size_t per_cta = batch_global_bytes(maxV, maxM, t.smem != 0);
        (void)b;
        BatchArgs a;
        a.desc = d_desc.as<BatchDesc>() + q0;
        a.count = q1 - q0;
        a.next = next;
        a.cost = d_cost.as<int32_t>();
        a.sd = d_sd.as<int32_t>();
        a.out_src = d_out.as<int32_t>();
        a.out_dst = d_out.as<int32_t>() + total_cells;
        a.out_qty = d_out.as<int32_t>() + 2 * total_cells;
        a.bfs_out = d_bfs.as<int32_t>();
        a.pot_out = d_pot.as<int64_t>();
        a.sc = d_sc.as<Scalars>();
        a.scratch_per_cta = per_cta;
        a.maxV = maxV; a.maxM = maxM;
        a.smem_mode = t.smem;
        a.bfs_method = opt.bfs_method == FLOCK_BFS_NWC ? FLOCK_BFS_NWC : FLOCK_BFS_VOGEL;
        a.mode = opt.pivot_method == FLOCK_PIVOT_SEQUENTIAL ? 0 : 1;
        a.max_rounds = opt.max_iterations > 0 ? opt.max_iterations : (1 << 30);
        a.scratch = nullptr;
        // scratch: one region per concurrent bucket launch, carved from d_scratch
        a.scratch = scratch_base[b];
        FLOCK_CK(cudaMemsetAsync(next, 0, sizeof(int32_t), s));
        k_batch<<<grid, t.threads, smem, s>>>(a);
        FLOCK_CK(cudaGetLastError());
        return FLOCK_OK;
    }

    uint8_t* scratch_base[kNumBuckets] = {};

    int reserve_scratch(const TuneCfg* cfg) {
        size_t total = 0;
        size_t offs[kNumBuckets];
        for (int b = 0; b < kNumBuckets; b++) {
            offs[b] = total;
            const int nb = bstart[b + 1] - bstart[b];
            if (!nb) continue;
            const size_t smem = cfg[b].smem ? batch_smem_bytes(bmaxV[b], bmaxM[b]) : 0;
            int per_sm = 0;
            FLOCK_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, cfg[b].threads, smem));
            if (per_sm < 1) per_sm = 1;
            const int grid = std::max(1, std::min(nb, per_sm * num_sms()));
            total += al256((size_t)grid * batch_global_bytes(bmaxV[b], bmaxM[b], cfg[b].smem != 0));
        }
        FLOCK_CK(d_scratch.ensure(total + 256));
        for (int b = 0; b < kNumBuckets; b++) scratch_base[b] = d_scratch.as<uint8_t>() + offs[b];
        return FLOCK_OK;
    }

    // H2D, all buckets concurrently, D2H.  Asynchronous; wait() to finish.
    int launch() {
        int rc = ensure_device();
        if (rc) return rc;
        TuneCfg cfg[kNumBuckets];
        for (int b = 0; b < kNumBuckets; b++) cfg[b] = cfg_for(b);
        if ((rc = reserve_scratch(cfg))) return rc;
        cudaStream_t s0 = st[0];
        FLOCK_CK(cudaEventRecord(ev_start, s0));
        FLOCK_CK(cudaMemcpyAsync(d_cost.p, h_cost.p, (size_t)total_cost * 4, cudaMemcpyHostToDevice, s0));
        FLOCK_CK(cudaMemcpyAsync(d_sd.p, h_sd.p, (size_t)total_sd * 4, cudaMemcpyHostToDevice, s0));
        FLOCK_CK(cudaMemcpyAsync(d_desc.p, h_desc.p, (size_t)count * sizeof(BatchDesc), cudaMemcpyHostToDevice, s0));
        FLOCK_CK(cudaEventRecord(ev_done, s0));
        for (int b = 1; b < kNumBuckets; b++) FLOCK_CK(cudaStreamWaitEvent(st[b], ev_done, 0));
        for (int b = 0; b < kNumBuckets; b++)
            if ((rc = launch_bucket(b, bstart[b], bstart[b + 1], cfg[b], st[b], d_next.as<int32_t>() + 32 * b))) return rc;
        for (int b = 1; b < kNumBuckets; b++) {
            FLOCK_CK(cudaEventRecord(ev_done, st[b]));
            FLOCK_CK(cudaStreamWaitEvent(s0, ev_done, 0));
        }
        FLOCK_CK(cudaMemcpyAsync(h_out.p, d_out.p, (size_t)total_cells * 12, cudaMemcpyDeviceToHost, s0));
        FLOCK_CK(cudaMemcpyAsync(h_sc.p, d_sc.p, (size_t)count * sizeof(Scalars), cudaMemcpyDeviceToHost, s0));
        FLOCK_CK(cudaEventRecord(ev_done, s0));
        return FLOCK_OK;
    }

    int wait() {
        FLOCK_CK(cudaEventSynchronize(ev_done));
        return FLOCK_OK;
    }
    bool ready() { return cudaEventQuery(ev_done) == cudaSuccess; }

    // Device-resident inputs only: rerun the kernels on what is already staged.
    int rerun_device_only(float* ms) {
        TuneCfg cfg[kNumBuckets];
        for (int b = 0; b < kNumBuckets; b++) cfg[b] = cfg_for(b);
        int rc = reserve_scratch(cfg);
        if (rc) return rc;
        cudaStream_t s0 = st[0];
        FLOCK_CK(cudaEventRecord(ev_start, s0));
        for (int b = 1; b < kNumBuckets; b++) FLOCK_CK(cudaStreamWaitEvent(st[b], ev_start, 0));
        for (int b = 0; b < kNumBuckets; b++)
            if ((rc = launch_bucket(b, bstart[b], bstart[b + 1], cfg[b], st[b], d_next.as<int32_t>() + 32 * b))) return rc;
        for (int b = 1; b < kNumBuckets; b++) {
            FLOCK_CK(cudaEventRecord(ev_done, st[b]));
            FLOCK_CK(cudaStreamWaitEvent(s0, ev_done, 0));
        }
        FLOCK_CK(cudaEventRecord(ev_done, s0));
        FLOCK_CK(cudaEventSynchronize(ev_done));
        if (ms) cudaEventElapsedTime(ms, ev_start, ev_done);
        return FLOCK_OK;
    }

    void collect(int k, flock_flow* flows, flock_stats* st_out) const {
        const Scalars& S = h_sc.as<Scalars>()[k];
        const int V = V_of[k];
        const int32_t* src = h_out.as<int32_t>() + out_off[k];
        const int32_t* dst = src + total_cells;
        const int32_t* qty = src + 2 * total_cells;
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
        }
    }

    // Autotune every bucket with enough instances: each candidate config
    // solves the bucket once (inputs already on the device); fastest wins.
    int autotune() {
        int rc = ensure_device();
        if (rc) return rc;
        cudaStream_t s0 = st[0];
        FLOCK_CK(cudaMemcpyAsync(d_cost.p, h_cost.p, (size_t)total_cost * 4, cudaMemcpyHostToDevice, s0));
        FLOCK_CK(cudaMemcpyAsync(d_sd.p, h_sd.p, (size_t)total_sd * 4, cudaMemcpyHostToDevice, s0));
        FLOCK_CK(cudaMemcpyAsync(d_desc.p, h_desc.p, (size_t)count * sizeof(BatchDesc), cudaMemcpyHostToDevice, s0));
        FLOCK_CK(cudaStreamSynchronize(s0));
        for (int b = 0; b < kNumBuckets; b++) {
            const int nb = bstart[b + 1] - bstart[b];
            {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                if (g_tuned_ok[b] || nb < 16) continue;
            }
            const int threads_opts[3] = {128, 256, 512};
            float best_ms = 1e30f;
            TuneCfg best = heuristic_cfg(bmaxV[b], bmaxM[b]);
            for (int ti = 0; ti < 3; ti++) {
                for (int sm = 1; sm >= 0; sm--) {
                    TuneCfg t{threads_opts[ti], sm};
                    if (sm && batch_smem_bytes(bmaxV[b], bmaxM[b]) > 200 * 1024) continue;
                    TuneCfg cfg[kNumBuckets];
                    for (int x = 0; x < kNumBuckets; x++) cfg[x] = t;
                    if ((rc = reserve_scratch(cfg))) return rc;
                    FLOCK_CK(cudaEventRecord(ev_start, s0));
                    if ((rc = launch_bucket(b, bstart[b], bstart[b + 1], t, s0, d_next.as<int32_t>() + 32 * b))) return rc;
                    FLOCK_CK(cudaEventRecord(ev_done, s0));
                    FLOCK_CK(cudaEventSynchronize(ev_done));
                    float ms = 0;
                    cudaEventElapsedTime(&ms, ev_start, ev_done);
                    if (ms < best_ms) { best_ms = ms; best = t; }
                }
            }
            std::lock_guard<std::mutex> lk(g_tune_mu);
            g_tuned[b] = best;
            g_tuned_ok[b] = true;
        }
        return FLOCK_OK;
    }
};

BatchRunner* batch_runner_new() { return new BatchRunner(); }
void batch_runner_free(BatchRunner* r) { delete r; }
int batch_runner_prepare(BatchRunner* r, int cnt, const flock_instance* insts, const flock_options* o) { return r->prepare(cnt, insts, o); }
int batch_runner_launch(BatchRunner* r) { return r->launch(); }
int batch_runner_wait(BatchRunner* r) { return r->wait(); }
bool batch_runner_ready(BatchRunner* r) { return r->ready(); }
void batch_runner_collect(BatchRunner* r, int k, flock_flow* flows, flock_stats* st) { r->collect(k, flows, st); }
int batch_runner_count(BatchRunner* r) { return r->count; }

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
    const char* at = getenv("FLOCK_AUTOTUNE");
    if (!at || strcmp(at, "0") != 0) { if ((rc = R.autotune())) return rc; }
    if ((rc = R.launch())) return rc;
    if ((rc = R.wait())) return rc;
    float ms = 0;
    cudaEventElapsedTime(&ms, R.ev_start, R.ev_done);
    int worst = FLOCK_OK;
    int64_t off = 0;
    for (int k = 0; k < cnt; k++) {
        flock_flow* f = flows ? flows + (flow_offset ? flow_offset[k] : off) : nullptr;
        off += R.V_of[k] - 1;
        flock_stats s;
        R.collect(k, f, &s);
        s.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        s.ms_simplex = ms;
        if (stats) stats[k] = s;
        if (s.status) worst = FLOCK_ERR_NOT_OPTIMAL;
    }
    return worst;
}

// Device-only timing hook for the benchmark: solve the last staged batch
// again with its inputs already resident.  Returns the kernel time in ms.
int batch_rerun_device(float* ms) {
    std::lock_guard<std::mutex> lk(g_batch_mu);
    if (!g_batch) return FLOCK_ERR_ARG;
    return g_batch->rerun_device_only(ms);
}

}  // namespace flock

// ================================================================ C ABI ===
extern "C" {

void flock_default_options(flock_options* opt) {
    if (!opt) return;
    opt->bfs_method = FLOCK_BFS_VOGEL;
    opt->pivot_method = FLOCK_PIVOT_PARALLEL;
    opt->max_iterations = 0;
    opt->verify = 1;
}

const char* flock_last_error(void) { return flock::g_err.c_str(); }
const char* flock_version(void) { return "flock-gb300 0.1 (sm_103a)"; }

int flock_vogel(const flock_instance* inst, flock_flow* flows, int32_t* events) {
    if (!flows) return FLOCK_ERR_ARG;
    return flock::vogel_plain(inst, flows, events);
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
int flock_bench_batch_rerun(float* ms) { return flock::batch_rerun_device(ms); }

/* Benchmark hook: average device time of the fused reduced-cost sweep on an
 * m x n matrix (random costs and duals, inputs resident). */
int flock_bench_sweep(int32_t m, int32_t n, int32_t iters, float* avg_ms, int32_t* tile) {
    return flock::bench_sweep(m, n, iters, avg_ms, tile);
}

}  // extern "C"
