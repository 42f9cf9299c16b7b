// emu_check.cpp -- executes the device-side solve sequence of one instance on
// an emulated CTA (cuda_emu.h) with every working array in its own heap
// allocation, so that AddressSanitizer reports any out-of-bounds access of the
// device logic.  Instances come from the library's generator.
//   emu_check <seed> <count> <lo> <hi> <first> <last> [mode] [pricing: 0 full, 1 partial, 2 partial + row keys
//   scrambled between rounds]
// Environment: EMU_THREADS (block size, a multiple of 32, default 32),
// EMU_VERIFY (1, default: after every single pivot the incrementally updated
// depths, duals, int32 duals and preorder intervals are checked against a full
// rebuild), EMU_COST_HI / EMU_QTY_LO / EMU_QTY_HI (generator ranges; small
// ranges give ties and degenerate bases), EMU_PP_ROWS / EMU_PP_REFRESH
// (partial pricing settings, default 64 and 32), EMU_FILE (solve the
// instance of that binary instance file instead).
#define FLOCK_EMU
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <vector>

#include "../simplex.cuh"
#include "../../../include/flock.h"

using namespace flock;

template <class T> static T* arr(std::vector<std::unique_ptr<char[]>>& keep, size_t n) {
    keep.emplace_back(new char[n * sizeof(T) + 1]);
    return (T*)keep.back().get();
}

static int verify = 1;

// The tree's derived state as the single pivot leaves it.
struct TreeState {
    std::vector<int32_t> depth, v32;
    std::vector<int64_t> pot;
    std::vector<int2> iv;
    int32_t ivp = 0, nwide = 0, narrow = 0;
};

static void save_tree(const Ctx& c, int V, TreeState& t) {
    t.depth.assign(c.depth, c.depth + V);
    t.pot.assign(c.pot, c.pot + V);
    t.v32.assign(c.v32, c.v32 + c.I.n);
    t.iv.assign(c.iv, c.iv + 2 * (size_t)V);
    t.ivp = c.sc->ivp; t.nwide = c.sc->nwide; t.narrow = c.sc->narrow;
}

static void restore_tree(const Ctx& c, int V, const TreeState& t) {
    memcpy(c.depth, t.depth.data(), 4 * (size_t)V);
    memcpy(c.pot, t.pot.data(), 8 * (size_t)V);
    memcpy(c.v32, t.v32.data(), 4 * (size_t)c.I.n);
    memcpy(c.iv, t.iv.data(), sizeof(int2) * 2 * (size_t)V);
    c.sc->ivp = t.ivp; c.sc->nwide = t.nwide; c.sc->narrow = t.narrow;
}

// Compare the incremental state `t` with the rebuilt one in `c`: depths,
// duals, int32 duals and the wide count exactly; intervals by their meaning
// (any preorder is valid): sizes equal, preorder numbers a permutation of
// 0..alive-1, every vertex's number inside its parent's interval.
static void check_incremental(const Ctx& c, int V, const TreeState& t, int* errors) {
    auto bad = [&](const char* what, int v, long long a, long long b) {
        if ((*errors)++ < 8) fprintf(stderr, "  %s at vertex %d: incremental %lld, rebuilt %lld\n", what, v, a, b);
    };
    const int m = c.I.m;
    const int2* inc = t.iv.data() + (t.ivp ? V : 0);
    const int2* reb = c.iv + (c.sc->ivp ? V : 0);
    std::vector<int> seen(V, 0);
    int alive = 0;
    for (int v = 0; v < V; v++) {
        if (c.parent[v] == -2) continue;
        alive++;
        if (t.depth[v] != c.depth[v]) bad("depth", v, t.depth[v], c.depth[v]);
        if (t.pot[v] != c.pot[v]) bad("dual", v, t.pot[v], c.pot[v]);
        if (v >= m && t.v32[v - m] != c.v32[v - m]) bad("int32 dual", v, t.v32[v - m], c.v32[v - m]);
        if (inc[v].y != reb[v].y) bad("subtree size", v, inc[v].y, reb[v].y);
        if (inc[v].x < 0 || inc[v].x >= V || seen[inc[v].x]++) bad("preorder number", v, inc[v].x, reb[v].x);
        const int p = c.parent[v];
        if (p >= 0 && (inc[v].x == inc[p].x || !iv_in(inc[p], inc[v].x))) bad("interval nesting", v, inc[v].x, inc[p].x);
    }
    for (int v = 0; v < V; v++)
        if (c.parent[v] != -2 && inc[v].x >= alive) bad("preorder range", v, inc[v].x, alive);
    if (t.nwide != c.sc->nwide) bad("wide count", -1, t.nwide, c.sc->nwide);
    if (t.narrow != c.sc->narrow) bad("narrow flag", -1, t.narrow, c.sc->narrow);
}

static int solve_one(int m, int n, const int32_t* s, const int32_t* d, const int32_t* cost, int mode, int pricing,
                     Scalars* out) {
    std::vector<std::unique_ptr<char[]>> keep;
    const int V = m + n, ldc = (n + 3) & ~3;
    int32_t* C = arr<int32_t>(keep, (size_t)m * ldc);
    for (int i = 0; i < m; i++) {
        memcpy(C + (size_t)i * ldc, cost + (size_t)i * n, (size_t)n * 4);
        for (int j = n; j < ldc; j++) C[(size_t)i * ldc + j] = 0;
    }
    Ctx c;
    c.I.m = m; c.I.n = n; c.I.ldc = ldc; c.I.cost = C; c.I.supply = s; c.I.demand = d;
    Scalars* sc = arr<Scalars>(keep, 1);
    memset(sc, 0, sizeof(Scalars));
    sc->mode = mode;
    sc->pricing = pricing ? 1 : 0;
    sc->pp_rows = getenv("EMU_PP_ROWS") ? atoi(getenv("EMU_PP_ROWS")) : kPPRowsLarge;
    sc->pp_refresh = getenv("EMU_PP_REFRESH") ? atoi(getenv("EMU_PP_REFRESH")) : kPPRefreshLarge;
    sc->max_rounds = 1 << 30;
    c.sc = sc;
    c.bfs_src = arr<int32_t>(keep, V); c.bfs_dst = arr<int32_t>(keep, V); c.bfs_qty = arr<int32_t>(keep, V);
    c.out_src = arr<int32_t>(keep, V); c.out_dst = arr<int32_t>(keep, V); c.out_qty = arr<int32_t>(keep, V);
    c.parent = arr<int32_t>(keep, V); c.flow = arr<int64_t>(keep, V); c.depth = arr<int32_t>(keep, V);
    c.pot = arr<int64_t>(keep, V);
    c.v32 = arr<int32_t>(keep, V);
    c.prow = arr<int32_t>(keep, kPPRows);
    c.iv = arr<int2>(keep, 2 * (size_t)V);
    set_jump(c, arr<int64_t>(keep, jump_bytes(V) / 8), V);
    c.path = c.len1; c.pflow = c.acc1;
    c.side = arr<uint8_t>(keep, V);
    c.row_best = arr<uint64_t>(keep, m); c.claim = arr<uint64_t>(keep, V);
    c.cand = arr<int32_t>(keep, m); c.cand_theta = arr<int64_t>(keep, m);
    c.cand_q = arr<int32_t>(keep, m); c.cand_info = arr<int32_t>(keep, m);
    c.covered = arr<uint8_t>(keep, V); c.diff = arr<int32_t>(keep, V); c.res = arr<int32_t>(keep, V);
    c.top2 = arr<int4>(keep, V); c.rescan = arr<int32_t>(keep, V);
    c.bsum = arr<int64_t>(keep, V); c.csr_start = arr<int32_t>(keep, V + 1);
    c.csr_adj = arr<int32_t>(keep, 2 * V); c.order = arr<int32_t>(keep, V); c.uf = arr<int32_t>(keep, V);
    c.ph = nullptr;
    BlockScratch bs;
    TreeState saved;
    int inc_errors = 0;
    const int mism = emu::run_cta([&] {
        vogel_cta(c, bs);
        if (threadIdx.x == 0 && c.sc->events < 0) c.sc->status |= ST_VOGEL_UNDEF;
        __syncthreads();
        sf_init_cta(c, bs);
        if (!c.sc->done) tree_build_cta(c, bs);
        uint64_t junk = 0x9E3779B97F4A7C15ull;
        for (;;) {
            if (c.sc->done) break;
            if (c.sc->stale) tree_build_cta(c, bs);
            if (c.sc->done) break;
            // pricing 2: row keys do not survive between rounds (as in the
            // round form, which stages them afresh): fill them with garbage
            if (pricing == 2 && threadIdx.x == 0)
                for (int i = 0; i < m; i++) { junk = junk * 6364136223846793005ull + 1442695040888963407ull; c.row_best[i] = junk; }
            __syncthreads();
            uint64_t entering = kNoKey;
            const bool partial = c.sc->pricing != 0;
            if (partial) entering = sweep_partial_cta(c, bs);
            else sweep_cta(c);
            pivot_round_cta<kJump, true>(c, bs, partial, entering);
            if (threadIdx.x == 0) c.sc->rounds++;
            __syncthreads();
            if (c.sc->done) break;
            if (verify && !c.sc->stale) {
                if (threadIdx.x == 0) save_tree(c, V, saved);
                __syncthreads();
                tree_build_cta(c, bs);
                if (threadIdx.x == 0) {
                    check_incremental(c, V, saved, &inc_errors);
                    restore_tree(c, V, saved);
                }
                __syncthreads();
                if (inc_errors) break;
            }
        }
        if (!(c.sc->status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE))) {
            finalize_cta(c, bs);
            certify_flows_cta(c, bs);
            certify_cells_cta(c, bs);
        }
    });
    *out = *sc;
    if (inc_errors) {
        fprintf(stderr, "incremental tree state differs from the rebuild (%d errors)\n", inc_errors);
        return mism ? mism : 1;
    }
    return mism;
}

int main(int argc, char** argv) {
    if (argc < 7) { fprintf(stderr, "usage: emu_check seed count lo hi first last [mode]\n"); return 2; }
    const uint64_t seed = strtoull(argv[1], 0, 10);
    const int count = atoi(argv[2]), lo = atoi(argv[3]), hi = atoi(argv[4]);
    const int first = atoi(argv[5]), last = atoi(argv[6]);
    const int mode = argc > 7 ? atoi(argv[7]) : 1;
    const int pricing = argc > 8 ? atoi(argv[8]) : 0;
    std::vector<int32_t> ms(count), ns(count);
    flock_generate_sizes(seed, count, lo, hi, ms.data(), ns.data());
    auto env = [](const char* k, int dflt) { const char* v = getenv(k); return v ? atoi(v) : dflt; };
    blockDim.x = (unsigned)env("EMU_THREADS", 32);
    verify = env("EMU_VERIFY", 1);
    const int cost_hi = env("EMU_COST_HI", 1000), qlo = env("EMU_QTY_LO", 100), qhi = env("EMU_QTY_HI", 1000);
    int bad = 0;
    // EMU_FILE: solve the instance of that binary instance file instead
    if (const char* f = getenv("EMU_FILE")) {
        int32_t m = 0, n = 0;
        if (flock_bin_shape(f, &m, &n)) { fprintf(stderr, "cannot read %s\n", f); return 2; }
        std::vector<int32_t> s(m), d(n), c((size_t)m * n);
        if (flock_read_bin(f, m, n, s.data(), d.data(), c.data())) { fprintf(stderr, "cannot read %s\n", f); return 2; }
        Scalars r;
        const int mism = solve_one(m, n, s.data(), d.data(), c.data(), mode, pricing, &r);
        const bool ok = r.status == 0 && r.cert == 0 && mism == 0;
        printf("%s m=%d n=%d obj=%lld rounds=%d pivots=%d status=%d cert=%d fail_site=%d barrier_mismatch=%d %s\n", f, m,
               n, (long long)r.objective, r.rounds, r.pivots, r.status, r.cert, r.fail_site, mism, ok ? "ok" : "BAD");
        return ok ? 0 : 1;
    }
    for (int k = first; k <= last && k < count; k++) {
        const int m = ms[k], n = ns[k];
        std::vector<int32_t> s(m), d(n), c((size_t)m * n);
        flock_generate(0, seed * 1000003ull + k + 1, m, n, 1, cost_hi, qlo, qhi, s.data(), d.data(), c.data());
        Scalars r;
        const int mism = solve_one(m, n, s.data(), d.data(), c.data(), mode, pricing, &r);
        const bool ok = r.status == 0 && r.cert == 0 && mism == 0;
        if (!ok) bad++;
        printf("k=%d m=%d n=%d obj=%lld rounds=%d pivots=%d status=%d cert=%d fail_site=%d barrier_mismatch=%d %s\n",
               k, m, n, (long long)r.objective, r.rounds, r.pivots, r.status, r.cert, r.fail_site, mism,
               ok ? "ok" : "BAD");
        fflush(stdout);
    }
    printf("bad=%d\n", bad);
    return bad ? 1 : 0;
}

// the batch runner lives in the CUDA translation unit; the emulator links
// only the host helpers (generator), so the server's hooks are stubbed
namespace flock {
struct BatchRunner {};
void set_error(const std::string&) {}
BatchRunner* batch_runner_new() { return nullptr; }
void batch_runner_free(BatchRunner*) {}
int batch_runner_prepare(BatchRunner*, int, const flock_instance*, const flock_options*) { return 1; }
int batch_runner_solve(BatchRunner*) { return 1; }
void batch_runner_collect(BatchRunner*, int, flock_flow*, flock_stats*) {}
}  // namespace flock
extern "C" void flock_default_options(flock_options*) {}
