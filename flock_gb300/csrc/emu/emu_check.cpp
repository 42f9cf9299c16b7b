// emu_check.cpp -- executes the device-side solve sequence of one instance on
// an emulated CTA (cuda_emu.h) with every working array in its own heap
// allocation, so that AddressSanitizer reports any out-of-bounds access of the
// device logic.  Instances come from the library's generator.
//   emu_check <seed> <count> <lo> <hi> <first> <last> [mode] [pricing: 0 full, 1 partial, 2 partial + row keys
//   scrambled between rounds]
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
    sc->max_rounds = 1 << 30;
    c.sc = sc;
    c.bfs_src = arr<int32_t>(keep, V); c.bfs_dst = arr<int32_t>(keep, V); c.bfs_qty = arr<int32_t>(keep, V);
    c.out_src = arr<int32_t>(keep, V); c.out_dst = arr<int32_t>(keep, V); c.out_qty = arr<int32_t>(keep, V);
    c.parent = arr<int32_t>(keep, V); c.flow = arr<int64_t>(keep, V); c.depth = arr<int32_t>(keep, V);
    c.pot = arr<int64_t>(keep, V);
    c.v32 = arr<int32_t>(keep, V);
    c.prow = arr<int32_t>(keep, kPPRows);
    c.lift_cap = lift_levels(V);
    c.lift = arr<int32_t>(keep, (size_t)V * c.lift_cap);
    c.anc0 = arr<int32_t>(keep, V); c.anc1 = arr<int32_t>(keep, V);
    c.len0 = arr<int32_t>(keep, V); c.len1 = arr<int32_t>(keep, V);
    c.acc0 = arr<int64_t>(keep, V); c.acc1 = arr<int64_t>(keep, V);
    c.row_best = arr<uint64_t>(keep, m); c.claim = arr<uint64_t>(keep, V);
    c.cand = arr<int32_t>(keep, m); c.cand_theta = arr<int64_t>(keep, m);
    c.cand_q = arr<int32_t>(keep, m); c.cand_info = arr<int32_t>(keep, m);
    c.covered = arr<uint8_t>(keep, V); c.diff = arr<int32_t>(keep, V); c.res = arr<int32_t>(keep, V);
    c.top2 = arr<int4>(keep, V); c.rescan = arr<int32_t>(keep, V);
    c.bsum = arr<int64_t>(keep, V); c.csr_start = arr<int32_t>(keep, V + 1);
    c.csr_adj = arr<int32_t>(keep, 2 * V); c.order = arr<int32_t>(keep, V); c.uf = arr<int32_t>(keep, V);
    BlockScratch bs;
    const int mism = emu::run_cta([&] {
        vogel_cta(c, bs);
        if (threadIdx.x == 0 && c.sc->events < 0) c.sc->status |= ST_VOGEL_UNDEF;
        __syncthreads();
        sf_init_cta(c, bs);
        if (!c.sc->done) tree_recompute_cta(c, bs);
        uint64_t junk = 0x9E3779B97F4A7C15ull;
        for (;;) {
            if (c.sc->done) break;
            // pricing 2: row keys do not survive between rounds (as in the
            // round form, which stages them afresh): fill them with garbage
            if (pricing == 2 && threadIdx.x == 0)
                for (int i = 0; i < m; i++) { junk = junk * 6364136223846793005ull + 1442695040888963407ull; c.row_best[i] = junk; }
            __syncthreads();
            if (c.sc->pricing) sweep_partial_cta(c, bs);
            else sweep_cta(c);
            pivot_round_cta(c, bs);
            if (threadIdx.x == 0) c.sc->rounds++;
            __syncthreads();
            if (c.sc->done) break;
            tree_recompute_cta(c, bs);
        }
        if (!(c.sc->status & (ST_TREE_CORRUPT | ST_SF_FAIL | ST_RANGE))) {
            finalize_cta(c, bs);
            certify_flows_cta(c, bs);
            certify_cells_cta(c, bs);
        }
    });
    *out = *sc;
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
    int bad = 0;
    for (int k = first; k <= last && k < count; k++) {
        const int m = ms[k], n = ns[k];
        std::vector<int32_t> s(m), d(n), c((size_t)m * n);
        flock_generate(0, seed * 1000003ull + k + 1, m, n, 1, 1000, 100, 1000, s.data(), d.data(), c.data());
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
