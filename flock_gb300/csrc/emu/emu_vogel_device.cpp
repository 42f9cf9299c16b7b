// emu_vogel_device.cpp -- runs the device functions of the "vam_device" Vogel
// variant (book_line_cta for every line, then vogel_books_cta) or, with
// EMU_VOGEL=host / wide, the "vam_host" Vogel (vogel_cta, its staged form /
// its wide-instance form with a column-major copy) on an emulated CTA
// (cuda_emu.h) under AddressSanitizer / UBSan, for the binary instance files
// given as arguments, and prints each allocation list:
//   <file> events=<e> barrier_mismatch=<k> flows=<src>,<dst>,<qty>;...
// The test harness compares the lists with its own expectation.
// Environment: EMU_THREADS (block size, a multiple of 32, default 64).
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

static int run_one(const char* path) {
    int32_t m = 0, n = 0;
    if (flock_bin_shape(path, &m, &n)) { fprintf(stderr, "cannot read %s\n", path); return 2; }
    std::vector<int32_t> s(m), d(n), cost((size_t)m * n);
    if (flock_read_bin(path, m, n, s.data(), d.data(), cost.data())) { fprintf(stderr, "cannot read %s\n", path); return 2; }
    std::vector<std::unique_ptr<char[]>> keep;
    const int V = m + n, ldc = (n + 3) & ~3;
    int32_t* C = arr<int32_t>(keep, (size_t)m * ldc);
    for (int i = 0; i < m; i++) {
        memcpy(C + (size_t)i * ldc, cost.data() + (size_t)i * n, (size_t)n * 4);
        for (int j = n; j < ldc; j++) C[(size_t)i * ldc + j] = 0;
    }
    Ctx c;
    c.I.m = m; c.I.n = n; c.I.ldc = ldc; c.I.cost = C; c.I.supply = s.data(); c.I.demand = d.data();
    Scalars* sc = arr<Scalars>(keep, 1);
    memset(sc, 0, sizeof(Scalars));
    c.sc = sc;
    c.bfs_src = arr<int32_t>(keep, V); c.bfs_dst = arr<int32_t>(keep, V); c.bfs_qty = arr<int32_t>(keep, V);
    c.res = arr<int32_t>(keep, V);
    c.top2 = arr<int4>(keep, V);
    const char* variant = getenv("EMU_VOGEL");
    if (variant && (!strcmp(variant, "host") || !strcmp(variant, "wide"))) {
        c.covered = arr<uint8_t>(keep, V);
        c.diff = arr<int32_t>(keep, V);
        c.rescan = arr<int32_t>(keep, V);
        BlockScratch bs;
        const bool wide = !strcmp(variant, "wide");
        // the wide form's column-major copy (n rows of ceil4(m))
        const int ldcT = (m + 3) & ~3;
        int32_t* T = arr<int32_t>(keep, (size_t)n * ldcT);
        for (int j = 0; j < n; j++)
            for (int i = 0; i < ldcT; i++) T[(size_t)j * ldcT + i] = i < m ? C[(size_t)i * ldc + j] : 0;
        const int r = emu::run_cta([&] {
            if (wide) vogel_cta<true>(c, bs, T);
            else vogel_cta(c, bs);
        });
        const int mism = r ? (r < 0 ? 1000 : r) : 0;
        printf("%s events=%d barrier_mismatch=%d flows=", path, sc->events, mism);
        for (int k = 0; k < V - 1; k++) printf("%d,%d,%d;", c.bfs_src[k], c.bfs_dst[k], c.bfs_qty[k]);
        printf("\n");
        fflush(stdout);
        return mism ? 1 : 0;
    }
    int2* rbook = arr<int2>(keep, (size_t)m * (n + 2));
    int2* cbook = arr<int2>(keep, (size_t)n * (m + 2));
    int P = 1;
    while (P < std::max(m, n) + 2) P <<= 1;
    uint64_t* sk = arr<uint64_t>(keep, P);
    int mism = 0;
    for (int line = 0; line < V; line++) {
        int2* out = line < m ? rbook + (size_t)line * (n + 2) : cbook + (size_t)(line - m) * (m + 2);
        const int r = emu::run_cta([&] { book_line_cta(c.I, line, sk, P, out); });
        if (r) mism += r < 0 ? 1000 : r;
    }
    BlockScratch bs;
    const int r = emu::run_cta([&] { vogel_books_cta(c, rbook, cbook, bs); });
    if (r) mism += r < 0 ? 1000 : r;
    printf("%s events=%d barrier_mismatch=%d flows=", path, sc->events, mism);
    for (int k = 0; k < V - 1; k++) printf("%d,%d,%d;", c.bfs_src[k], c.bfs_dst[k], c.bfs_qty[k]);
    printf("\n");
    fflush(stdout);
    return mism ? 1 : 0;
}

int main(int argc, char** argv) {
    if (argc < 2) { fprintf(stderr, "usage: emu_vogel_device file.fbin...\n"); return 2; }
    const char* t = getenv("EMU_THREADS");
    blockDim.x = (unsigned)(t ? atoi(t) : 64);
    int rc = 0;
    for (int a = 1; a < argc; a++) rc |= run_one(argv[a]);
    return rc;
}

// host.cpp refers to the batch runner of the CUDA translation unit; the
// emulator links only the host helpers, so those hooks are stubbed
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
