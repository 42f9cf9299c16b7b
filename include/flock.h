/*
 * flock.h -- C ABI of flock-gb300, a GB300-native (sm_103a) solver for the
 * balanced transportation problem
 *      min sum c_ij x_ij  s.t.  sum_j x_ij = s_i,  sum_i x_ij = d_j,  x >= 0
 * with the method of researchgroup-zx93920/flock: Vogel's approximation for
 * the initial basic feasible solution, u-v duals on the basis tree, a
 * reduced-cost sweep and stepping-stone pivots (single or deconflicted
 * parallel).  All arithmetic is integer: int32 costs and quantities, int64
 * duals and objective.
 *
 * Conventions: every function returns a flock_status (0 = FLOCK_OK).  The
 * caller owns every host buffer; the library owns device state.  Costs are
 * row-major, cell (i, j) at cost[i * n + j].  Calls are thread-safe (a
 * process-wide lock serialises the plain-path device workspace).
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   flock_read_dat / flock_dat_shape  <- readSize / readCosts, src/instance.cpp:80-141
 *                                        (ProblemInstance, src/structs.h:19-40)
 *   flock_vogel                       <- find_vogel_bfs_sequencial,
 *                                        src/parallel_simplex_method/IBFS_vogel.cu:546-769
 *   flock_vogel_device                <- find_vogel_bfs_parallel,
 *                                        src/parallel_simplex_method/IBFS_vogel.cu:3-543
 *   flock_solve                       <- uvModel_parallel / ssModel_parallel ctor + execute()
 *                                        + create_flows(), src/algos.h:1-4,
 *                                        parallel_uv_method/uv_model_parallel.cu:20-400,
 *                                        parallel_ss_method/ss_model_parallel.cu:128-250
 *   flock_flow                        <- flowInformation, src/structs.h:45-52
 *   flock_options                     <- BFS_METHOD / MAX_ITERATIONS / pivoting switches,
 *                                        src/parallel_simplex_method/parallel_structs.h:34-89
 *   flock_stats                       <- model statistics (objVal, totalIterations,
 *                                        totalSolveTime, ...), uv_model_parallel.h:33-38
 *   flock_batch_solve, flock_server_* <- no counterpart (the reference solves one instance
 *                                        per process); batched and served forms of flock_solve
 */
#ifndef FLOCK_GB300_H
#define FLOCK_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FLOCK_OK = 0,
    FLOCK_ERR_ARG = 1,          /* null pointer, m or n < 1, negative quantity */
    FLOCK_ERR_UNBALANCED = 2,   /* sum of supplies != sum of demands */
    FLOCK_ERR_FILE = 3,         /* file not found / unreadable (reference: FileNotFoundException) */
    FLOCK_ERR_PARSE = 4,        /* malformed .dat content */
    FLOCK_ERR_INEXACT = 5,      /* a cost is not an integer after decimal scaling */
    FLOCK_ERR_RANGE = 6,        /* |cost| > 2^30, or the instance is too large */
    FLOCK_ERR_CUDA = 7,         /* CUDA error (message via flock_last_error) */
    FLOCK_ERR_NOT_OPTIMAL = 8,  /* solve stopped before optimality (see flock_stats.status) */
    FLOCK_ERR_BUDGET = 9,       /* serving: request larger than the memory budget */
    FLOCK_ERR_CAPACITY = 10     /* output buffer too small */
} flock_status;

/* One balanced instance (host memory). */
typedef struct {
    int32_t m, n;               /* supplies (rows), demands (columns) */
    const int32_t* supply;      /* m */
    const int32_t* demand;      /* n */
    const int32_t* cost;        /* m*n, row-major */
} flock_instance;

/* One flow: qty units from supply `source` to demand `destination`. */
typedef struct {
    int32_t source, destination, qty;
} flock_flow;

/* BFS_METHOD nwc_host / vam_host / vam_device.  VOGEL_DEVICE: the reference's
 * device Vogel semantics (flock_vogel_device); flock_solve only (batched and
 * served forms return FLOCK_ERR_ARG), lines of at most 16382 cells. */
enum { FLOCK_BFS_NWC = 0, FLOCK_BFS_VOGEL = 1, FLOCK_BFS_VOGEL_DEVICE = 2 };
/* Pivoting.  SEQUENTIAL (-a parallel_uv): one pivot per round, the most
 * negative reduced cost (Dantzig, row-major first minimum).  PARALLEL: the
 * rows with the most negative keys (at most 32) walk their cycles and the
 * edge-disjoint ones pivot together.  SWITCH (-a switch_hybrid) runs
 * parallel rounds until one applies fewer than 10 pivots, then sequential
 * ones (switch/switch_model_parallel.cu:182-184).  SS (-a parallel_ss,
 * parallel_ss_method/PIVOT_ss.cu:294-571): every cell with a negative cycle
 * cost is a candidate (the most negative ones, at most min(1024, m) per
 * round); they are taken most negative first and a cycle is accepted unless
 * it shares a tree edge with one accepted before it; all accepted cycles
 * pivot in the same round.  SS prices every cell each round (the pricing
 * option is ignored), runs its rounds on one block at every size, and is
 * flock_solve's only (the batched and served forms return FLOCK_ERR_ARG). */
enum { FLOCK_PIVOT_SEQUENTIAL = 0, FLOCK_PIVOT_PARALLEL = 1, FLOCK_PIVOT_SWITCH = 2, FLOCK_PIVOT_SS = 3 };
/* Pricing.  FULL: every round sweeps every cell (the reference's Dantzig rule,
 * uv_model_parallel.cu:151-200).  PARTIAL (the default; no counterpart in the
 * reference): a full sweep keeps the R rows with the most negative reduced
 * costs as candidates and the following rounds re-price only those rows,
 * until they hold no negative reduced cost or K rounds have passed;
 * optimality is only declared after a full sweep.  R / K: 32 / 8 for
 * instances of up to 1024 vertices, 64 / 32 above (batched and served forms,
 * the plain one-launch solve below 2400 vertices), 128 / 64 for the plain
 * solver from 2400 vertices (its grid and cluster rounds).  The optimum is the same; the pivot sequence differs.  FLOCK_PIVOT_SS
 * always prices fully. */
enum { FLOCK_PRICING_FULL = 0, FLOCK_PRICING_PARTIAL = 1 };

typedef struct {
    int32_t bfs_method;      /* FLOCK_BFS_VOGEL (default), FLOCK_BFS_NWC or FLOCK_BFS_VOGEL_DEVICE */
    int32_t pivot_method;    /* FLOCK_PIVOT_SWITCH (default), _PARALLEL, _SEQUENTIAL or _SS */
    int32_t max_iterations;  /* cap on pricing rounds; <= 0: 1 << 30 */
    int32_t verify;          /* nonzero: run the exact certificate check (default on) */
    int32_t pricing;         /* FLOCK_PRICING_PARTIAL (default) or FLOCK_PRICING_FULL */
} flock_options;

/* Failures reported in flock_stats.status (bit set; 0 = optimal). */
enum {
    FLOCK_ST_ITER_CAP = 1,        /* round cap reached before optimality */
    FLOCK_ST_TREE_CORRUPT = 2,    /* internal consistency failure */
    FLOCK_ST_SF_FAIL = 4,         /* internal: start tree not strongly feasible */
    FLOCK_ST_CERT_FAIL = 32,      /* certificate failed */
    FLOCK_ST_RANGE = 64           /* perturbed flows would overflow */
};
/* Notes reported in flock_stats.notes (informational, the result is still optimal). */
enum {
    FLOCK_NOTE_VOGEL_UNDEF = 8,     /* Vogel reached the reference's undefined case */
    FLOCK_NOTE_START_REPAIRED = 16  /* simplex started from the NW corner instead */
};

typedef struct {
    int64_t objective;       /* sum c_ij x_ij (exact) */
    int32_t iterations;      /* pricing rounds (full reduced-cost sweeps) */
    int32_t pivots;          /* pivots applied */
    int32_t active_flows;    /* nonzero flows written to `flows` */
    int32_t status;          /* FLOCK_ST_* failure bits, 0 = optimal */
    int32_t notes;           /* FLOCK_NOTE_* bits; bits 8+: internal check site on failure */
    int32_t certified;       /* 1: certificate checked and passed */
    int32_t vogel_events;    /* Vogel steps whose line had no uncovered cell; -1 undefined */
    double ms_total;         /* wall time of the call (ms) */
    double ms_bfs;           /* device time of the initial solution (Vogel or NW corner) */
    double ms_simplex;       /* device time of the start tree and the pivot loop */
    /* Device time per simplex phase (ms), the reference's model statistics
     * (uv_time, reduced_cost_time, pivot_time, cycle_discovery_time,
     * resolve_time, adjustment_time; uv_model_parallel.cu:301-341).  Set by
     * the plain solver (flock_solve, and the instances of more than 4096
     * vertices that the batched and served forms hand to it); 0 otherwise.
     *   ms_dual:    the strongly feasible start tree, rebuilds of the tree's
     *               duals, depths and intervals (at the start and after a
     *               round that applied several pivots; a single pivot
     *               updates the duals in place, inside ms_adjust)
     *   ms_sweep:   reduced-cost sweeps and the choice of the entering cells
     *   ms_cycle:   cycle discovery (tree paths of the entering cells)
     *   ms_resolve: deconfliction of the candidates of a parallel round
     *   ms_adjust:  leaving edge, flow change and the in-place tree update
     *   ms_pivot = ms_cycle + ms_resolve + ms_adjust.
     * Launch gaps count toward the phase before them, so ms_dual + ms_sweep
     * + ms_pivot is close to ms_simplex. */
    double ms_dual, ms_sweep, ms_pivot, ms_cycle, ms_resolve, ms_adjust;
} flock_stats;

void flock_default_options(flock_options* opt);
const char* flock_last_error(void);
const char* flock_version(void);

/* .dat reader.  Format: "m n", m supplies, n demands, m*n costs (row-major),
 * whitespace separated (src/instance.cpp:96-141).  Costs are decimal text and
 * are multiplied by 10^decimal_scale exactly (FLOCK_ERR_INEXACT otherwise).
 * flock_dat_scale reports the smallest scale making every cost integral. */
int flock_dat_shape(const char* path, int32_t* m, int32_t* n);
int flock_dat_scale(const char* path, int32_t* scale);
int flock_read_dat(const char* path, int32_t decimal_scale, int32_t m, int32_t n,
                   int32_t* supply, int32_t* demand, int32_t* cost);

/* .dat writer in the reference's file layout (its data/ files): "m n", the
 * supplies and the demands on one line each (a tab after every value), then
 * one cost per line as cost / 10^decimal_scale (0..9), trailing zeros trimmed.
 * flock_read_dat with the same scale returns the same integers. */
int flock_write_dat(const char* path, const flock_instance* inst, int32_t decimal_scale);

/* Binary instance file (no counterpart in the reference; for large instances,
 * where the text format's parse dominates): "FLKBIN01", int32 m, int32 n, then
 * m supplies, n demands and m*n costs as int32 little-endian, costs row-major.
 * The costs are stored as the solver takes them (no decimal scaling); reading
 * returns them unchecked (flock_solve validates). */
int flock_write_bin(const char* path, const flock_instance* inst);
int flock_bin_shape(const char* path, int32_t* m, int32_t* n);
int flock_read_bin(const char* path, int32_t m, int32_t n, int32_t* supply, int32_t* demand, int32_t* cost);

/* Vogel's approximation on the GPU with the reference's exact semantics.
 * Writes m+n-1 allocations in allocation order.  *events as flock_stats.
 * FLOCK_ERR_CUDA for a CUDA failure or a failed internal device check. */
int flock_vogel(const flock_instance* inst, flock_flow* flows, int32_t* events);

/* Vogel's approximation with the semantics of the reference's device variant
 * (find_vogel_bfs_parallel, BFS_METHOD "vam_device",
 * src/parallel_simplex_method/IBFS_vogel.cu:3-543): regrets from positions
 * into cost-sorted per-line books, the first largest regret; a different BFS
 * from flock_vogel.  Writes m+n-1 allocations in allocation order.  *events:
 * 0, or -1 where the reference indexes past its arrays (costs at or above its
 * 32767 sentinels); its allocations from there on are written as (-1, -1, 0).
 * FLOCK_ERR_RANGE for a line of more than 16382 cells. */
int flock_vogel_device(const flock_instance* inst, flock_flow* flows, int32_t* events);

/* No counterpart in the reference.  flock_vogel without any allocation:
 * the same kernel and the same allocation list and event count, but every
 * device array of the call lives in one static 6 MiB __device__ array per
 * device, so the call makes no cudaMalloc/cudaFree, allocates no pinned host
 * memory and creates no stream or event itself.  It is for callers that
 * cannot allocate: a process whose device memory is already reserved by
 * another allocator (a caching allocator or a fixed serving budget holding
 * the device), where cudaMalloc fails or takes memory promised elsewhere; and
 * latency-bound callers on a busy device, where cudaFree's implicit
 * device-wide synchronisation would stall other streams.
 * Limits: m + n <= FLOCK_VOGEL_STATIC_MAX_V and m * ceil4(n) <=
 * FLOCK_VOGEL_STATIC_MAX_CELLS; larger instances return FLOCK_ERR_RANGE
 * (message via flock_last_error) before any CUDA call.
 * The first call on a device does the set-up (cudaGetSymbolAddress of the
 * scratch array, cached per device and context under a per-device lock) and
 * should come before any stream capture.  Work runs on the calling thread's
 * per-thread default stream (cudaStreamPerThread, which the runtime creates
 * on the thread's first use; it does not synchronise with the legacy default
 * stream), and the call returns after synchronising it.  Calls that overlap
 * in time on one device share the scratch and race: callers serialise them.
 * Errors as flock_vogel: argument and range errors before any CUDA call,
 * FLOCK_ERR_CUDA for a CUDA failure or a failed internal device check. */
#define FLOCK_VOGEL_STATIC_MAX_V 8192
#define FLOCK_VOGEL_STATIC_MAX_CELLS 1048576
int flock_vogel_static(const flock_instance* inst, flock_flow* flows, int32_t* events);

/* Solve one instance on the GPU.  `flows` has room for m+n-1 entries; the
 * nonzero flows are written first (stats->active_flows of them), then the
 * zero-flow basic cells, so flows[0..m+n-2] is always the full basis.
 * duals_u (m) and duals_v (n) are optional (NULL): the optimal duals with
 * c_ij - u_i - v_j >= 0 everywhere and = 0 on the basis.
 * Returns FLOCK_ERR_NOT_OPTIMAL when stats->status != 0. */
int flock_solve(const flock_instance* inst, const flock_options* opt, flock_flow* flows,
                int64_t* duals_u, int64_t* duals_v, flock_stats* stats);

/* Batched form: `count` independent instances solved by one persistent kernel
 * family (one CTA per instance, work stealing, size buckets).  Flows of
 * instance k start at flows[flow_offset[k]] with room for m_k+n_k-1 entries
 * (same layout as flock_solve); flow_offset may be NULL (packed in order).
 * stats has `count` entries. */
int flock_batch_solve(int32_t count, const flock_instance* insts, const flock_options* opt,
                      flock_flow* flows, const int64_t* flow_offset, flock_stats* stats);

/* Served form: continuous batching with admission by a device-memory budget.
 * Requests are admitted in arrival order while their resident device state
 * fits the budget; each admitted group is launched at once and overlaps with
 * earlier launches; every instance retires (and frees its state) as soon as
 * it is solved.  Instances with m + n > 4096 run on the plain solver. */
typedef struct flock_server flock_server;
typedef struct {
    int64_t memory_budget_bytes;   /* resident device state allowed (default 40 GiB) */
    int32_t max_inflight_batches;  /* launch streams (at least 64 are used), default 16 */
    int32_t max_batch;             /* instances admitted per launch group, default 512 */
    flock_options options;
} flock_server_config;
typedef struct {
    uint64_t ticket;
    int32_t status;                /* flock_status of this request */
    flock_stats stats;
    double latency_ms;             /* submit -> result ready */
} flock_result;

void flock_default_server_config(flock_server_config* cfg);
int flock_server_create(const flock_server_config* cfg, flock_server** out);
/* Device bytes one m x n request holds while it is in the served form (its
 * budget charge); -1 for m or n < 1. */
int64_t flock_server_request_bytes(int32_t m, int32_t n);
/* Copies the instance; the result's flows are returned by flock_server_poll. */
int flock_server_submit(flock_server* s, const flock_instance* inst, uint64_t* ticket);
/* Returns up to `max` finished results; flows of result k go to flows_out[k]
 * (each with room for m+n-1 entries; may be NULL).  *count is set. */
int flock_server_poll(flock_server* s, flock_result* results, flock_flow** flows_out,
                      int32_t max, int32_t* count);
/* Blocks until every submitted request has finished. */
int flock_server_drain(flock_server* s);
int flock_server_destroy(flock_server* s);

/* Deterministic instance generators (splitmix64 + Lemire bounded integers).
 * kind 0: uniform costs [c_lo, c_hi], supplies [q_lo, q_hi], raw demands
 *         [q_lo, q_hi] rescaled to sum to the supply total (remainder to the
 *         last demand).
 * kind 1: Euclidean: m sources and n sinks uniform in [0,1000]^2, cost =
 *         round(distance) half away from zero; quantities as kind 0.
 * Buffers are caller-owned (m, n, m*n). */
int flock_generate(int32_t kind, uint64_t seed, int32_t m, int32_t n,
                   int32_t c_lo, int32_t c_hi, int32_t q_lo, int32_t q_hi,
                   int32_t* supply, int32_t* demand, int32_t* cost);
/* log-uniform integer sizes in [lo, hi]: round(exp(U(ln lo, ln hi))) */
int flock_generate_sizes(uint64_t seed, int32_t count, int32_t lo, int32_t hi,
                         int32_t* ms, int32_t* ns);

#ifdef __cplusplus
}
#endif
#endif
