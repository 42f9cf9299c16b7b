/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * A plain-C restatement of the reference's CPU path for the transportation
 * simplex (researchgroup-zx93920/flock, "vam_host" + host dual BFS +
 * sequential reduced-cost scan + stepping-stone pivot), plus an exact int64
 * optimality-certificate checker.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load it.
 *
 * Parity is pinned: tests/test_oracle_pin.py checks this restatement against
 * the published run logs (results/pure_sequencial: iterations + objective for
 * every data file present; results/parallel_uv the same with the device Vogel
 * restatement as the BFS) and, where the reference sources are available,
 * against the reference's own functions compiled into oracle/_ref.
 */
#ifndef FLOCK_ORACLE_H
#define FLOCK_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Vogel's approximation exactly as find_vogel_bfs_sequencial
 * (src/parallel_simplex_method/IBFS_vogel.cu:546-769).  Costs are the
 * reference's float costs.  Writes m+n-1 flows in allocation order.  qty is
 * the reference's float quantity (epsilon 1e-6 in the row branch when zero).
 * Returns the number of steps whose chosen line had no uncovered crossing
 * cell (the reference then reuses the previous step's index; see oracle.c),
 * or -1 when that reused index is out of range for the line: the reference
 * then reads past its arrays, so the flows from that step on are undefined and
 * written as (-1, -1, 0). */
int orc_vogel(int m, int n, const int32_t* s, const int32_t* d, const float* c,
              int32_t* src, int32_t* dst, float* qty);

/* orc_vogel stopped after max_steps allocations (a bounded CPU timing sample
 * of a large instance); *steps_done = allocations made.  Same return value. */
int orc_vogel_steps(int m, int n, const int32_t* s, const int32_t* d, const float* c, int max_steps,
                    int32_t* src, int32_t* dst, float* qty, int32_t* steps_done);

/* One sequential reduced-cost scan as uv_model_parallel.cu:178-200: returns
 * the first (row-major) strict minimum of c_ij - h_i - h_{m+j} and its cell.
 * h holds the m row duals, then the n column duals (float). */
float orc_sweep(int m, int n, const float* c, const float* h, int32_t* row, int32_t* col);

/* The benchmark's instance generator restated (no reference counterpart; it
 * lets the timed CPU path build its inputs without the product library):
 * the same integers as flock_generate / flock_generate_sizes.  0 = ok. */
int orc_generate(int kind, uint64_t seed, int m, int n, int c_lo, int c_hi, int q_lo, int q_hi,
                 int32_t* supply, int32_t* demand, int32_t* cost);
int orc_generate_sizes(uint64_t seed, int count, int lo, int hi, int32_t* ms, int32_t* ns);

/* Vogel's approximation as the reference's device variant
 * find_vogel_bfs_parallel ("vam_device", IBFS_vogel.cu:3-543): regrets from
 * positions into per-line cost-sorted books, first largest regret, its own
 * tie rules (a different BFS from orc_vogel).  Writes m+n-1 flows in
 * allocation order.  Returns 0, or -1 when the reference would index past
 * its arrays (costs at or above the books' 32767 sentinels, a one-column
 * line run dry); the flows from that step on are written as (-1, -1, 0). */
int orc_vogel_device(int m, int n, const int32_t* s, const int32_t* d, const float* c,
                     int32_t* src, int32_t* dst, float* qty);

/* North-west corner rule (src/parallel_simplex_method/IBFS_nwc.cu:3-33). */
int orc_nwc(int m, int n, const int32_t* s, const int32_t* d,
            int32_t* src, int32_t* dst, float* qty);

/* Result of the reference CPU path. */
typedef struct {
    int32_t iterations;     /* reference's iteration counter (pivots + final check) */
    int32_t status;         /* 0 optimal, 1 forest guard, 2 iteration cap,
                               3 undefined in the reference (see orc_vogel) */
    int32_t active_flows;   /* nonzero rounded flows returned */
    int32_t vogel_events;   /* see orc_vogel */
    double objective;       /* sum of float(qty*cost) in double, as the reference */
} orc_result;

/* The reference CPU path: BFS (1 = vam_host, 0 = nwc_host, 2 = vam_device), then loop
 * { duals by BFS from row 0; row-major strict-< scan; pivot } until
 * min r >= 0 or |min r| <= 0.01 or max_iter.  Outputs the active flows
 * (slot order) and, if tree_src/tree_dst are given, the m+n-1 final basis
 * cells (slot order, including zero flows) for exact dual recovery. */
int orc_solve_ref(int m, int n, const int32_t* s, const int32_t* d, const float* c,
                  int bfs_method, int max_iter,
                  int32_t* fsrc, int32_t* fdst, float* fqty,
                  int32_t* tree_src, int32_t* tree_dst, orc_result* out);

/* Run orc_solve_ref over many instances with nthreads host threads.  Instance
 * k has shape (ms[k], ns[k]) and its arrays start at the given offsets into the
 * packed s/d/c arrays.  Objectives/iterations/status written per instance. */
int orc_solve_ref_batch(int count, const int32_t* ms, const int32_t* ns,
                        const int64_t* s_off, const int64_t* d_off, const int64_t* c_off,
                        const int32_t* s, const int32_t* d, const float* c,
                        int bfs_method, int max_iter, int nthreads,
                        double* objective, int32_t* iterations, int32_t* status);

/* Exact int64 duals for a spanning tree given as m+n-1 cells: u_0 = 0,
 * u_i + v_j = c_ij on every tree cell.  Returns 0 if the cells span all
 * m+n vertices as a tree, -1 otherwise. */
int orc_tree_duals(int m, int n, const int32_t* c, int32_t k,
                   const int32_t* tsrc, const int32_t* tdst, int64_t* u, int64_t* v);

/* Optimality certificate, all integer:
 *   bit 0: a flow index is out of range or a quantity is negative
 *   bit 1: some row sum != supply
 *   bit 2: some column sum != demand
 *   bit 3: some reduced cost c_ij - u_i - v_j < 0
 *   bit 4: complementary slackness fails (qty > 0 with reduced cost != 0)
 * Returns 0 when the flows are optimal; writes the objective sum c*qty. */
int orc_certify(int m, int n, const int32_t* s, const int32_t* d, const int32_t* c,
                int32_t k, const int32_t* fsrc, const int32_t* fdst, const int64_t* fqty,
                const int64_t* u, const int64_t* v, int64_t* objective);

#ifdef __cplusplus
}
#endif
#endif
