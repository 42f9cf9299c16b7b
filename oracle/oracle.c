/*
 * oracle.c -- TEST INFRASTRUCTURE ONLY: the checker, never the product.
 *
 * Plain-C restatement of the reference CPU path of researchgroup-zx93920/flock
 * (float arithmetic reproduced operation by operation) and an exact int64
 * optimality-certificate checker.  See oracle.h for the contract; each
 * function cites the reference lines it follows.  Built with
 * -ffp-contract=off so that x86 and Arm give the same float results.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EPSILON 0.000001f /* parallel_structs.h:34 (epsilon)            */
#define ORC_EPSILON2 10e-3    /* parallel_structs.h:35 (epsilon2, a double) */

/* float -> int as the x86 `cvttss2si` the reference was built and run with:
 * truncation toward zero, and INT_MIN for NaN or anything outside
 * [-2^31, 2^31).  The C cast is undefined there (and saturates on Arm), so
 * it is spelled out.  This matters for a line with one uncovered crossing
 * cell, whose penalty is float(2^31) - c (IBFS_vogel.cu:591-606). */
static int32_t f2i_x86(float f) {
    double x = (double)f;
    if (x != x || x >= 2147483648.0 || x < -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}

/* Flows from `from` on are undefined in the reference (it indexes past its
 * arrays); they are written as (-1, -1, 0). */
static void fill_undefined(int32_t* src, int32_t* dst, float* qty, int from, int to) {
    for (int k = from; k < to; k++) { src[k] = -1; dst[k] = -1; qty[k] = 0.0f; }
}

/* IBFS_vogel.cu:546-769, find_vogel_bfs_sequencial, stopped after
 * max_steps allocations (*steps_done of them made; orc_vogel runs all m+n-1). */
static int vogel_steps(int m, int n, const int32_t* s, const int32_t* d, const float* c, int max_steps,
                       int32_t* src, int32_t* dst, float* qty, int* steps_done) {
    const int V = m + n;
    int32_t* rs = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
    int32_t* rd = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    int32_t* rowCov = (int32_t*)calloc((size_t)m, sizeof(int32_t));
    int32_t* colCov = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    int32_t* diff = (int32_t*)calloc((size_t)V, sizeof(int32_t));
    memcpy(rs, s, sizeof(int32_t) * (size_t)m);
    memcpy(rd, d, sizeof(int32_t) * (size_t)n);
    int coveredRows = 0, coveredCols = 0;
    int prev_row = 1, prev_col = 1;
    /* The reference declares its min-cost index inside the loop without an
     * initialiser; when the chosen line has no uncovered crossing cell the
     * index keeps the previous step's value.  That is reproduced here (the
     * variable lives outside the loop) and counted. */
    int i_minCost = 0;
    int events = 0;
    const float FMAX = (float)2147483647; /* INT_MAX converted: 2^31 */

    int steps = 0;
    while (coveredRows + coveredCols < V - 1 && steps < max_steps) {
        steps++;
        if (prev_row) { /* :588-613 */
            for (int i = 0; i < m; i++) {
                if (rowCov[i] == 0) {
                    float t1 = FMAX, t2 = FMAX;
                    for (int j = 0; j < n; j++) {
                        if (colCov[j] == 0) {
                            float e = c[(size_t)i * n + j];
                            if (e <= t1) { t2 = t1; t1 = e; }
                            else if (e <= t2) { t2 = e; }
                        }
                    }
                    diff[i] = f2i_x86(t2 - t1);
                } else {
                    diff[i] = -1;
                }
            }
            prev_row = 0;
        }
        if (prev_col) { /* :616-642 */
            for (int j = 0; j < n; j++) {
                if (colCov[j] == 0) {
                    float t1 = FMAX, t2 = FMAX;
                    for (int i = 0; i < m; i++) {
                        if (rowCov[i] == 0) {
                            float e = c[(size_t)i * n + j];
                            if (e <= t1) { t2 = t1; t1 = e; }
                            else if (e <= t2) { t2 = e; }
                        }
                    }
                    diff[m + j] = f2i_x86(t2 - t1);
                } else {
                    diff[m + j] = -1;
                }
            }
            prev_col = 0;
        }
        /* :651-659 -- compared as float, ties to the LAST index */
        float tempDiff = (float)INT32_MIN;
        int sel = -1;
        for (int k = 0; k < V; k++) {
            if ((float)diff[k] >= tempDiff) { tempDiff = (float)diff[k]; sel = k; }
        }
        int counter = coveredRows + coveredCols;
        int row, col;
        float q;
        if (sel >= m) { /* column branch :666-714 */
            col = sel - m;
            float ct = FMAX;
            int found = 0;
            for (int i = 0; i < m; i++) {
                float e = c[(size_t)i * n + col];
                if (e < ct && rowCov[i] == 0) { ct = e; i_minCost = i; found = 1; }
            }
            if (!found) events++;
            row = i_minCost;
            if (row < 0 || row >= m) { events = -1; fill_undefined(src, dst, qty, counter, V - 1); break; }
            if (rd[col] > rs[row]) {
                q = 1.0f * rs[row];
                rd[col] -= rs[row]; rs[row] = 0; rowCov[row] = 1; prev_row = 1; coveredRows += 1;
            } else {
                q = 1.0f * rd[col];
                rs[row] -= rd[col]; rd[col] = 0; colCov[col] = 1; prev_col = 1; coveredCols += 1;
            }
        } else { /* row branch :716-762 */
            row = sel;
            float ct = FMAX;
            int found = 0;
            for (int j = 0; j < n; j++) {
                float e = c[(size_t)row * n + j];
                if (e < ct && colCov[j] == 0) { ct = e; i_minCost = j; found = 1; }
            }
            if (!found) events++;
            col = i_minCost;
            if (col < 0 || col >= n) { events = -1; fill_undefined(src, dst, qty, counter, V - 1); break; }
            if (rd[col] > rs[row]) {
                q = fmaxf(1.0f * rs[row], ORC_EPSILON);
                rd[col] -= rs[row]; rs[row] = 0; rowCov[row] = 1; prev_row = 1; coveredRows += 1;
            } else {
                q = fmaxf(1.0f * rd[col], ORC_EPSILON);
                rs[row] -= rd[col]; rd[col] = 0; colCov[col] = 1; prev_col = 1; coveredCols += 1;
            }
        }
        src[counter] = row;
        dst[counter] = col;
        qty[counter] = q;
    }
    free(rs); free(rd); free(rowCov); free(colCov); free(diff);
    if (steps_done) *steps_done = steps;
    return events;
}

int orc_vogel(int m, int n, const int32_t* s, const int32_t* d, const float* c,
              int32_t* src, int32_t* dst, float* qty) {
    return vogel_steps(m, n, s, d, c, m + n - 1, src, dst, qty, NULL);
}

int orc_vogel_steps(int m, int n, const int32_t* s, const int32_t* d, const float* c, int max_steps,
                    int32_t* src, int32_t* dst, float* qty, int32_t* steps_done) {
    int k = 0;
    const int ev = vogel_steps(m, n, s, d, c, max_steps, src, dst, qty, &k);
    if (steps_done) *steps_done = k;
    return ev;
}

/* ---------------------------------------------------------------------- */
/* IBFS_vogel.cu:3-543, find_vogel_bfs_parallel ("vam_device").
 *
 * Books (IBFS_vogel.cu:126-350): each row lists its n cells plus two
 * sentinels (index n and n+1, cost 32767), stably sorted by float cost, so
 * equal costs keep index order; then the entry at position n+1 gets cost - 1
 * (override_row_sorts).  Columns likewise over m rows.
 * Line state (parallel_structs.h:184-187): positions il1, il2 into the book
 * (initially 0 and 1), the entry's index and the float regret diff.
 * A step (IBFS_vogel.cu:417-537): refresh the lines of the kind that was not
 * eliminated last (both kinds at the first step, rows first), pick the FIRST
 * largest diff over [rows, columns] (thrust::max_element), allocate, and
 * reset the eliminated line to {idx -1, il1 = other-kind count, il2 = +1,
 * diff -1}.  A refresh (computeDifferences, :3-122) only moves positions whose
 * entry is the eliminated line: il2 advances while it is below the last real
 * position and the line at the new position is covered (its il1 >= the
 * count of the refreshing kind).  */
typedef struct { int32_t idx; float cost; } orc_book_cell;
typedef struct { int32_t idx, il1, il2; float diff; } orc_vdiff;

static int cmp_book(const void* a, const void* b) {
    const orc_book_cell *x = (const orc_book_cell*)a, *y = (const orc_book_cell*)b;
    if (x->cost < y->cost) return -1;
    if (y->cost < x->cost) return 1;
    return (x->idx > y->idx) - (x->idx < y->idx);   /* stable: original (index) order */
}

/* One line's book: len real entries, two sentinels, sorted, last decremented. */
static void build_book(orc_book_cell* b, int len, const float* cost, size_t stride) {
    for (int k = 0; k < len; k++) { b[k].idx = k; b[k].cost = cost[(size_t)k * stride]; }
    b[len].idx = len; b[len].cost = 1.0f * 32767;
    b[len + 1].idx = len + 1; b[len + 1].cost = 1.0f * 32767;
    qsort(b, (size_t)len + 2, sizeof(orc_book_cell), cmp_book);
    b[len + 1].cost -= 1;
}

/* Refresh one line (computeDifferences).  book: the line's book (len real
 * entries), other: the state of the other kind's lines (count len), covered
 * when other[x].il1 >= own_count.  Returns -1 if an index leaves the arrays. */
static int vdiff_refresh(orc_vdiff* e, const orc_book_cell* book, int len, const orc_vdiff* other,
                         int own_count, int reject) {
    orc_book_cell l1 = book[e->il1], l2 = book[e->il2];
    if (l1.idx == reject || l2.idx == reject) {
        if (l1.idx == reject) { e->il1 = e->il2; l1 = l2; }
        while (e->il2 < len - 1) {
            e->il2 += 1;
            const int x = book[e->il2].idx;
            if (x < 0 || x >= len) return -1;
            if (other[x].il1 < own_count) break;
        }
        l2 = book[e->il2];
    }
    e->diff = l2.cost - l1.cost;
    e->idx = l1.idx;
    return 0;
}

int orc_vogel_device(int m, int n, const int32_t* s, const int32_t* d, const float* c,
                     int32_t* src, int32_t* dst, float* qty) {
    const int V = m + n;
    orc_book_cell* rb = (orc_book_cell*)malloc(sizeof(orc_book_cell) * (size_t)m * (n + 2));
    orc_book_cell* cb = (orc_book_cell*)malloc(sizeof(orc_book_cell) * (size_t)n * (m + 2));
    orc_vdiff* v = (orc_vdiff*)malloc(sizeof(orc_vdiff) * (size_t)V);
    int32_t* rs = (int32_t*)malloc(sizeof(int32_t) * (size_t)m);
    int32_t* rd = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    for (int i = 0; i < m; i++) build_book(rb + (size_t)i * (n + 2), n, c + (size_t)i * n, 1);
    for (int j = 0; j < n; j++) build_book(cb + (size_t)j * (m + 2), m, c + j, (size_t)n);
    for (int x = 0; x < V; x++) { v[x].idx = 0; v[x].il1 = 0; v[x].il2 = 1; v[x].diff = 0.0f; }
    memcpy(rs, s, sizeof(int32_t) * (size_t)m);
    memcpy(rd, d, sizeof(int32_t) * (size_t)n);
    int prev = -1, rc = 0, counter = 0;
    for (; counter < V - 1; counter++) {
        /* refresh: rows after a column (or at the start), columns after a row */
        for (int pass = 0; pass < (counter == 0 ? 2 : 1); pass++) {
            const int p = counter == 0 ? (pass == 0 ? V : -1) : prev;
            if (p >= m) {
                for (int i = 0; i < m && !rc; i++)
                    rc = vdiff_refresh(&v[i], rb + (size_t)i * (n + 2), n, v + m, m, p - m);
            } else {
                for (int j = 0; j < n && !rc; j++)
                    rc = vdiff_refresh(&v[m + j], cb + (size_t)j * (m + 2), m, v, n, p);
            }
        }
        if (rc) break;
        int best = 0;                                  /* first maximum */
        for (int x = 1; x < V; x++) if (v[best].diff < v[x].diff) best = x;
        int row, col;
        if (best >= m) { col = best - m; row = v[best].idx; }
        else { row = best; col = v[best].idx; }
        if (row < 0 || row >= m || col < 0 || col >= n) { rc = -1; break; }
        src[counter] = row;
        dst[counter] = col;
        if (rd[col] > rs[row]) {
            qty[counter] = fmaxf(1.0f * rs[row], ORC_EPSILON);
            rd[col] -= rs[row];
            rs[row] = 0;
            prev = row;
            v[row].idx = -1; v[row].il1 = n; v[row].il2 = n + 1; v[row].diff = -1.0f;
        } else {
            qty[counter] = fmaxf(1.0f * rd[col], ORC_EPSILON);
            rs[row] -= rd[col];
            rd[col] = 0;
            prev = m + col;
            v[m + col].idx = -1; v[m + col].il1 = m; v[m + col].il2 = m + 1; v[m + col].diff = -1.0f;
        }
    }
    if (rc) fill_undefined(src, dst, qty, counter, V - 1);
    free(rb); free(cb); free(v); free(rs); free(rd);
    return rc;
}

/* IBFS_nwc.cu:3-33 (reads one element past the end only after the last
 * allocation; the restatement stops first). */
int orc_nwc(int m, int n, const int32_t* s, const int32_t* d,
            int32_t* src, int32_t* dst, float* qty) {
    int r = 0, k = 0, cnt = 0;
    int32_t cd = d[0], cs = s[0];
    while (r < m && k < n) {
        if (cd >= cs) {
            src[cnt] = r; dst[cnt] = k; qty[cnt] = fmaxf(1.0f * cs, ORC_EPSILON);
            cd -= cs; r++; cs = (r < m) ? s[r] : 0;
        } else {
            src[cnt] = r; dst[cnt] = k; qty[cnt] = fmaxf(1.0f * cd, ORC_EPSILON);
            cs -= cd; k++; cd = (k < n) ? d[k] : 0;
        }
        cnt++;
    }
    return cnt;
}

/* ---------------------------------------------------------------------- */
/* Reference CPU path: uv_model_parallel.cu:227-395 with
 *   BFS_METHOD "vam_host", REDUCED_COST_MODE "sequencial",
 *   CALCULATE_DUAL "host_bfs", SEQ_CYCLE_SEARCH "dfs".
 * The basis is kept as m+n-1 flow slots with a cell->slot map, exactly the
 * reference's TREE_LOOKUP adjacency matrix + flowMtx (parallel_kernels.cu:
 * 46-67): a later slot on the same cell replaces the earlier one.  Adjacency
 * lists are kept like the reference's h_Graph: initially in ascending
 * neighbour order, then erase + push_back per pivot (PIVOT_uv.cu:248-258).
 * The order only matters when the basis is not a tree (Vogel can return a
 * cycle plus a separate component on degenerate input); the reference's own
 * initial order there is the GPU atomic order, and ascending order is the
 * one its host driver in oracle/_ref uses.                                  */

typedef struct {
    int32_t* a;
    int32_t len, cap;
} orc_list;

static void list_push(orc_list* l, int32_t x) {
    if (l->len == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 4;
        l->a = (int32_t*)realloc(l->a, sizeof(int32_t) * (size_t)l->cap);
    }
    l->a[l->len++] = x;
}

static void list_erase_all(orc_list* l, int32_t x) {
    int w = 0;
    for (int r = 0; r < l->len; r++) if (l->a[r] != x) l->a[w++] = l->a[r];
    l->len = w;
}

typedef struct { int32_t index, depth; } orc_stack_node;

/* TREE_LOOKUP(a, b) -> flow slot (parallel_structs.h:93); -1 if not basic. */
static int slot_of_cell(const int32_t* cell_slot, int m, int n, int a, int b) {
    int r = a < b ? a : b;
    int k = (a < b ? b : a) - m;
    if (r < 0 || r >= m || k < 0 || k >= n) return -1;
    return cell_slot[(size_t)r * n + k];
}

static int cmp_i64(const void* a, const void* b) {
    int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/* uv_model_parallel.cu:178-200: the sequential reduced-cost scan, row-major,
 * the first strict minimum of c_ij - h_i - h_{m+j} (float). */
static void seq_sweep(int m, int n, const float* c, const float* h, float* min_out, int* row, int* col) {
    float min_r = (float)2147483647;
    int pr = -1, pc = -1;
    for (int i = 0; i < m; i++) {
        const float* ci = c + (size_t)i * n;
        float ui = h[i];
        for (int j = 0; j < n; j++) {
            float r = ci[j] - ui - h[m + j];
            if (r < min_r) { min_r = r; pr = i; pc = j; }
        }
    }
    *min_out = min_r; *row = pr; *col = pc;
}

float orc_sweep(int m, int n, const float* c, const float* h, int32_t* row, int32_t* col) {
    float r;
    int a, b;
    seq_sweep(m, n, c, h, &r, &a, &b);
    if (row) *row = a;
    if (col) *col = b;
    return r;
}

int orc_solve_ref(int m, int n, const int32_t* s, const int32_t* d, const float* c,
                  int bfs_method, int max_iter,
                  int32_t* fsrc, int32_t* fdst, float* fqty,
                  int32_t* tree_src, int32_t* tree_dst, orc_result* out) {
    const int V = m + n;
    int32_t* slot_row = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
    int32_t* slot_col = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
    float* flow = (float*)malloc(sizeof(float) * (size_t)V);
    int32_t* cell_slot = (int32_t*)malloc(sizeof(int32_t) * (size_t)m * n);
    orc_list* adj = (orc_list*)calloc((size_t)V, sizeof(orc_list));
    float* h = (float*)malloc(sizeof(float) * (size_t)V);
    char* vis = (char*)malloc((size_t)V);
    int32_t* queue = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
    int32_t* bt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V + 2));
    size_t stack_cap = (size_t)(2 * V + 4);
    orc_stack_node* stack = (orc_stack_node*)malloc(sizeof(orc_stack_node) * stack_cap);
    for (size_t x = 0; x < (size_t)m * n; x++) cell_slot[x] = -1;

    float* q0 = (float*)malloc(sizeof(float) * (size_t)V);
    int ev = 0;
    if (bfs_method == 0) orc_nwc(m, n, s, d, slot_row, slot_col, q0);
    else if (bfs_method == 2) ev = orc_vogel_device(m, n, s, d, c, slot_row, slot_col, q0);
    else ev = orc_vogel(m, n, s, d, c, slot_row, slot_col, q0);
    if (ev < 0) {
        /* The reference's run is undefined from here on (out-of-range index). */
        if (out) { out->iterations = 0; out->status = 3; out->active_flows = 0;
                   out->vogel_events = ev; out->objective = 0.0; }
        free(q0); free(slot_row); free(slot_col); free(flow); free(cell_slot); free(adj);
        free(h); free(vis); free(queue); free(bt); free(stack);
        return 0;
    }
    /* parallel_kernels.cu:53-66: zero flow -> epsilon */
    for (int g = 0; g < V - 1; g++) {
        float qq = 1.0f * q0[g];
        if (qq == 0) qq = ORC_EPSILON;
        flow[g] = qq;
        cell_slot[(size_t)slot_row[g] * n + slot_col[g]] = g;
    }
    free(q0);
    {   /* initial adjacency in ascending neighbour order */
        int64_t* cells = (int64_t*)malloc(sizeof(int64_t) * (size_t)V);
        int k = 0;
        for (int g = 0; g < V - 1; g++) {
            int64_t cell = (int64_t)slot_row[g] * n + slot_col[g];
            if (cell_slot[cell] == g) cells[k++] = cell;
        }
        qsort(cells, (size_t)k, sizeof(int64_t), cmp_i64);
        for (int e = 0; e < k; e++) {
            int r = (int)(cells[e] / n), col = (int)(cells[e] % n);
            list_push(&adj[r], m + col);
        }
        /* columns: rows ascending -> iterate cells column-major */
        for (int col = 0; col < n; col++)
            for (int r = 0; r < m; r++)
                if (cell_slot[(size_t)r * n + col] >= 0) list_push(&adj[m + col], r);
        free(cells);
    }

    int it = 0, status = 2, done = 0;
    while (!done && it < max_iter) {
        /* DUAL_solver.cu:34-63 */
        for (int v = 0; v < V; v++) { h[v] = 0.0f; vis[v] = 0; }
        {
            int qh = 0, qt = 0;
            vis[0] = 1;
            queue[qt++] = 0;
            while (qh < qt) {
                int p = queue[qh++];
                for (int e = 0; e < adj[p].len; e++) {
                    int ch = adj[p].a[e];
                    if (!vis[ch]) {
                        vis[ch] = 1;
                        int row = p < ch ? p : ch;
                        int col = (p < ch ? ch : p) - m;
                        h[ch] = c[(size_t)row * n + col] - h[p];
                        queue[qt++] = ch;
                    }
                }
            }
        }
        float min_r;
        int pr, pc;
        seq_sweep(m, n, c, h, &min_r, &pr, &pc);
        /* PIVOT_uv.cu:318-401 */
        if (min_r < 0 && (double)fabsf(min_r) > ORC_EPSILON2) {
            /* PIVOT_uv.cu:156-209 (DFS from column vertex m+pc to row pr) */
            int depth = 1;
            {
                for (int v = 0; v < V; v++) vis[v] = 0;
                int top = -1;
                stack[++top] = (orc_stack_node){m + pc, 1};
                while (top != -1) {
                    orc_stack_node cv = stack[top--];
                    if (!vis[cv.index]) {
                        vis[cv.index] = 1;
                        int cur_depth = cv.depth + 1;
                        bt[cv.depth] = cv.index;
                        int adjacent = 0;
                        if (cv.index >= m && cell_slot[(size_t)pr * n + (cv.index - m)] >= 0) adjacent = 1;
                        if (adjacent && cur_depth > 1) { depth = cur_depth; break; }
                        for (int e = 0; e < adj[cv.index].len; e++) {
                            if ((size_t)(top + 1) >= stack_cap) {
                                stack_cap *= 2;
                                stack = (orc_stack_node*)realloc(stack, sizeof(orc_stack_node) * stack_cap);
                            }
                            stack[++top] = (orc_stack_node){adj[cv.index].a[e], cur_depth};
                        }
                    }
                    if (top == -1) depth = 1;
                }
            }
            if (depth <= 1) { status = 1; done = 1; it++; break; }
            bt[0] = pr;
            bt[depth] = pr;
            float min_flow = (float)2147483647;
            int min_slot = -1, min_from = -1, min_to = -1;
            for (int i = 1; i < depth; i += 2) { /* PIVOT_uv.cu:280-296 */
                int a = bt[i], b = bt[i + 1];
                int g = slot_of_cell(cell_slot, m, n, a, b);
                float f = flow[g];
                if (f < min_flow) { min_flow = f; min_slot = g; min_from = a; min_to = b; }
            }
            for (int i = 1; i < depth; i++) { /* PIVOT_uv.cu:236-244 */
                int g = slot_of_cell(cell_slot, m, n, bt[i], bt[i + 1]);
                float fl = (float)((i % 2) ? -1 : 1) * min_flow;
                flow[g] += fl;
            }
            /* PIVOT_uv.cu:248-261 */
            {
                int r = min_from < min_to ? min_from : min_to;
                int k = (min_from < min_to ? min_to : min_from) - m;
                cell_slot[(size_t)r * n + k] = -1;
                list_erase_all(&adj[min_to], min_from);
                list_erase_all(&adj[min_from], min_to);
            }
            cell_slot[(size_t)pr * n + pc] = min_slot;
            list_push(&adj[pr], m + pc);
            list_push(&adj[m + pc], pr);
            slot_row[min_slot] = pr;
            slot_col[min_slot] = pc;
            flow[min_slot] = min_flow;
        } else {
            status = 0;
            done = 1;
        }
        it++;
    }

    /* parallel_kernels.cu:72-96,154-181 and uv_model_parallel.cu:375-385 */
    int cnt = 0;
    double obj = 0.0;
    int tk = 0;
    for (int g = 0; g < V - 1; g++) {
        int r = slot_row[g], k = slot_col[g];
        if (cell_slot[(size_t)r * n + k] != g) continue;
        if (tree_src) { tree_src[tk] = r; tree_dst[tk] = k; }
        tk++;
        float q = roundf(flow[g]);
        if (q == 0) continue;
        if (fsrc) { fsrc[cnt] = r; fdst[cnt] = k; fqty[cnt] = q; }
        float prod = q * c[(size_t)r * n + k];
        obj += prod;
        cnt++;
    }
    if (tree_src) for (; tk < V - 1; tk++) { tree_src[tk] = -1; tree_dst[tk] = -1; }
    if (out) {
        out->iterations = it;
        out->status = status;
        out->active_flows = cnt;
        out->vogel_events = ev;
        out->objective = obj;
    }
    for (int v = 0; v < V; v++) free(adj[v].a);
    free(adj); free(slot_row); free(slot_col); free(flow); free(cell_slot);
    free(h); free(vis); free(queue); free(bt); free(stack);
    return 0;
}

/* ---------------------------------------------------------------------- */
typedef struct {
    int count;
    const int32_t *ms, *ns;
    const int64_t *s_off, *d_off, *c_off;
    const int32_t *s, *d;
    const float* c;
    int bfs_method, max_iter;
    double* objective;
    int32_t *iterations, *status;
    int next;
    pthread_mutex_t mu;
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* job = (batch_job*)arg;
    for (;;) {
        pthread_mutex_lock(&job->mu);
        int k = job->next++;
        pthread_mutex_unlock(&job->mu);
        if (k >= job->count) break;
        orc_result r;
        orc_solve_ref(job->ms[k], job->ns[k], job->s + job->s_off[k], job->d + job->d_off[k],
                      job->c + job->c_off[k], job->bfs_method, job->max_iter,
                      NULL, NULL, NULL, NULL, NULL, &r);
        job->objective[k] = r.objective;
        job->iterations[k] = r.iterations;
        job->status[k] = r.status;
    }
    return NULL;
}

int orc_solve_ref_batch(int count, const int32_t* ms, const int32_t* ns,
                        const int64_t* s_off, const int64_t* d_off, const int64_t* c_off,
                        const int32_t* s, const int32_t* d, const float* c,
                        int bfs_method, int max_iter, int nthreads,
                        double* objective, int32_t* iterations, int32_t* status) {
    batch_job job;
    job.count = count; job.ms = ms; job.ns = ns;
    job.s_off = s_off; job.d_off = d_off; job.c_off = c_off;
    job.s = s; job.d = d; job.c = c;
    job.bfs_method = bfs_method; job.max_iter = max_iter;
    job.objective = objective; job.iterations = iterations; job.status = status;
    job.next = 0;
    pthread_mutex_init(&job.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &job);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&job.mu);
    return 0;
}

/* ---------------------------------------------------------------------- */
int orc_tree_duals(int m, int n, const int32_t* c, int32_t k,
                   const int32_t* tsrc, const int32_t* tdst, int64_t* u, int64_t* v) {
    const int V = m + n;
    int32_t* deg = (int32_t*)calloc((size_t)V + 1, sizeof(int32_t));
    int32_t* start = (int32_t*)malloc(sizeof(int32_t) * ((size_t)V + 1));
    int32_t* nbr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(2 * (k + 1)));
    int32_t* seen = (int32_t*)calloc((size_t)V, sizeof(int32_t));
    int64_t* pot = (int64_t*)calloc((size_t)V, sizeof(int64_t));
    int32_t* queue = (int32_t*)malloc(sizeof(int32_t) * (size_t)V);
    int ok = 0;
    for (int e = 0; e < k; e++) {
        if (tsrc[e] < 0 || tsrc[e] >= m || tdst[e] < 0 || tdst[e] >= n) { ok = -1; break; }
        deg[tsrc[e]]++; deg[m + tdst[e]]++;
    }
    if (ok == 0) {
        start[0] = 0;
        for (int x = 0; x < V; x++) start[x + 1] = start[x] + deg[x];
        memset(deg, 0, sizeof(int32_t) * (size_t)V);
        for (int e = 0; e < k; e++) {
            int a = tsrc[e], b = m + tdst[e];
            nbr[start[a] + deg[a]++] = b;
            nbr[start[b] + deg[b]++] = a;
        }
        int qh = 0, qt = 0;
        queue[qt++] = 0; seen[0] = 1; pot[0] = 0;
        while (qh < qt) {
            int p = queue[qh++];
            for (int e = start[p]; e < start[p + 1]; e++) {
                int ch = nbr[e];
                if (!seen[ch]) {
                    seen[ch] = 1;
                    int row = p < ch ? p : ch, col = (p < ch ? ch : p) - m;
                    pot[ch] = (int64_t)c[(size_t)row * n + col] - pot[p];
                    queue[qt++] = ch;
                }
            }
        }
        if (qt != V || k != V - 1) ok = -1;
        for (int i = 0; i < m; i++) u[i] = pot[i];
        for (int j = 0; j < n; j++) v[j] = pot[m + j];
    }
    free(deg); free(start); free(nbr); free(seen); free(pot); free(queue);
    return ok;
}

int orc_certify(int m, int n, const int32_t* s, const int32_t* d, const int32_t* c,
                int32_t k, const int32_t* fsrc, const int32_t* fdst, const int64_t* fqty,
                const int64_t* u, const int64_t* v, int64_t* objective) {
    int bad = 0;
    int64_t* rs = (int64_t*)calloc((size_t)m, sizeof(int64_t));
    int64_t* cs = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t obj = 0;
    for (int e = 0; e < k; e++) {
        int i = fsrc[e], j = fdst[e];
        if (i < 0 || i >= m || j < 0 || j >= n || fqty[e] < 0) { bad |= 1; continue; }
        rs[i] += fqty[e];
        cs[j] += fqty[e];
        obj += fqty[e] * (int64_t)c[(size_t)i * n + j];
        if (fqty[e] > 0 && (int64_t)c[(size_t)i * n + j] - u[i] - v[j] != 0) bad |= 16;
    }
    for (int i = 0; i < m; i++) if (rs[i] != s[i]) bad |= 2;
    for (int j = 0; j < n; j++) if (cs[j] != d[j]) bad |= 4;
    for (int i = 0; i < m && !(bad & 8); i++) {
        const int32_t* ci = c + (size_t)i * n;
        for (int j = 0; j < n; j++) {
            if ((int64_t)ci[j] - u[i] - v[j] < 0) { bad |= 8; break; }
        }
    }
    if (objective) *objective = obj;
    free(rs); free(cs);
    return bad;
}

/* ---------------------------------------------------------------------- */
/* The benchmark's instance generator (flock_generate / flock_generate_sizes
 * of the native library), restated here so that the timed CPU path can make
 * its inputs without loading the product: a splitmix64 stream, Lemire's
 * bounded integers (multiply-shift with rejection below 2^32 mod range),
 * 53-bit unit doubles; Euclidean costs round(sqrt(dx^2 + dy^2)) half away
 * from zero; demands scaled to the supply total, remainder to the last.
 * tests/test_oracle_pin.py checks it against the library bit for bit. */
typedef struct { uint64_t s; } orc_rng;

static uint64_t rng_next(orc_rng* r) {
    uint64_t z = (r->s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint32_t rng_bounded(orc_rng* r, uint32_t range) {
    uint32_t x = (uint32_t)(rng_next(r) >> 32);
    uint64_t mm = (uint64_t)x * range;
    uint32_t lo = (uint32_t)mm;
    if (lo < range) {
        const uint32_t t = (uint32_t)(0u - range) % range;
        while (lo < t) { x = (uint32_t)(rng_next(r) >> 32); mm = (uint64_t)x * range; lo = (uint32_t)mm; }
    }
    return (uint32_t)(mm >> 32);
}

static int32_t rng_uniform(orc_rng* r, int32_t lo, int32_t hi) {
    return lo + (int32_t)rng_bounded(r, (uint32_t)(hi - lo + 1));
}

static double rng_unit(orc_rng* r) { return (double)(rng_next(r) >> 11) * (1.0 / 9007199254740992.0); }

int orc_generate(int kind, uint64_t seed, int m, int n, int c_lo, int c_hi, int q_lo, int q_hi,
                 int32_t* supply, int32_t* demand, int32_t* cost) {
    if (m < 1 || n < 1 || q_lo < 0 || q_hi < q_lo) return 1;
    orc_rng r = {seed};
    if (kind == 0) {
        if (c_hi < c_lo) return 1;
        for (int64_t k = 0; k < (int64_t)m * n; k++) cost[k] = rng_uniform(&r, c_lo, c_hi);
    } else if (kind == 1) {
        double* px = (double*)malloc(sizeof(double) * (size_t)(2 * m + 2 * n));
        double *py = px + m, *qx = py + m, *qy = qx + n;
        for (int i = 0; i < m; i++) { px[i] = 1000.0 * rng_unit(&r); py[i] = 1000.0 * rng_unit(&r); }
        for (int j = 0; j < n; j++) { qx[j] = 1000.0 * rng_unit(&r); qy[j] = 1000.0 * rng_unit(&r); }
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) {
                const double dx = px[i] - qx[j], dy = py[i] - qy[j];
                const double sq = dx * dx;
                const double s2 = sq + dy * dy;
                cost[(size_t)i * n + j] = (int32_t)round(sqrt(s2));
            }
        free(px);
    } else {
        return 1;
    }
    int64_t S = 0, R = 0, D = 0;
    for (int i = 0; i < m; i++) { supply[i] = rng_uniform(&r, q_lo, q_hi); S += supply[i]; }
    int64_t* raw = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    for (int j = 0; j < n; j++) { raw[j] = rng_uniform(&r, q_lo, q_hi); R += raw[j]; }
    for (int j = 0; j < n; j++) {
        const int64_t dj = R > 0 ? (raw[j] * S) / R : (j == n - 1 ? S : 0);
        demand[j] = (int32_t)dj;
        D += dj;
    }
    demand[n - 1] += (int32_t)(S - D);
    free(raw);
    return 0;
}

int orc_generate_sizes(uint64_t seed, int count, int lo, int hi, int32_t* ms, int32_t* ns) {
    if (count < 0 || lo < 1 || hi < lo) return 1;
    orc_rng r = {seed};
    const double a = log((double)lo), b = log((double)hi);
    for (int k = 0; k < count; k++) {
        const double um = a + (b - a) * rng_unit(&r);
        const double un = a + (b - a) * rng_unit(&r);
        double x = round(exp(um)), y = round(exp(un));
        x = x < lo ? lo : (x > hi ? hi : x);
        y = y < lo ? lo : (y > hi ? hi : y);
        ms[k] = (int32_t)x;
        ns[k] = (int32_t)y;
    }
    return 0;
}
