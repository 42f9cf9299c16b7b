// Test-infrastructure only: a thin host driver that links the reference's own
// CPU-path functions (compiled from the reference's sources by oracle/Makefile)
// and exposes them through a C ABI for the parity tests.  Nothing here is part
// of the product; the product never loads this library.
//
// Reference functions called as they are:
//   find_vogel_bfs_sequencial         src/parallel_simplex_method/IBFS_vogel.cu:546
//   UV_METHOD::find_dual_using_host_bfs  src/parallel_simplex_method/parallel_uv_method/DUAL_solver.cu:34
//   UV_METHOD::perform_a_sequencial_pivot src/parallel_simplex_method/parallel_uv_method/PIVOT_uv.cu:318
// Pieces that live in GPU-coupled code and are therefore restated here:
//   initial tree (zero flow -> epsilon)  src/parallel_simplex_method/parallel_kernels.cu:46-67
//   sequential reduced-cost scan          src/parallel_simplex_method/parallel_uv_method/uv_model_parallel.cu:178-200
//   final retrieval + objective           src/parallel_simplex_method/parallel_kernels.cu:72-96,154-181,
//                                         src/parallel_simplex_method/parallel_uv_method/uv_model_parallel.cu:375-385
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <vector>

#include "parallel_structs.h"
#include "IBFS_vogel.h"
#include "parallel_uv_method/DUAL_solver.h"
#include "parallel_uv_method/PIVOT_uv.h"

static void to_cells(int m, int n, const float* c, std::vector<MatrixCell>& cells) {
    cells.resize((size_t)m * n);
    for (int i = 0; i < m; i++)
        for (int j = 0; j < n; j++) {
            MatrixCell x;
            x.row = i; x.col = j; x.cost = c[(size_t)i * n + j];
            cells[(size_t)i * n + j] = x;
        }
}

extern "C" int ref_vogel(int m, int n, const int* s, const int* d, const float* c,
                         int* src, int* dst, float* qty) {
    std::vector<MatrixCell> cells;
    to_cells(m, n, c, cells);
    std::vector<int> ss(s, s + m), dd(d, d + n);
    std::vector<flowInformation> flows(m + n - 1);
    for (auto& f : flows) { f.source = -1; f.destination = -1; f.qty = 0; }
    find_vogel_bfs_sequencial(ss.data(), dd.data(), cells.data(), flows.data(), m, n);
    for (int k = 0; k < m + n - 1; k++) {
        src[k] = flows[k].source; dst[k] = flows[k].destination; qty[k] = flows[k].qty;
    }
    return 0;
}

// status: 0 optimal, 1 forest (reference's guard), 2 iteration cap reached
extern "C" int ref_solve(int m, int n, const int* s, const int* d, const float* c, int max_iter,
                         int* iterations, double* objective, int* active,
                         int* fsrc, int* fdst, float* fqty, int* status) {
    const int V = m + n;
    std::vector<MatrixCell> cells;
    to_cells(m, n, c, cells);
    std::vector<int> ss(s, s + m), dd(d, d + n);
    std::vector<flowInformation> flows(V - 1);
    find_vogel_bfs_sequencial(ss.data(), dd.data(), cells.data(), flows.data(), m, n);

    Graph graph;
    graph.V = V;
    size_t utm = (size_t)V * (V + 1) / 2;
    graph.h_adjMtx_ptr = (int*)calloc(utm, sizeof(int));
    graph.h_flowMtx_ptr = (float*)calloc(V - 1, sizeof(float));
    for (int g = 0; g < V - 1; g++) {
        int row = flows[g].source, col = m + flows[g].destination;
        float q = 1.0f * flows[g].qty;
        if (q == 0) q = epsilon;
        graph.h_flowMtx_ptr[g] = q;
        graph.h_adjMtx_ptr[TREE_LOOKUP(row, col, V)] = g + 1;
    }
    graph.h_Graph.assign(V, std::vector<int>());
    for (int a = 0; a < V; a++)
        for (int b = a + 1; b < V; b++)
            if (graph.h_adjMtx_ptr[TREE_LOOKUP(a, b, V)] > 0) {
                graph.h_Graph[a].push_back(b);
                graph.h_Graph[b].push_back(a);
            }

    DualHandler dual;
    dual.h_visited = (bool*)malloc(sizeof(bool) * V);
    dual.h_variables = (float*)malloc(sizeof(float) * V);
    PivotHandler pivot;
    pivot.backtracker = (int*)malloc(sizeof(int) * (V + 1));
    pivot.stack = (stackNode*)malloc(sizeof(stackNode) * (V + 1) * 2);
    pivot.visited = (bool*)malloc(sizeof(bool) * V);
    PivotTimer timer;

    bool result = false;
    int it = 0;
    int st = 0;
    while (!result && it < max_iter) {
        UV_METHOD::find_dual_using_host_bfs(dual, graph, (float*)c, m, n);
        float min_r = INT_MAX * 1.0f;
        int pr = -1, pc = -1;
        for (int i = 0; i < m; i++)
            for (int j = 0; j < n; j++) {
                float r = c[(size_t)i * n + j] - dual.h_variables[i] - dual.h_variables[m + j];
                if (r < min_r) { min_r = r; pr = i; pc = j; }
            }
        pivot.reduced_cost = min_r;
        pivot.pivot_row = pr;
        pivot.pivot_col = pc;
        // The reference reports the forest case through stdout only: a pivot
        // that was wanted but ended the loop is that case.
        float rc = min_r;
        bool want_pivot = (rc < 0 && std::abs(rc) > epsilon2);
        UV_METHOD::perform_a_sequencial_pivot(pivot, timer, graph, result, m, n);
        if (result && want_pivot) st = 1;
        it++;
    }
    if (!result) st = 2;

    // Retrieval (slot order, rounded, zero removed) and objective.
    std::vector<int> slot_row(V - 1, -1), slot_col(V - 1, -1);
    for (int a = 0; a < m; a++)
        for (int b = m; b < V; b++) {
            int id = graph.h_adjMtx_ptr[TREE_LOOKUP(a, b, V)];
            if (id > 0) { slot_row[id - 1] = a; slot_col[id - 1] = b - m; }
        }
    int cnt = 0;
    double obj = 0.0;
    for (int k = 0; k < V - 1; k++) {
        if (slot_row[k] < 0) continue;
        float q = roundf(graph.h_flowMtx_ptr[k]);
        if (q == 0) continue;
        fsrc[cnt] = slot_row[k]; fdst[cnt] = slot_col[k]; fqty[cnt] = q;
        float prod = q * c[(size_t)slot_row[k] * n + slot_col[k]];
        obj += prod;
        cnt++;
    }
    *iterations = it;
    *objective = obj;
    *active = cnt;
    *status = st;
    free(graph.h_adjMtx_ptr); free(graph.h_flowMtx_ptr);
    free(dual.h_visited); free(dual.h_variables);
    free(pivot.backtracker); free(pivot.stack); free(pivot.visited);
    return 0;
}
