// flock/algos.h -- C++ drop-in facade with the reference's solver API
// (src/algos.h:1-4, src/structs.h:19-52, src/instance.h:13-48,
// parallel_uv_method/uv_model_parallel.h:19-41): construct a model from a
// ProblemInstance and a caller-owned flow array of m+n-1 entries, call
// execute(), then create_flows(), and read objVal / totalIterations /
// totalSolveTime and the phase timers.  Header-only over the C ABI in flock.h.
// With this directory on the include path, the reference's own src/main.cpp
// compiles unchanged: structs.h, instance.h, logger.h and parameters.h carry
// the reference's names.
//
// Differences from the reference, by design: costs are exact integers
// (ProblemInstance::cost_scale decimal digits; the float `costs` array is kept
// for source compatibility), errors are reported by exceptions carrying the
// flock_status instead of exit(), every model runs on the GPU, and the
// Gurobi model (lpModel) is present only as a name: its execute() throws.
#pragma once
#include "instance.h"
#include "logger.h"
#include "parameters.h"
#include "structs.h"

namespace flock_detail {
class ModelBase {
public:
    ProblemInstance* data;
    flowInformation* optimal_flows;
    // Model statistics (uv_model_parallel.h:33-38); phase times in microseconds.
    double uv_time = 0, reduced_cost_time = 0, pivot_time = 0, cycle_discovery_time = 0, resolve_time = 0,
           adjustment_time = 0;
    double objVal = 0;            // objective in the instance's cost units
    int64_t objective_scaled = 0; // exact objective (costs * 10^cost_scale)
    int totalIterations = 0;
    double totalSolveTime = 0;    // ms
    flock_stats stats{};
    std::vector<flock_flow> result;

    ModelBase(ProblemInstance* problem, flowInformation* flows, int pivot)
        : data(problem), optimal_flows(flows), pivot_method(pivot) {}

    void execute() {
        const int m = data->numSupplies, n = data->numDemands;
        if (data->int_costs.size() != (size_t)m * n) {   // costs given as floats only
            data->int_costs.resize((size_t)m * n);
            const double p = std::pow(10.0, data->cost_scale);
            for (size_t k = 0; k < data->int_costs.size(); k++)
                data->int_costs[k] = (int32_t)std::llround(data->costs[k] * p);
        }
        flock_instance inst{m, n, data->supplies, data->demands, data->int_costs.data()};
        flock_options opt;
        flock_default_options(&opt);
        opt.bfs_method = FLOCK_DEFAULT_BFS;
        opt.pivot_method = pivot_method;
        opt.max_iterations = MAX_ITERATIONS;
        result.assign((size_t)m + n - 1, flock_flow{0, 0, 0});
        int rc = flock_solve(&inst, &opt, result.data(), nullptr, nullptr, &stats);
        if (rc && rc != FLOCK_ERR_NOT_OPTIMAL) throw flock_error(rc, flock_last_error());
        objective_scaled = stats.objective;
        objVal = (double)stats.objective / std::pow(10.0, data->cost_scale);
        totalIterations = stats.iterations;
        totalSolveTime = stats.ms_bfs + stats.ms_simplex;
        // phase times in microseconds (the reference's unit; main.cpp divides by 1000)
        uv_time = stats.ms_dual * 1000.0;
        reduced_cost_time = stats.ms_sweep * 1000.0;
        pivot_time = stats.ms_pivot * 1000.0;
        cycle_discovery_time = stats.ms_cycle * 1000.0;
        resolve_time = stats.ms_resolve * 1000.0;
        adjustment_time = stats.ms_adjust * 1000.0;
        data->active_flows = stats.active_flows;
        data->totalFlowCost = objVal;
        data->solveTime = totalSolveTime;
    }

    // Copies the active (nonzero) flows, as uvModel_parallel::create_flows.
    void create_flows() {
        for (int k = 0; k < data->active_flows; k++)
            optimal_flows[k] = flowInformation{result[k].source, result[k].destination, (float)result[k].qty};
    }

private:
    int pivot_method;
};
}  // namespace flock_detail

// -a parallel_uv: one pivot per reduced-cost sweep (Dantzig, row-major first minimum).
class uvModel_parallel : public flock_detail::ModelBase {
public:
    uvModel_parallel(ProblemInstance* p, flowInformation* f) : ModelBase(p, f, FLOCK_PIVOT_SEQUENTIAL) {}
};
// -a parallel_ss: every negative cell a candidate, the greedy most-negative
// set of tree-edge-disjoint cycles pivoted together each round.
class ssModel_parallel : public flock_detail::ModelBase {
public:
    ssModel_parallel(ProblemInstance* p, flowInformation* f) : ModelBase(p, f, FLOCK_PIVOT_SS) {}
};
// -a switch_hybrid: parallel rounds until one applies fewer than 10 pivots,
// then sequential ones (switch/switch_model_parallel.cu:182-184).
class switchModel_parallel : public flock_detail::ModelBase {
public:
    switchModel_parallel(ProblemInstance* p, flowInformation* f) : ModelBase(p, f, FLOCK_PIVOT_SWITCH) {}
};

// -a cpu_lp_solve: the reference's Gurobi model (gurobi_lp_method/lp_model.h).
// Not part of this library: execute() throws flock_error; main.cpp only
// reaches it when built with MAKE_WITH_GUROBI.
class lpModel {
public:
    ProblemInstance* data;
    flowInformation* optimal_flows;
    double objVal = 0;
    int totalIterations = 0;
    double totalSolveTime = 0;
    lpModel(ProblemInstance* problem, flowInformation* flows) : data(problem), optimal_flows(flows) {}
    void execute() { throw flock_error(FLOCK_ERR_ARG, "cpu_lp_solve needs Gurobi, which this library does not include"); }
    void create_flows() {}
};
