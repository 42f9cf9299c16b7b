// flock/algos.h -- C++ drop-in facade with the reference's solver API
// (src/algos.h:1-4, src/structs.h:19-52, src/instance.h:13-48,
// parallel_uv_method/uv_model_parallel.h:19-41): construct a model from a
// ProblemInstance and a caller-owned flow array of m+n-1 entries, call
// execute(), then create_flows(), and read objVal / totalIterations /
// totalSolveTime and the phase timers.  Header-only over the C ABI in flock.h.
//
// Differences from the reference, by design: costs are exact integers
// (ProblemInstance::cost_scale decimal digits; the float `costs` array is kept
// for source compatibility), errors are reported by exceptions carrying the
// flock_status instead of exit(), and every model runs on the GPU.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "../flock.h"
#include "parameters.h"

struct FileNotFoundException : public std::exception {
    const char* what() const throw() { return "File not found!"; }
};

struct flock_error : public std::runtime_error {
    int status;
    flock_error(int s, const std::string& w) : std::runtime_error(w), status(s) {}
};

// Container for the problem (src/structs.h:19-40).
class ProblemInstance {
public:
    bool read_mode = false;
    std::string filename;
    enum my_algo { cpu_lp_solve, parallel_uv, parallel_ss, switch_hybrid };
    my_algo algo = parallel_uv;
    int numDemands = 0, numSupplies = 0, *demands = nullptr, *supplies = nullptr, active_flows = 0;
    double readTime = 0, preprocessTime = 0, solveTime = 0, postprocessTime = 0;
    double totalFlowCost = 0;
    float* costs = nullptr;               // reference-compatible view
    std::vector<int32_t> int_costs;       // exact costs * 10^cost_scale
    int cost_scale = 0;

    void allocate_memory() {
        supplies = (int*)malloc(sizeof(int) * numSupplies);
        demands = (int*)malloc(sizeof(int) * numDemands);
        costs = (float*)malloc(sizeof(float) * (size_t)numSupplies * numDemands);
        int_costs.assign((size_t)numSupplies * numDemands, 0);
    }
    ProblemInstance() {}
    ~ProblemInstance() { free(supplies); free(demands); free(costs); }
    ProblemInstance(const ProblemInstance&) = delete;
    ProblemInstance& operator=(const ProblemInstance&) = delete;
};

// Information for a flow variable (src/structs.h:45-52).
struct flowInformation {
    int source, destination;
    float qty;
};

// .dat reader (src/instance.cpp:80-141 readSize/readCosts): exact decimal costs.
inline void make_problem(const std::string& filename, ProblemInstance& problem) {
    problem.filename = filename;
    problem.read_mode = true;
    int32_t m = 0, n = 0, scale = 0;
    int rc = flock_dat_shape(filename.c_str(), &m, &n);
    if (rc == FLOCK_ERR_FILE) throw FileNotFoundException();
    if (rc) throw flock_error(rc, flock_last_error());
    if ((rc = flock_dat_scale(filename.c_str(), &scale))) throw flock_error(rc, flock_last_error());
    problem.numSupplies = m;
    problem.numDemands = n;
    problem.allocate_memory();
    problem.cost_scale = scale;
    rc = flock_read_dat(filename.c_str(), scale, m, n, problem.supplies, problem.demands, problem.int_costs.data());
    if (rc) throw flock_error(rc, flock_last_error());
    const double p = std::pow(10.0, scale);
    for (size_t k = 0; k < problem.int_costs.size(); k++) problem.costs[k] = (float)(problem.int_costs[k] / p);
    problem.active_flows = m + n - 1;
}

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
        pivot_time = stats.ms_simplex * 1000.0;
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
// -a parallel_ss: deconflicted parallel stepping-stone pivots per sweep.
class ssModel_parallel : public flock_detail::ModelBase {
public:
    ssModel_parallel(ProblemInstance* p, flowInformation* f) : ModelBase(p, f, FLOCK_PIVOT_PARALLEL) {}
};
// -a switch_hybrid: parallel rounds until one applies fewer than 10 pivots,
// then sequential ones (switch/switch_model_parallel.cu:182-184).
class switchModel_parallel : public flock_detail::ModelBase {
public:
    switchModel_parallel(ProblemInstance* p, flowInformation* f) : ModelBase(p, f, FLOCK_PIVOT_SWITCH) {}
};
