// facade_main.cpp -- test driver for the C++ facade (include/flock/algos.h),
// written the way the reference's callers use its solver API
// (src/main.cpp:53-154): parse -i/-a, make_problem, a caller-owned
// flowInformation array of m+n-1 entries, the model for the algorithm,
// execute(), create_flows(), then the statistics.  Besides the reference's
// BASIC STATISTICS line it prints a CHECK line: the objective recomputed
// from the created flows and the instance's float costs, the number of
// created flows, and the exact objective, for the test to compare.
#include <cstdio>
#include <cstdlib>
#include <iomanip>
#include <sstream>

#include "flock/algos.h"

template <class Model>
static int run(ProblemInstance& problem, flowInformation* flows) {
    Model model = Model(&problem, flows);
    model.execute();
    model.create_flows();
    std::stringstream log_msg;
    log_msg << ">>>> BASIC STATISTICS | Objective: " << std::setprecision(17) << model.objVal
            << " | Iterations: " << model.totalIterations << " | Time: " << model.totalSolveTime
            << " | MATRIX : " << problem.numSupplies << " X " << problem.numDemands;
    add_log_msg("info", log_msg.str());
    log_msg.str("");
    log_msg << ">>>> PHASES | UV Time: " << model.uv_time << " | R Time: " << model.reduced_cost_time
            << " | PIVOT Time: " << model.pivot_time << " | CYCLE Time: " << model.cycle_discovery_time
            << " | RESOLVE Time: " << model.resolve_time << " | ADJUST Time: " << model.adjustment_time;
    add_log_msg("info", log_msg.str());
    log_msg.str("");
    double recomputed = 0;
    for (int k = 0; k < problem.active_flows; k++)
        recomputed += (double)flows[k].qty * problem.costs[(size_t)flows[k].source * problem.numDemands +
                                                         flows[k].destination];
    log_msg << ">>>> CHECK | Flow cost: " << std::setprecision(17) << recomputed << " | Flows: " << problem.active_flows
            << " | Exact: " << model.objective_scaled << " | Scale: " << problem.cost_scale;
    add_log_msg("info", log_msg.str());
    return model.stats.status ? 1 : 0;
}

int main(int argc, char** argv) {
    InputParser input(argc, argv);
    ProblemInstance problem = ProblemInstance();
    make_problem(input, problem);
    flowInformation* flows =
        (flowInformation*)malloc(((size_t)problem.numSupplies + problem.numDemands - 1) * sizeof(flowInformation));
    int rc = 2;
    if (problem.algo == ProblemInstance::my_algo::parallel_uv) rc = run<uvModel_parallel>(problem, flows);
    else if (problem.algo == ProblemInstance::my_algo::parallel_ss) rc = run<ssModel_parallel>(problem, flows);
    else if (problem.algo == ProblemInstance::my_algo::switch_hybrid) rc = run<switchModel_parallel>(problem, flows);
    free(flows);
    return rc;
}
