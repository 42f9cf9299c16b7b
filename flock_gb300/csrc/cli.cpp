// cli.cpp -- `flock -i <file.dat> -a <algo>`, the reference's command line
// (src/main.cpp:16-167, src/instance.cpp:6-78) on the GPU solver, written
// against the reference-named facade (flock/algos.h: InputParser,
// make_problem, the model classes) the way a reference caller uses it.
// Prints the reference's BASIC, LVL1 and LVL2 STATISTICS lines, which its
// batch scripts parse, with the objective exact in the input's decimal units.
// Differences: -a defaults to parallel_uv (the reference: cpu_lp_solve, a
// Gurobi model this library does not include), and errors go to stderr with
// an exit status (255 input file, 254 algorithm, 253 solve).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/flock/algos.h"

static void log_error(const std::string& msg) { fprintf(stderr, "[error] => %s\n", msg.c_str()); }

// The exact objective in the input's units: objective_scaled / 10^scale.
static std::string exact_objective(int64_t q, int scale) {
    char buf[64];
    if (scale <= 0) {
        snprintf(buf, sizeof buf, "%lld", (long long)q);
        return buf;
    }
    long long p = 1;
    for (int k = 0; k < scale; k++) p *= 10;
    const unsigned long long a = q < 0 ? 0ull - (unsigned long long)q : (unsigned long long)q;
    snprintf(buf, sizeof buf, "%s%llu.%0*llu", q < 0 ? "-" : "", a / p, scale, a % p);
    return buf;
}

int main(int argc, char** argv) {
    InputParser input(argc, argv);
    std::string algo = input.cmdOptionExists("-a") ? input.getCmdOption("-a") : std::string("parallel_uv");
    if (!input.cmdOptionExists("-i") || input.getCmdOption("-i").empty()) {
        log_error("Provide input file with argument -i");
        return 255;
    }
    if (algo == "cpu_lp_solve") {
        log_error("cpu_lp_solve needs Gurobi, which this library does not include");
        return 254;
    }
    if (algo != "parallel_uv" && algo != "parallel_ss" && algo != "switch_hybrid") {
        log_error("Invalid Algorithm!");
        return 254;
    }
    ProblemInstance problem;
    try {
        make_problem(input, problem);
    } catch (const FileNotFoundException&) {
        log_error("File :" + input.getCmdOption("-i") + " doesn't exist!");
        return 255;
    } catch (const std::exception& e) {
        log_error(e.what());
        return 254;
    }
    if (!input.cmdOptionExists("-a")) problem.algo = ProblemInstance::parallel_uv;   // this CLI's default
    printf("[info] => Problem Dimension => Supplies: %d\tDemands: %d\n", problem.numSupplies, problem.numDemands);
    std::vector<flowInformation> flows((size_t)problem.numSupplies + problem.numDemands - 1);
    std::unique_ptr<flock_detail::ModelBase> model;
    if (problem.algo == ProblemInstance::parallel_uv) model.reset(new uvModel_parallel(&problem, flows.data()));
    else if (problem.algo == ProblemInstance::parallel_ss) model.reset(new ssModel_parallel(&problem, flows.data()));
    else model.reset(new switchModel_parallel(&problem, flows.data()));
    try {
        model->execute();
        model->create_flows();
    } catch (const std::exception& e) {
        log_error(e.what());
        return 253;
    }
    // The reference's statistics lines (src/main.cpp:85-154): phase times in
    // milliseconds, rounded, from the models' microsecond timers; doubles in
    // iostream's default format (%g).
    const char* mat_fmt = " | MATRIX : %d X %d\n";
    const int M = problem.numSupplies, N = problem.numDemands;
    auto ms = [](double us) { return std::round(us / 1000.0); };
    printf("[info] => >>>> BASIC STATISTICS | Objective: %s | Iterations: %d | Time: %g",
           exact_objective(model->objective_scaled, problem.cost_scale).c_str(), model->totalIterations,
           model->totalSolveTime);
    printf(mat_fmt, M, N);
    if (algo == "parallel_uv") {
        printf("[info] => >>>> LVL1 STATISTICS | Total Time: %g | UV Time: %g | R Time: %g | PIVOT Time: %g",
               model->totalSolveTime, ms(model->uv_time), ms(model->reduced_cost_time), ms(model->pivot_time));
        printf(mat_fmt, M, N);
    } else if (algo == "parallel_ss") {
        printf("[info] => >>>> LVL1 STATISTICS | Total Time: %g | PIVOT Time: %g", model->totalSolveTime,
               ms(model->pivot_time));
        printf(mat_fmt, M, N);
    } else {
        printf("[info] => >>>> LVL1 STATISTICS(A) | PIVOT Time: %g", ms(model->pivot_time));
        printf(mat_fmt, M, N);
        printf("[info] => >>>> LVL1 STATISTICS(B) | UV Time: %g | R Time: %g | PIVOT Time: %g", ms(model->uv_time),
               ms(model->reduced_cost_time), ms(model->pivot_time));
        printf(mat_fmt, M, N);
    }
    printf("[info] => >>>> LVL2 PIVOT STATISTICS | Total Pivot Time: %g | %s: %g | RESOLVE Time: %g | ADJUST Time: %g",
           ms(model->pivot_time), algo == "switch_hybrid" ? "CYCLE Time (parallel BFS + seq DFS)" : "CYCLE Time",
           ms(model->cycle_discovery_time), ms(model->resolve_time), ms(model->adjustment_time));
    printf(mat_fmt, M, N);
    // not in the reference: pivots, the exact certificate and the status bits
    printf("[info] => >>>> FLOCK STATISTICS | PIVOTS: %d | CERTIFIED: %d | STATUS: %d", model->stats.pivots,
           model->stats.certified, model->stats.status);
    printf(mat_fmt, M, N);
    printf("[info] => Flows created successfully!\n");
    return model->stats.status ? 1 : 0;
}
