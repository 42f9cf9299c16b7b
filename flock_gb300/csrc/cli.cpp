// cli.cpp -- `flock -i <file.dat> -a <algo> [-s <decimal scale>]`, the
// reference's command line (src/main.cpp:16-167, src/instance.cpp:6-78) on
// the GPU solver.  Prints the reference's BASIC STATISTICS line, which its
// batch scripts parse.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/flock/algos.h"

static const char* opt_value(int argc, char** argv, const char* key) {
    for (int k = 1; k + 1 < argc; k++) if (!strcmp(argv[k], key)) return argv[k + 1];
    return nullptr;
}

int main(int argc, char** argv) {
    const char* file = opt_value(argc, argv, "-i");
    const char* algo = opt_value(argc, argv, "-a");
    std::string a = algo ? algo : "parallel_uv";
    if (!file) {
        fprintf(stderr, "[error] => Provide input file with argument -i\n");
        return 255;
    }
    ProblemInstance problem;
    try {
        make_problem(file, problem);
    } catch (const FileNotFoundException&) {
        fprintf(stderr, "[error] => File :%s doesn't exist!\n", file);
        return 255;
    } catch (const std::exception& e) {
        fprintf(stderr, "[error] => %s\n", e.what());
        return 254;
    }
    printf("[info] => Problem Dimension => Supplies: %d\tDemands: %d\n", problem.numSupplies, problem.numDemands);
    std::vector<flowInformation> flows((size_t)problem.numSupplies + problem.numDemands - 1);
    flock_detail::ModelBase* model = nullptr;
    if (a == "parallel_uv") model = new uvModel_parallel(&problem, flows.data());
    else if (a == "parallel_ss") model = new ssModel_parallel(&problem, flows.data());
    else if (a == "switch_hybrid") model = new switchModel_parallel(&problem, flows.data());
    else if (a == "cpu_lp_solve") {
        fprintf(stderr, "[error] => cpu_lp_solve needs Gurobi, which this build does not include\n");
        return 254;
    } else {
        fprintf(stderr, "[error] => Invalid Algorithm!\n");
        return 254;
    }
    try {
        model->execute();
        model->create_flows();
    } catch (const std::exception& e) {
        fprintf(stderr, "[error] => %s\n", e.what());
        return 253;
    }
    char obj[64];
    if (problem.cost_scale > 0) {
        long long q = (long long)model->objective_scaled;
        long long p = 1;
        for (int k = 0; k < problem.cost_scale; k++) p *= 10;
        snprintf(obj, sizeof obj, "%s%lld.%0*lld", q < 0 ? "-" : "", (q < 0 ? -q : q) / p, problem.cost_scale,
                 (q < 0 ? -q : q) % p);
    } else {
        snprintf(obj, sizeof obj, "%lld", (long long)model->objective_scaled);
    }
    printf("[info] => >>>> BASIC STATISTICS | Objective: %s | Iterations: %d | Time: %.0f | MATRIX : %d X %d\n", obj,
           model->totalIterations, model->totalSolveTime, problem.numSupplies, problem.numDemands);
    printf("[info] => >>>> LVL1 STATISTICS | Total Time: %.0f | PIVOTS: %d | CERTIFIED: %d | STATUS: %d | MATRIX : %d X %d\n",
           model->totalSolveTime, model->stats.pivots, model->stats.certified, model->stats.status,
           problem.numSupplies, problem.numDemands);
    const int rc = model->stats.status ? 1 : 0;
    delete model;
    return rc;
}
