// flock/structs.h -- the reference's problem container and flow record
// (src/structs.h:19-52, src/structs.cpp:3-29) over the flock C ABI.
//
// Differences from the reference, by design: costs are exact integers
// (ProblemInstance::int_costs = cost * 10^cost_scale; the float `costs` array
// is kept for source compatibility) and the members start initialised.
#pragma once
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../flock.h"
#include "parameters.h"

// A failed library call: the flock_status and flock_last_error()'s message
// (the reference exits the process instead, parallel_structs.h:96-104).
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
        free(supplies); free(demands); free(costs);
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

inline std::ostream& operator<<(std::ostream& o, const flowInformation& x) {
    o << "Flow - " << x.qty << " units from source/rowNo: " << x.source << " to destination/colNo: " << x.destination;
    return o;
}
