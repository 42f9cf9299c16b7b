// flock/instance.h -- the reference's command-line parser and instance reader
// (src/instance.h:1-48, src/instance.cpp:6-179): `-i <file>` and
// `-a <algorithm>`, `.dat` files read through the flock C ABI with exact
// decimal costs.
#pragma once
#include "logger.h"
#include "structs.h"

struct FileNotFoundException : public std::exception {
    const char* what() const throw() { return "File not found!"; }
};

class InputParser {
public:
    InputParser(int& argc, char** argv) {
        for (int i = 1; i < argc; ++i) tokens.push_back(std::string(argv[i]));
    }
    // The argument after `option`, or "" when the option is absent or last.
    const std::string& getCmdOption(const std::string& option) const {
        auto it = std::find(tokens.begin(), tokens.end(), option);
        if (it != tokens.end() && ++it != tokens.end()) return *it;
        static const std::string empty;
        return empty;
    }
    bool cmdOptionExists(const std::string& option) const {
        return std::find(tokens.begin(), tokens.end(), option) != tokens.end();
    }

private:
    std::vector<std::string> tokens;
};

// `-i <file>`: a missing option or an empty name throws FileNotFoundException.
inline void get_input_mode_and_filename(InputParser input, ProblemInstance& problem) {
    problem.read_mode = input.cmdOptionExists("-i");
    problem.filename = problem.read_mode ? input.getCmdOption("-i") : std::string();
    if (problem.filename.empty()) {
        add_log_msg("error", problem.read_mode ? "No file name given after -i" : "Provide input file with argument -i");
        throw FileNotFoundException();
    }
    add_log_msg("info", "File Name = " + problem.filename);
}

// `-a <algorithm>` (default cpu_lp_solve, as the reference); an unknown name
// is logged and leaves `algo` as it was.
inline void get_algorithm(InputParser input, ProblemInstance& problem) {
    std::string a = input.cmdOptionExists("-a") ? input.getCmdOption("-a") : std::string();
    if (a.empty()) a = "cpu_lp_solve";
    if (a == "cpu_lp_solve") problem.algo = ProblemInstance::cpu_lp_solve;
    else if (a == "parallel_uv") problem.algo = ProblemInstance::parallel_uv;
    else if (a == "parallel_ss") problem.algo = ProblemInstance::parallel_ss;
    else if (a == "switch_hybrid") problem.algo = ProblemInstance::switch_hybrid;
    else add_log_msg("error", "Invalid Algorithm!");
}

// The .dat reader (readSize / readCosts): shape, the smallest decimal scale
// that makes every cost an integer, then supplies, demands and exact costs.
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

// make_problem(input, problem) of src/instance.cpp:149-179: file name, read,
// algorithm, read time.
inline void make_problem(InputParser input, ProblemInstance& problem) {
    const auto t0 = std::chrono::high_resolution_clock::now();
    get_input_mode_and_filename(input, problem);
    if (!std::ifstream(problem.filename).good()) {
        add_log_msg("error", "File :" + problem.filename + " doesn't exist!");
        throw FileNotFoundException();
    }
    make_problem(problem.filename, problem);
    get_algorithm(input, problem);
    problem.readTime += std::chrono::duration_cast<std::chrono::milliseconds>(
                            std::chrono::high_resolution_clock::now() - t0).count();
}
