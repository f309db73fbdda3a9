// Progress tables for the examples (include/gpuboscia/logger.h of the
// reference): the same types, fields and calls, so a program that logs its
// search compiles unchanged. The search itself never logs; the caller wires
// Logger::print_row into Settings::progress. Plain host C++.
#pragma once

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <string>
#include <vector>

#include "gap_utils.h"

struct LoggerParams {
    std::string traversal_strategy = "best_first";
    std::string branching_strategy = "branch_pow2";
    std::string algorithm = "Frank-Wolfe";
    std::string line_search_method = "open-loop";
    int n_vars = 0;
    int n_int_vars = 0;
    double abs_gap_tol = 1e-6;
    double rel_gap_tol = 1e-2;
    double time_limit_s = std::numeric_limits<double>::infinity();
    double natural_lower_bound = -std::numeric_limits<double>::infinity();
    std::uint64_t random_seed = 0;
    bool print_random_seed = false;
};

struct SolutionStats {
    std::string solution_status = "Unknown";
    double primal_objective = std::numeric_limits<double>::infinity();
    double dual_bound = -std::numeric_limits<double>::infinity();
    int total_nodes = 0;
    double total_time_s = 0.0;
    std::vector<double> solution;
    int solution_preview_size = 12;
};

class Logger {
public:
    bool enabled;

    // node_interval: a row is printed when the processed-node count has
    // advanced by at least this much since the last row, or the incumbent is new
    explicit Logger(bool on = true, int node_interval = 1000)
        : enabled(on), interval_(std::max(1, node_interval)), start_(std::chrono::steady_clock::now()) {}

    void print_header(const LoggerParams& p) {
        if (!enabled) return;
        rule();
        std::printf("variables %d (integer %d)  algorithm %s  line search %s\n", p.n_vars, p.n_int_vars,
                    p.algorithm.c_str(), p.line_search_method.c_str());
        std::printf("traversal %s  branching %s\n", p.traversal_strategy.c_str(), p.branching_strategy.c_str());
        std::printf("gap tolerance abs %s rel %s  time limit %s  natural bound %s\n", num(p.abs_gap_tol).c_str(),
                    num(p.rel_gap_tol).c_str(), std::isfinite(p.time_limit_s) ? num(p.time_limit_s).c_str() : "none",
                    num(p.natural_lower_bound).c_str());
        if (p.print_random_seed) std::printf("seed %llu\n", (unsigned long long)p.random_seed);
        rule();
        std::printf("  %-2s %10s %10s %14s %14s %10s %10s %9s\n", "", "nodes", "open", "bound", "incumbent",
                    "gap", "rel gap", "time s");
        rule();
    }

    void print_stage(const char* stage) {
        if (!enabled) return;
        std::printf("-- %s (%.3f s)\n", stage, elapsed());
    }

    void print_row(int iter, int open_nodes, double dual_bound, double incumbent, bool is_new_incumbent = false) {
        if (!enabled) return;
        if (!is_new_incumbent && iter - last_ < interval_ && iter != 0) return;
        last_ = iter;
        std::printf("  %-2s %10d %10d %14s %14s %10s %10s %9.3f\n", is_new_incumbent ? "*" : "", iter, open_nodes,
                    num(dual_bound).c_str(), num(incumbent).c_str(),
                    num(gpuboscia::gap_absolute(dual_bound, incumbent)).c_str(),
                    num(gpuboscia::gap_relative(dual_bound, incumbent)).c_str(), elapsed());
    }

    void print_footer(const SolutionStats& s) {
        if (!enabled) return;
        rule();
        std::printf("status %s\n", s.solution_status.c_str());
        std::printf("objective %s  bound %s  rel gap %s\n", num(s.primal_objective).c_str(), num(s.dual_bound).c_str(),
                    num(gpuboscia::gap_relative(s.dual_bound, s.primal_objective)).c_str());
        std::printf("nodes %d  time %.3f s\n", s.total_nodes, s.total_time_s);
        if (!s.solution.empty()) {
            int nonzeros = 0;
            for (double v : s.solution) nonzeros += v != 0.0;
            const int shown = std::min<int>(std::max(0, s.solution_preview_size), (int)s.solution.size());
            std::printf("solution (%d of %zu entries nonzero):", nonzeros, s.solution.size());
            for (int i = 0; i < shown; ++i) std::printf(" %g", s.solution[i]);
            std::printf("%s\n", shown < (int)s.solution.size() ? " ..." : "");
        }
        rule();
    }

private:
    int interval_;
    int last_ = 0;
    std::chrono::steady_clock::time_point start_;

    double elapsed() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - start_).count();
    }
    static std::string num(double v) {
        if (std::isnan(v)) return "nan";
        if (std::isinf(v)) return v > 0 ? "inf" : "-inf";
        char b[32];
        std::snprintf(b, sizeof b, "%.6e", v);
        return b;
    }
    static void rule() { std::printf("%s\n", std::string(92, '-').c_str()); }
};
