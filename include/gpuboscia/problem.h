// problem.h -- B&B problem description (reference: include/gpuboscia/problem.h:4-9).
#pragma once
#include <vector>

struct Problem {
    int n_vars = 0;
    std::vector<double> lb;
    std::vector<double> ub;
    std::vector<int> int_vars;
};
