// The drop-in logger (include/gpuboscia/logger.h) driven the way the
// reference's examples drive it: header, throttled progress rows wired as the
// solver's progress callback would call them, footer with a solution preview.
#include <cstdio>
#include <vector>

#include <gpuboscia/line_search_options.h>
#include <gpuboscia/logger.h>

int main() {
    Logger logger(true, 100);
    LoggerParams lp;
    lp.traversal_strategy = "best_first (shared queue)";
    lp.branching_strategy = "branch_pow2(k=3, binary)";
    lp.algorithm = fw_algorithm_name(FWAlgorithmKind::DICG);
    lp.line_search_method = line_search_name(LineSearchKind::Secant);
    lp.n_vars = 20;
    lp.n_int_vars = 20;
    logger.print_header(lp);
    // processed nodes 0, 40, 80, ... 400; a new incumbent at 120
    for (int i = 0; i <= 400; i += 40) logger.print_row(i, 1000 - i, -1.0 + i * 1e-3, 2.0, i == 120);
    logger.print_stage("done");
    SolutionStats st;
    st.solution_status = "Reached tolerance";
    st.primal_objective = 2.0;
    st.dual_bound = 1.999;
    st.total_nodes = 400;
    st.solution = std::vector<double>(20, 0.0);
    st.solution[3] = st.solution[7] = 1.0;
    logger.print_footer(st);
    Logger quiet(false);
    quiet.print_header(lp);
    quiet.print_row(0, 0, 0.0, 0.0, true);
    quiet.print_footer(st);
    return 0;
}
