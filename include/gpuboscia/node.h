// node.h -- B&B node with relaxation continuation (reference: include/gpuboscia/node.h:9-31).
#pragma once
#include <utility>
#include <vector>

enum class NodeStatus { Active, Solved };

struct Node {
    int id;
    int parent_id;
    int depth;
    std::vector<double> lb;
    std::vector<double> ub;
    // A non-empty iterate with zero iterations is a fresh caller-supplied start;
    // with iterations > 0 it resumes an interrupted relaxation.
    std::vector<double> relaxation_x;
    int relaxation_iterations = 0;
    double dual_bound;
    NodeStatus status;

    Node(int id_, int parent_id_, int depth_, std::vector<double> lb_, std::vector<double> ub_)
        : id(id_), parent_id(parent_id_), depth(depth_), lb(std::move(lb_)), ub(std::move(ub_)),
          dual_bound(-1e300), status(NodeStatus::Active) {}
};
