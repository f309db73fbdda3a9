// node_select.h -- batch selection policies over a list of open nodes
// (reference: include/gpuboscia/node_select.h): the indices of the
// min(batch_size, size) nodes with the lowest dual bound (best first) or the
// greatest depth (depth first), in that order.
#pragma once
#include <algorithm>
#include <functional>
#include <numeric>
#include <vector>

#include "node.h"

using NodeSelector = std::function<std::vector<int>(const std::vector<Node>&, int)>;

namespace gpuboscia_detail {
template <class Before>
inline std::vector<int> select_first(const std::vector<Node>& nodes, int batch_size, Before before) {
    std::vector<int> idx(nodes.size());
    std::iota(idx.begin(), idx.end(), 0);
    const int take = std::max(0, std::min(batch_size, (int)nodes.size()));
    std::partial_sort(idx.begin(), idx.begin() + take, idx.end(), before);
    idx.resize(take);
    return idx;
}
}  // namespace gpuboscia_detail

inline std::vector<int> best_first(const std::vector<Node>& nodes, int batch_size) {
    return gpuboscia_detail::select_first(nodes, batch_size,
                                          [&](int a, int b) { return nodes[a].dual_bound < nodes[b].dual_bound; });
}

inline std::vector<int> depth_first(const std::vector<Node>& nodes, int batch_size) {
    return gpuboscia_detail::select_first(nodes, batch_size,
                                          [&](int a, int b) { return nodes[a].depth > nodes[b].depth; });
}
