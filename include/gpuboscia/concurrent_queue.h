// concurrent_queue.h -- the host frontier: open nodes ordered by dual bound,
// and the bounds of nodes taken off it and not yet retired.
//
// Interface of the reference's include/gpuboscia/concurrent_queue.h:10-123
// (type names, member functions, pruning rules). The frontier here is a
// binary heap kept in a plain vector by the standard heap algorithms, so
// nodes of equal bound leave in the order every std::priority_queue-based
// scheduler produces for the same pushes; a node whose bound reaches the
// cutoff is never handed out. The retired-bound set is a count per distinct
// bound.
#pragma once
#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

#include "node.h"

struct ConcurrentQueue {
    void push(Node nd) {
        std::lock_guard<std::mutex> lk(mtx_);
        insert(std::move(nd));
    }

    // Up to n nodes whose bound is below the cutoff; cut-off nodes met on the
    // way are dropped.
    std::vector<Node> pop_batch(int n, double cutoff) {
        std::lock_guard<std::mutex> lk(mtx_);
        std::vector<Node> out;
        out.reserve(n > 0 ? n : 0);
        while ((int)out.size() < n && !heap_.empty()) {
            Node nd = extract();
            if (nd.dual_bound < cutoff) out.push_back(std::move(nd));
        }
        return out;
    }

    // Exactly n nodes below the cutoff, or none. The frontier is best-first,
    // so the first cut-off node means every node after it is cut off too:
    // those are dropped either way, and a short batch goes back.
    std::vector<Node> pop_full_batch(int n, double cutoff) {
        std::lock_guard<std::mutex> lk(mtx_);
        drop_cut_head(cutoff);
        if ((int)heap_.size() < n) return {};
        std::vector<Node> out;
        out.reserve(n > 0 ? n : 0);
        while ((int)out.size() < n && !heap_.empty() && heap_.front().dual_bound < cutoff) out.push_back(extract());
        if ((int)out.size() == n) return out;
        heap_.clear();
        for (Node& nd : out) insert(std::move(nd));
        return {};
    }

    int size() const {
        std::lock_guard<std::mutex> lk(mtx_);
        return (int)heap_.size();
    }
    bool empty() const {
        std::lock_guard<std::mutex> lk(mtx_);
        return heap_.empty();
    }

    // Removes every queued child of parent_id (children dispatched early whose
    // parent was then invalidated on the host).
    void discard_children(int parent_id) {
        std::lock_guard<std::mutex> lk(mtx_);
        std::vector<Node> rest;
        rest.reserve(heap_.size());
        while (!heap_.empty()) {
            Node nd = extract();
            if (nd.parent_id != parent_id) rest.push_back(std::move(nd));
        }
        for (Node& nd : rest) insert(std::move(nd));
    }

    // The least queued bound, capped at the cutoff (the cutoff when empty).
    double best_bound(double cutoff) const {
        std::lock_guard<std::mutex> lk(mtx_);
        return heap_.empty() ? cutoff : std::min(heap_.front().dual_bound, cutoff);
    }

private:
    // heap order: the front holds the least dual bound
    static bool later(const Node& a, const Node& b) { return a.dual_bound > b.dual_bound; }

    void insert(Node nd) {
        heap_.push_back(std::move(nd));
        std::push_heap(heap_.begin(), heap_.end(), later);
    }
    Node extract() {
        std::pop_heap(heap_.begin(), heap_.end(), later);
        Node nd = std::move(heap_.back());
        heap_.pop_back();
        return nd;
    }
    void drop_cut_head(double cutoff) {
        while (!heap_.empty() && heap_.front().dual_bound >= cutoff) extract();
    }

    mutable std::mutex mtx_;
    std::vector<Node> heap_;
};

// Bounds of the nodes being relaxed or expanded (taken off the frontier, not
// yet retired): the live bound is the least of these and the frontier's.
struct ConcurrentBoundSet {
    void insert(double bound) {
        std::lock_guard<std::mutex> lk(mtx_);
        ++count_[bound];
    }
    void insert(const std::vector<Node>& nodes) {
        std::lock_guard<std::mutex> lk(mtx_);
        for (const Node& nd : nodes) ++count_[nd.dual_bound];
    }
    // Retires one node of this bound (no effect when none is held).
    void erase_one(double bound) {
        std::lock_guard<std::mutex> lk(mtx_);
        auto it = count_.find(bound);
        if (it != count_.end() && --it->second == 0) count_.erase(it);
    }
    double best_bound(double cutoff) const {
        std::lock_guard<std::mutex> lk(mtx_);
        return count_.empty() ? cutoff : std::min(count_.begin()->first, cutoff);
    }

private:
    mutable std::mutex mtx_;
    std::map<double, int> count_;   // distinct bound -> nodes holding it
};
