// concurrent_queue.h -- best-first frontier and in-flight bound set
// (reference: include/gpuboscia/concurrent_queue.h:10-123).
#pragma once
#include <mutex>
#include <queue>
#include <set>
#include <vector>

#include "node.h"

// Min-heap on dual_bound; pruned (cut-off) nodes are dropped when popped.
struct ConcurrentQueue {
    void push(Node nd) {
        std::lock_guard<std::mutex> lk(mtx_);
        pq_.push(std::move(nd));
    }

    // Up to n live nodes.
    std::vector<Node> pop_batch(int n, double cutoff) {
        std::lock_guard<std::mutex> lk(mtx_);
        std::vector<Node> batch;
        batch.reserve(n);
        while (!pq_.empty() && (int)batch.size() < n) {
            if (pq_.top().dual_bound >= cutoff) { pq_.pop(); continue; }
            batch.push_back(pq_.top());
            pq_.pop();
        }
        return batch;
    }

    // Exactly n live nodes, or none (the heap is left unchanged apart from
    // dropping cut-off nodes).
    std::vector<Node> pop_full_batch(int n, double cutoff) {
        std::lock_guard<std::mutex> lk(mtx_);
        while (!pq_.empty() && pq_.top().dual_bound >= cutoff) pq_.pop();
        if ((int)pq_.size() < n) return {};
        std::vector<Node> batch;
        batch.reserve(n);
        for (int i = 0; i < n && !pq_.empty(); ++i) {
            if (pq_.top().dual_bound >= cutoff) {
                while (!pq_.empty()) pq_.pop();
                break;
            }
            batch.push_back(pq_.top());
            pq_.pop();
        }
        if ((int)batch.size() < n) {
            for (auto& nd : batch) pq_.push(std::move(nd));
            return {};
        }
        return batch;
    }

    int size() const { std::lock_guard<std::mutex> lk(mtx_); return (int)pq_.size(); }
    bool empty() const { std::lock_guard<std::mutex> lk(mtx_); return pq_.empty(); }

    void discard_children(int parent_id) {
        std::lock_guard<std::mutex> lk(mtx_);
        decltype(pq_) kept;
        while (!pq_.empty()) {
            if (pq_.top().parent_id != parent_id) kept.push(pq_.top());
            pq_.pop();
        }
        pq_.swap(kept);
    }

    double best_bound(double cutoff) const {
        std::lock_guard<std::mutex> lk(mtx_);
        if (pq_.empty()) return cutoff;
        const double b = pq_.top().dual_bound;
        return b < cutoff ? b : cutoff;
    }

private:
    struct MinHeap {
        bool operator()(const Node& a, const Node& b) const { return a.dual_bound > b.dual_bound; }
    };
    mutable std::mutex mtx_;
    std::priority_queue<Node, std::vector<Node>, MinHeap> pq_;
};

// Bounds of nodes taken off the frontier and not yet retired.
struct ConcurrentBoundSet {
    void insert(double b) { std::lock_guard<std::mutex> lk(mtx_); bounds_.insert(b); }
    void insert(const std::vector<Node>& nodes) {
        std::lock_guard<std::mutex> lk(mtx_);
        for (const Node& nd : nodes) bounds_.insert(nd.dual_bound);
    }
    void erase_one(double b) {
        std::lock_guard<std::mutex> lk(mtx_);
        auto it = bounds_.find(b);
        if (it != bounds_.end()) bounds_.erase(it);
    }
    double best_bound(double cutoff) const {
        std::lock_guard<std::mutex> lk(mtx_);
        if (bounds_.empty()) return cutoff;
        const double b = *bounds_.begin();
        return b < cutoff ? b : cutoff;
    }

private:
    mutable std::mutex mtx_;
    std::multiset<double> bounds_;
};
