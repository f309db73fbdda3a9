// atomic_incumbent.h -- the best integer solution found so far.
//
// Interface of the reference's include/gpuboscia/atomic_incumbent.h:10-35
// (members value, x, x_mtx; try_update, get, get_x). Pruning reads `value`
// without a lock. An improvement takes the mutex, re-checks under it and
// publishes the point before the value, so a reader that sees a value also
// finds its point (or a better one) behind get_x().
#pragma once
#include <atomic>
#include <limits>
#include <mutex>
#include <vector>

struct AtomicIncumbent {
    std::atomic<double> value{std::numeric_limits<double>::infinity()};
    std::vector<double> x;
    mutable std::mutex x_mtx;

    // True when val is strictly below the incumbent (which it then becomes).
    bool try_update(double val, const std::vector<double>& new_x) {
        if (!(val < value.load(std::memory_order_acquire))) return false;
        std::lock_guard<std::mutex> lk(x_mtx);
        if (!(val < value.load(std::memory_order_relaxed))) return false;
        x = new_x;
        value.store(val, std::memory_order_release);
        return true;
    }

    double get() const { return value.load(std::memory_order_acquire); }

    std::vector<double> get_x() const {
        std::lock_guard<std::mutex> lk(x_mtx);
        return x;
    }
};
