// atomic_incumbent.h -- best integer solution (reference: include/gpuboscia/atomic_incumbent.h:10-35).
#pragma once
#include <atomic>
#include <limits>
#include <mutex>
#include <vector>

struct AtomicIncumbent {
    std::atomic<double> value{std::numeric_limits<double>::infinity()};
    std::vector<double> x;
    mutable std::mutex x_mtx;

    // True when val improves the incumbent.
    bool try_update(double val, const std::vector<double>& new_x) {
        double old = value.load(std::memory_order_relaxed);
        while (val < old) {
            if (value.compare_exchange_weak(old, val, std::memory_order_acq_rel, std::memory_order_relaxed)) {
                std::lock_guard<std::mutex> lk(x_mtx);
                x = new_x;
                return true;
            }
        }
        return false;
    }
    double get() const { return value.load(std::memory_order_acquire); }
    std::vector<double> get_x() const { std::lock_guard<std::mutex> lk(x_mtx); return x; }
};
