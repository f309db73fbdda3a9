// device_resident_solver.h -- host branch-and-bound scheduler over the GB300
// relaxation library (reference: include/gpuboscia/device_resident_solver.cuh:1002-2086).
//
// The scheduling semantics are the reference's: best-first batches of up to
// gpu_batch_size nodes, num_streams batches in flight, a completed batch's
// slot is refilled before its results are post-processed, an empty frontier
// is refilled by branching completed nodes early, near-integral nodes without
// a certificate are requeued with their iterate (continuation), and the FW
// lower bound f - gap is trusted only for a finite non-negative gap.
//
// What differs is the mechanism. The reference spawns a std::thread per
// launch that issues 8 H2D copies, the kernel, 7 D2H copies and a host
// callback. Here each slot owns one pinned and one device block laid out so a
// batch is one H2D copy, one gbx_relax_batch() launch and one D2H copy,
// followed by an event the scheduler polls; no thread is created per batch.
// After the search completes, batches still in flight are awaited and
// post-processed, so a run with num_streams == 1 is deterministic.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <unordered_set>
#include <utility>
#include <vector>

#include "../gpuboscia_gb300.h"
#include "algorithms.h"
#include "atomic_incumbent.h"
#include "bnb.h"
#include "nvtx.h"
#include "branching.h"
#include "concurrent_queue.h"
#include "dense_quadratic_objectives.h"
#include "gap_utils.h"
#include "heuristics.h"
#include "lmo.h"
#include "node.h"
#include "problem.h"

#define GBX_CUDA_CHECK(call)                                                              \
    do {                                                                                  \
        cudaError_t _e = (call);                                                          \
        if (_e != cudaSuccess)                                                            \
            throw std::runtime_error(std::string("CUDA ") + __FILE__ + ":" +              \
                                     std::to_string(__LINE__) + " - " + cudaGetErrorString(_e)); \
    } while (0)

// The reference's name for the same check (device_resident_solver.cuh:114-122),
// for programs that use it around their own CUDA calls.
#ifndef DRS_CUDA_CHECK
#define DRS_CUDA_CHECK(call) GBX_CUDA_CHECK(call)
#endif

// Per-node status bytes of a relaxation (device_resident_solver.cuh:192-202):
// the C ABI's GBX_NODE_* values under the reference's names.
enum DRSNodeState : uint8_t {
    DRSFractionalUnconverged = GBX_NODE_FRACTIONAL_UNCONVERGED,
    DRSFractionalConverged = GBX_NODE_FRACTIONAL_CONVERGED,
    DRSInfeasible = GBX_NODE_INFEASIBLE,
    DRSIntegralUnconverged = GBX_NODE_INTEGRAL_UNCONVERGED,
    DRSIntegralConverged = GBX_NODE_INTEGRAL_CONVERGED
};
// input flag: the node's x holds a start point (a warm start or a continuation)
constexpr uint8_t DRSInitialPointSupplied = GBX_NODE_INITIAL_POINT_SUPPLIED;

enum class FWExecutionMode { SingleBlock, MultiBlock };

struct DeviceResidentConfig {
    enum class DICGOracleParallelism { Auto, Serial, Paired };
    int gpu_batch_size = 1024;
    int num_streams = 8;
    int gpu_block_threads = 0;  // accepted for source compatibility; the kernel uses 256
    int gpu_max_iters = 20000;
    double gpu_eps = 1e-3;
    double gpu_eps_decay = 0.8;
    double gpu_eps_min = 1e-6;
    double integer_tol = 1e-6;
    double abs_gap_tol = 1e-6;
    double rel_gap_tol = 1e-2;
    DICGOracleParallelism dicg_oracle_parallelism = DICGOracleParallelism::Auto;
    double dicg_paired_occupancy_fraction = 0.8;
    FWExecutionMode execution_mode = FWExecutionMode::SingleBlock;
    int blocks_per_node = 4;
    // appended GB300 fields
    int precision = GBX_PRECISION_FP64;
    bool use_cuda_graph = true;  // replay each slot's copy-relax-copy sequence from a CUDA graph
    bool autotune = true;        // time the launch shapes on the first full batch (gbx_relax_autotune)
    // frontier in device memory: every round of the search runs as kernels
    // (gbx_solve with gbx_settings.device_frontier); branching is branch_pow2
    // over branch_k variables and the BranchStrategy callback is not called
    bool device_frontier = false;
    int frontier_capacity = 0;   // open nodes in the device pool (0: automatic)
    int frontier_slots = 2;      // batches in flight on the device frontier (1 or 2)
    int branch_k = 3;
    // stop a node's relaxation once its FW bound clears the incumbent
    // (gbx_node_batch.cutoff): the node is pruned at any bound above it
    bool incumbent_cutoff = false;
    // stop once this many nodes are processed (0: no limit; no counterpart in
    // the reference): the search ends with the batch that reaches it, and the
    // reported dual bound is the live bound at that point
    int node_limit = 0;
};

enum class DRSSchedulingEventType { Dispatched, CompletionDetached, PostprocessStarted };

struct DRSSchedulingEvent {
    DRSSchedulingEventType type;
    int slot_id;
    std::uint64_t generation;
    int n_nodes;
};

namespace gpuboscia {

// How the engine relaxes a batch when the objective is not a built-in kind:
// the workspace it needs and the launch (user_relax.cuh provides both for
// user-written device objectives). Empty: the library's gbx_relax_batch.
struct RelaxHooks {
    std::function<size_t(const gbx_lmo&, int)> workspace_bytes;
    std::function<int(const gbx_lmo&, const gbx_algorithm&, const gbx_node_batch&, void*, size_t, cudaStream_t)>
        launch;
};

// Built-in objective kinds describe themselves to the C ABI (descriptor());
// any other objective type is a user-written device objective.
template <class T, class = void>
struct HasDescriptor : std::false_type {};
template <class T>
struct HasDescriptor<T, std::void_t<decltype(std::declval<const T&>().descriptor())>> : std::true_type {};

// The relaxation of a user objective type: defined by <gpuboscia/user_relax.cuh>,
// which the translation unit that calls solve() with such a type must include
// (compiled by nvcc).
template <class Obj, class = void>
struct UserRelax;

namespace detail {

inline void gbx_check(int rc, const char* what) {
    if (rc != GBX_OK) {
        const char* m = gbx_last_error();
        const std::string msg = std::string(what) + ": " + (m ? m : "");
        if (rc == GBX_ERR_INVALID || rc == GBX_ERR_UNSUPPORTED) throw std::invalid_argument(msg);
        throw std::runtime_error(msg);
    }
}

class BnBEngine {
public:
    BnBEngine(const Problem& prob, const gbx_objective& obj, const LMOSpec& lmo, const gbx_algorithm& alg,
              BranchStrategy branch, DeviceResidentConfig cfg, double time_limit_seconds, RelaxHooks hooks = {})
        : prob_(prob), obj_(obj), lmo_spec_(lmo), alg_(alg), branch_sel_(std::move(branch)), cfg_(cfg),
          time_limit_seconds_(time_limit_seconds), hooks_(std::move(hooks)) {
        if (cfg_.gpu_max_iters <= 0 || cfg_.gpu_batch_size <= 0 || cfg_.num_streams <= 0)
            throw std::invalid_argument("GPU iterations, batch size and streams must be positive");
        for (int j : prob_.int_vars)
            if (j < 0 || j >= prob_.n_vars) throw std::invalid_argument("integer variable index out of range");
        if (!std::isfinite(cfg_.gpu_eps) || cfg_.gpu_eps <= 0.0 || !std::isfinite(cfg_.gpu_eps_min)
                || cfg_.gpu_eps_min <= 0.0 || !std::isfinite(cfg_.gpu_eps_decay) || cfg_.gpu_eps_decay <= 0.0
                || cfg_.gpu_eps_decay > 1.0 || !std::isfinite(cfg_.abs_gap_tol) || cfg_.abs_gap_tol < 0.0
                || !std::isfinite(cfg_.rel_gap_tol) || cfg_.rel_gap_tol < 0.0
                || !std::isfinite(cfg_.dicg_paired_occupancy_fraction)
                || cfg_.dicg_paired_occupancy_fraction <= 0.0 || cfg_.dicg_paired_occupancy_fraction > 1.0)
            throw std::invalid_argument("invalid tolerance configuration");
        if (std::isnan(time_limit_seconds_) || time_limit_seconds_ <= 0.0)
            throw std::invalid_argument("time limit must be positive");
        if (cfg_.node_limit < 0) throw std::invalid_argument("node_limit must be non-negative");
        if (cfg_.gpu_block_threads != 0 && (cfg_.gpu_block_threads < 32 || cfg_.gpu_block_threads % 32 != 0))
            throw std::invalid_argument("gpu_block_threads must be zero or a positive multiple of 32");
        if (obj_.n != prob_.n_vars)
            throw std::runtime_error("DeviceObjective::n_vars does not match Problem::n_vars");
        if (cfg_.execution_mode == FWExecutionMode::MultiBlock && cfg_.blocks_per_node < 1)
            throw std::invalid_argument("MultiBlock blocks_per_node must be positive");
        alg_.precision = cfg_.precision;
        if (hooks_.launch) {
            if (cfg_.precision != GBX_PRECISION_FP64)
                throw std::invalid_argument("mixed precision covers the built-in graph-matching objective only");
            if (cfg_.device_frontier)
                throw std::invalid_argument("the device frontier relaxes the built-in objective kinds only");
        }
        const int n = prob_.n_vars;
        lmo_ = gbx_lmo{};
        lmo_.kind = lmo_spec_.kind;
        lmo_.n = n;
        lmo_.right_side = lmo_spec_.right_side;
        lmo_.order = lmo_spec_.order;
        lmo_.upper = lmo_spec_.upper;
        std::vector<uint8_t> flags(n, 0);
        for (int j : prob_.int_vars) flags[j] = 1;
        GBX_CUDA_CHECK(cudaMalloc(&d_flags_, std::max<size_t>(n, 1)));
        GBX_CUDA_CHECK(cudaMemcpy(d_flags_, flags.data(), n, cudaMemcpyHostToDevice));
        if (!lmo_spec_.is_int.empty()) {
            GBX_CUDA_CHECK(cudaMalloc(&d_lmo_is_int_, n));
            GBX_CUDA_CHECK(cudaMemcpy(d_lmo_is_int_, lmo_spec_.is_int.data(), n, cudaMemcpyHostToDevice));
            lmo_.is_int = d_lmo_is_int_;
        }
        ws_bytes_ = hooks_.launch ? hooks_.workspace_bytes(lmo_, cfg_.gpu_batch_size)
                                  : gbx_relax_workspace_bytes(&obj_, &lmo_, &alg_, cfg_.gpu_batch_size);
        if (ws_bytes_ == 0) gbx_check(GBX_ERR_INVALID, "gbx_relax_workspace_bytes");
        slots_.resize(cfg_.num_streams);
        for (int i = 0; i < cfg_.num_streams; ++i) alloc_slot(slots_[i], i);
    }

    BnBEngine(const BnBEngine&) = delete;
    BnBEngine& operator=(const BnBEngine&) = delete;

    virtual ~BnBEngine() {
        for (auto& s : slots_) free_slot(s);
        if (d_flags_) cudaFree(d_flags_);
        if (d_lmo_is_int_) cudaFree(d_lmo_is_int_);
    }

    void push(const Node& nd) {
        if (nd.lb.size() != (size_t)prob_.n_vars || nd.ub.size() != nd.lb.size()
                || (!nd.relaxation_x.empty() && nd.relaxation_x.size() != nd.lb.size())
                || (nd.relaxation_iterations > 0 && nd.relaxation_x.empty()) || nd.relaxation_iterations < 0)
            throw std::invalid_argument("invalid node buffer dimensions or resume state");
        for (size_t j = 0; j < nd.relaxation_x.size(); ++j)
            if (!std::isfinite(nd.relaxation_x[j]) || nd.relaxation_x[j] < nd.lb[j] - 1e-9
                    || nd.relaxation_x[j] > nd.ub[j] + 1e-9)
                throw std::invalid_argument("initial/resumed node iterate violates finite bounds");
        queue_.push(nd);
    }

    void set_progress_callback(std::function<void(int, int, double, double, bool)> cb) { progress_cb_ = std::move(cb); }
    void set_scheduling_callback(std::function<void(const DRSSchedulingEvent&)> cb) { scheduling_cb_ = std::move(cb); }
    // Children get ids next_id .. next_id + stride - 1 per expansion (8 in the reference).
    void set_child_id_stride(int s) { id_stride_ = std::max(1, s); }
    // Called with every completed batch before any of its nodes is branched
    // (nodes, x [N*n], gap, value, status), so that a branching rule can score
    // all candidates of the batch in one device call.
    using BranchBatchHook = std::function<void(int, const Node*, const double*, const double*, const double*,
                                               const uint8_t*)>;
    void set_branch_batch_hook(BranchBatchHook h) { branch_hook_ = std::move(h); }

    void solve() {
        solve_started_ = Clock::now();
        if (cfg_.device_frontier) {
            solve_device_frontier();
            return;
        }
        gpu_worker();
        for (auto& s : slots_) if (s.stream) GBX_CUDA_CHECK(cudaStreamSynchronize(s.stream));
        if (final_dual_bound_ == -std::numeric_limits<double>::infinity())
            final_dual_bound_ = queue_.best_bound(incumbent_.get());
    }

    double incumbent_value() const { return incumbent_.get(); }
    std::vector<double> incumbent_x() const { return incumbent_.get_x(); }
    int nodes_processed() const { return nodes_done_.load(); }
    double dual_bound() const { return final_dual_bound_; }
    int last_gpu_iterations() const { return last_gpu_iterations_.load(); }
    double last_gpu_gap() const { return last_gpu_gap_.load(); }
    bool last_gpu_converged() const { return last_gpu_converged_.load(); }
    bool reached_tolerance() const { return reached_tolerance_; }
    bool reached_time_limit() const { return reached_time_limit_; }
    bool reached_node_limit() const { return reached_node_limit_; }
    int effective_gpu_batch_size() const { return cfg_.gpu_batch_size; }
    int effective_num_streams() const { return cfg_.num_streams; }
    // Batches whose forward and in-face oracles ran concurrently in one launch.
    int paired_gpu_batches() const { return paired_gpu_batches_.load(std::memory_order_relaxed); }
    long long gpu_batches() const { return batches_launched_; }
    long long gpu_nodes_relaxed() const { return nodes_launched_; }

private:
    using Clock = std::chrono::steady_clock;

    struct Slot {
        int id = -1;
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        int n_nodes = 0;
        bool in_use = false;
        std::uint64_t generation = 0;
        std::uint64_t seq = 0;
        std::vector<std::pair<int, cudaGraphExec_t>> graphs;
        bool graphs_failed = false;
        std::vector<Node> nodes;
        unsigned char* h = nullptr;
        unsigned char* d = nullptr;
        void* ws = nullptr;
        // byte offsets of the current batch
        size_t o_lb = 0, o_ub = 0, o_eps = 0, o_cut = 0, o_x = 0, o_it = 0, o_st = 0, o_gap = 0, o_val = 0,
               o_bvv = 0, o_best = 0, end = 0;
    };

    struct Completed {
        int slot_id = -1;
        std::uint64_t generation = 0;
        std::vector<Node> nodes;
        std::vector<double> x, gap, value, best_vertex, best_vertex_val, lower_bound;
        std::vector<int> iterations;
        std::vector<uint8_t> status, branched_early;
    };

    static size_t a8(size_t v) { return (v + 7) & ~size_t(7); }

    void layout(Slot& s, int N) const {
        const size_t n = (size_t)prob_.n_vars, vb = N * n * sizeof(double), sb = N * sizeof(double);
        size_t p = 0;
        s.o_lb = p; p += vb;
        s.o_ub = p; p += vb;
        s.o_eps = p; p += sb;
        s.o_cut = p; p += sizeof(double);   // incumbent at dispatch (the cutoff)
        s.o_x = p; p += vb;
        s.o_it = p; p += a8(N * sizeof(int));
        s.o_st = p; p += a8((size_t)N);
        s.o_gap = p; p += sb;
        s.o_val = p; p += sb;
        s.o_bvv = p; p += sb;
        s.o_best = p; p += vb;
        s.end = p;
    }

    // Graph of one dispatch of N nodes on this slot (H2D, relaxation, D2H),
    // captured on first use; a few sizes are kept per slot.
    cudaGraphExec_t slot_graph(Slot& s, int N, const gbx_node_batch& b) {
        for (auto& g : s.graphs) if (g.first == N) return g.second;
        if (s.graphs_failed) return nullptr;
        cudaGraph_t graph = nullptr;
        if (cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            s.graphs_failed = true;
            cudaGetLastError();
            return nullptr;
        }
        cudaMemcpyAsync(s.d, s.h, s.o_gap, cudaMemcpyHostToDevice, s.stream);
        const int rc = relax_call(b, s);
        cudaMemcpyAsync(s.h + s.o_x, s.d + s.o_x, s.end - s.o_x, cudaMemcpyDeviceToHost, s.stream);
        const cudaError_t e = cudaStreamEndCapture(s.stream, &graph);
        cudaGraphExec_t exec = nullptr;
        if (rc != GBX_OK || e != cudaSuccess || !graph || cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            s.graphs_failed = true;   // fall back to direct launches on this slot
            cudaGetLastError();
            return nullptr;
        }
        cudaGraphDestroy(graph);
        if (s.graphs.size() >= 4) {
            cudaGraphExecDestroy(s.graphs.front().second);
            s.graphs.erase(s.graphs.begin());
        }
        s.graphs.push_back({N, exec});
        return exec;
    }

    void alloc_slot(Slot& s, int id) {
        s.id = id;
        layout(s, cfg_.gpu_batch_size);
        const size_t bytes = s.end;
        GBX_CUDA_CHECK(cudaHostAlloc(&s.h, bytes, cudaHostAllocDefault));
        GBX_CUDA_CHECK(cudaMalloc(&s.d, bytes));
        GBX_CUDA_CHECK(cudaMalloc(&s.ws, ws_bytes_));
        GBX_CUDA_CHECK(cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking));
        GBX_CUDA_CHECK(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    }

    static void free_slot(Slot& s) {
        if (s.stream) cudaStreamSynchronize(s.stream);
        for (auto& g : s.graphs) cudaGraphExecDestroy(g.second);
        if (s.done) cudaEventDestroy(s.done);
        if (s.stream) cudaStreamDestroy(s.stream);
        if (s.h) cudaFreeHost(s.h);
        if (s.d) cudaFree(s.d);
        if (s.ws) cudaFree(s.ws);
        s = Slot{};
    }

    template <class T>
    static T* at(unsigned char* base, size_t off) { return reinterpret_cast<T*>(base + off); }

    double node_tolerance(const Node& nd) const {
        return depth_dependent_tolerance(cfg_.gpu_eps, cfg_.gpu_eps_decay, cfg_.gpu_eps_min, nd.depth);
    }
    bool should_prune(const Node& nd) const { return nd.dual_bound >= incumbent_.get(); }
    // one batch relaxation on the slot's stream: the library's kernel, or the
    // user objective's template kernel
    int relax_call(const gbx_node_batch& b, Slot& s) {
        if (hooks_.launch) return hooks_.launch(lmo_, alg_, b, s.ws, ws_bytes_, s.stream);
        return gbx_relax_batch(&obj_, &lmo_, &alg_, &b, s.ws, ws_bytes_, s.stream);
    }
    double global_live_bound(double inc) const {
        return std::min(queue_.best_bound(inc), active_bounds_.best_bound(inc));
    }
    bool has_dispatchable_slot() const {
        for (const auto& s : slots_) if (!s.in_use) return true;
        return false;
    }

    void emit_scheduling_event(DRSSchedulingEventType t, int slot, std::uint64_t gen, int n) {
        if (scheduling_cb_) scheduling_cb_({t, slot, gen, n});
    }
    void emit_progress(int iter, bool fresh) {
        if (!progress_cb_) return;
        const double inc = incumbent_.get();
        progress_cb_(iter, queue_.size() + active_tasks_.load(std::memory_order_acquire),
                     global_live_bound(inc), inc, fresh);
    }
    void signal_done() { done_.store(true, std::memory_order_release); }

    bool finish_if_time_limit_reached() {
        if (!std::isfinite(time_limit_seconds_)) return false;
        const double el = std::chrono::duration<double>(Clock::now() - solve_started_).count();
        if (el < time_limit_seconds_) return false;
        final_dual_bound_ = global_live_bound(incumbent_.get());
        reached_time_limit_ = true;
        signal_done();
        return true;
    }

    // the node limit ends the search like a time limit: live bound, no tolerance
    bool finish_if_node_limit_reached() {
        if (cfg_.node_limit <= 0 || nodes_done_.load() < cfg_.node_limit) return false;
        final_dual_bound_ = global_live_bound(incumbent_.get());
        reached_node_limit_ = true;
        signal_done();
        return true;
    }

    bool finish_if_search_complete() {
        if (done_.load(std::memory_order_acquire)) return true;
        if (queue_.empty() && active_tasks_.load(std::memory_order_acquire) == 0) {
            final_dual_bound_ = incumbent_.get();
            signal_done();
            return true;
        }
        const double inc = incumbent_.get();
        const double bound = global_live_bound(inc);
        if (gap_within_tolerance(bound, inc, cfg_.abs_gap_tol, cfg_.rel_gap_tol)) {
            final_dual_bound_ = bound;
            reached_tolerance_ = true;
            signal_done();
            return true;
        }
        return false;
    }

    void submit_slot(Slot& s, std::vector<Node> batch) {
        detail::NvtxRange range("gbx.dispatch");
        const int n = prob_.n_vars;
        const int N = (int)batch.size();
        layout(s, N);
        s.nodes = std::move(batch);
        s.n_nodes = N;
        s.in_use = true;
        ++s.generation;
        s.seq = ++submit_seq_;
        double* lb = at<double>(s.h, s.o_lb);
        double* ub = at<double>(s.h, s.o_ub);
        double* eps = at<double>(s.h, s.o_eps);
        double* x = at<double>(s.h, s.o_x);
        int* it = at<int>(s.h, s.o_it);
        uint8_t* st = at<uint8_t>(s.h, s.o_st);
        for (int i = 0; i < N; ++i) {
            const Node& nd = s.nodes[i];
            std::memcpy(lb + (size_t)i * n, nd.lb.data(), n * sizeof(double));
            std::memcpy(ub + (size_t)i * n, nd.ub.data(), n * sizeof(double));
            std::memcpy(x + (size_t)i * n, nd.relaxation_x.empty() ? nd.lb.data() : nd.relaxation_x.data(),
                        n * sizeof(double));
            eps[i] = node_tolerance(nd);
            it[i] = nd.relaxation_iterations;
            st[i] = nd.relaxation_x.empty() ? 0 : GBX_NODE_INITIAL_POINT_SUPPLIED;
        }
        *at<double>(s.h, s.o_cut) = incumbent_.get();
        gbx_node_batch b{};
        b.n_nodes = N;
        b.max_iters = cfg_.gpu_max_iters;
        b.candidate_tol = cfg_.integer_tol;
        b.x = at<double>(s.d, s.o_x);
        b.lb = at<double>(s.d, s.o_lb);
        b.ub = at<double>(s.d, s.o_ub);
        b.eps = at<double>(s.d, s.o_eps);
        b.iterations = at<int>(s.d, s.o_it);
        b.status = at<uint8_t>(s.d, s.o_st);
        b.gap = at<double>(s.d, s.o_gap);
        b.value = at<double>(s.d, s.o_val);
        b.best_vertex = at<double>(s.d, s.o_best);
        b.best_vertex_val = at<double>(s.d, s.o_bvv);
        b.integer_flags = d_flags_;
        b.cutoff = cfg_.incumbent_cutoff ? at<double>(s.d, s.o_cut) : nullptr;
        if (cfg_.autotune && !tuned_ && N == cfg_.gpu_batch_size && !hooks_.launch) {
            // once, on the first full batch: the tuner relaxes it under every launch
            // shape and restores it, and later launches (and graphs) use the winner
            tuned_ = true;
            GBX_CUDA_CHECK(cudaMemcpyAsync(s.d, s.h, s.o_gap, cudaMemcpyHostToDevice, s.stream));
            gbx_check(gbx_relax_autotune(&obj_, &lmo_, &alg_, &b, s.ws, ws_bytes_, s.stream, 2, nullptr),
                      "gbx_relax_autotune");
        }
        cudaGraphExec_t exec = cfg_.use_cuda_graph ? slot_graph(s, N, b) : nullptr;
        if (exec) {
            detail::NvtxRange r("gbx.graph_replay");   // upload, relaxation, download
            GBX_CUDA_CHECK(cudaGraphLaunch(exec, s.stream));
        } else {
            {
                detail::NvtxRange r("gbx.h2d");
                GBX_CUDA_CHECK(cudaMemcpyAsync(s.d, s.h, s.o_gap, cudaMemcpyHostToDevice, s.stream));
            }
            {
                detail::NvtxRange r("gbx.relax");
                gbx_check(relax_call(b, s), "gbx_relax_batch");
            }
            detail::NvtxRange r("gbx.d2h");
            GBX_CUDA_CHECK(cudaMemcpyAsync(s.h + s.o_x, s.d + s.o_x, s.end - s.o_x, cudaMemcpyDeviceToHost,
                                           s.stream));
        }
        GBX_CUDA_CHECK(cudaEventRecord(s.done, s.stream));
        ++batches_launched_;
        nodes_launched_ += N;
        if (alg_.kind == GBX_ALG_DICG && lmo_.kind == GBX_LMO_BIRKHOFF
                && cfg_.dicg_oracle_parallelism != DeviceResidentConfig::DICGOracleParallelism::Serial)
            paired_gpu_batches_.fetch_add(1, std::memory_order_relaxed);
        emit_scheduling_event(DRSSchedulingEventType::Dispatched, s.id, s.generation, N);
    }

    void fill_free_slots(bool allow_partial = false) {
        for (auto& s : slots_) {
            if (s.in_use) continue;
            auto batch = queue_.pop_full_batch(cfg_.gpu_batch_size, incumbent_.get());
            if (batch.empty() && allow_partial) batch = queue_.pop_batch(cfg_.gpu_batch_size, incumbent_.get());
            if (batch.empty()) break;
            active_bounds_.insert(batch);
            active_tasks_.fetch_add((int)batch.size(), std::memory_order_relaxed);
            submit_slot(s, std::move(batch));
            if (allow_partial) break;
        }
    }

    Completed detach_completed_slot(Slot& s) {
        const int n = prob_.n_vars, N = s.n_nodes;
        Completed c;
        c.slot_id = s.id;
        c.generation = s.generation;
        c.branched_early.assign(N, 0);
        const uint8_t* st = at<uint8_t>(s.h, s.o_st);
        c.status.assign(st, st + N);
        const double* gap = at<double>(s.h, s.o_gap);
        const double* val = at<double>(s.h, s.o_val);
        c.gap.assign(gap, gap + N);
        c.value.assign(val, val + N);
        c.lower_bound.resize(N);
        for (int i = 0; i < N; ++i) {
            c.lower_bound[i] = certified_fw_lower_bound(s.nodes[i].dual_bound, c.value[i], c.gap[i]);
            if (c.status[i] == GBX_NODE_INFEASIBLE) c.lower_bound[i] = std::numeric_limits<double>::infinity();
        }
        c.nodes = std::move(s.nodes);
        const double* x = at<double>(s.h, s.o_x);
        c.x.assign(x, x + (size_t)N * n);
        const int* it = at<int>(s.h, s.o_it);
        c.iterations.assign(it, it + N);
        const double* best = at<double>(s.h, s.o_best);
        c.best_vertex.assign(best, best + (size_t)N * n);
        const double* bvv = at<double>(s.h, s.o_bvv);
        c.best_vertex_val.assign(bvv, bvv + N);
        s.n_nodes = 0;
        s.in_use = false;
        emit_scheduling_event(DRSSchedulingEventType::CompletionDetached, s.id, c.generation, N);
        return c;
    }

    // Completed slots in submission order.
    std::vector<Slot*> ready_slots() {
        std::vector<Slot*> r;
        for (auto& s : slots_) {
            if (!s.in_use) continue;
            const cudaError_t e = cudaEventQuery(s.done);
            if (e == cudaSuccess) r.push_back(&s);
            else if (e != cudaErrorNotReady) GBX_CUDA_CHECK(e);
        }
        std::sort(r.begin(), r.end(), [](const Slot* a, const Slot* b) { return a->seq < b->seq; });
        return r;
    }

    void call_branch_hook(const Completed& b) {
        if (branch_hook_ && !b.nodes.empty())
            branch_hook_((int)b.nodes.size(), b.nodes.data(), b.x.data(), b.gap.data(), b.value.data(),
                         b.status.data());
    }

    void branch_starved_batches(std::vector<Completed>& batches) {
        for (const auto& b : batches) call_branch_hook(b);
        struct Cand { size_t batch; int node; double bound; };
        std::vector<Cand> cands;
        for (size_t b = 0; b < batches.size(); ++b)
            for (int i = 0; i < (int)batches[b].nodes.size(); ++i) cands.push_back({b, i, batches[b].lower_bound[i]});
        std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& b) { return a.bound < b.bound; });
        const int n = prob_.n_vars;
        for (const auto& cd : cands) {
            if (finish_if_time_limit_reached() || !has_dispatchable_slot()) return;
            auto& batch = batches[cd.batch];
            const int i = cd.node;
            Node nd = batch.nodes[i];
            nd.dual_bound = cd.bound;
            if (pruned_early_parents_.count(nd.parent_id) || should_prune(nd)) continue;
            std::vector<double> x(batch.x.begin() + (size_t)i * n, batch.x.begin() + (size_t)(i + 1) * n);
            if (!std::all_of(x.begin(), x.end(), [](double v) { return std::isfinite(v); })
                    || batch.status[i] >= GBX_NODE_INTEGRAL_UNCONVERGED)
                continue;
            int nid = next_id_;
            next_id_ += id_stride_;
            auto children = branch_sel_(nd, nid, x, prob_.int_vars);
            batch.branched_early[i] = 1;
            for (auto& ch : children) {
                ch.relaxation_x.clear();
                ch.relaxation_iterations = 0;
                if (!should_prune(ch)) queue_.push(ch);
            }
            if (queue_.size() >= cfg_.gpu_batch_size) {
                fill_free_slots(true);
                return;
            }
        }
    }

    void process_completed_batch(Completed& batch) {
        detail::NvtxRange range("gbx.complete");
        const int n = prob_.n_vars;
        const int N = (int)batch.nodes.size();
        call_branch_hook(batch);
        emit_scheduling_event(DRSSchedulingEventType::PostprocessStarted, batch.slot_id, batch.generation, N);
        for (int i = 0; i < N; ++i) {
            if (finish_if_time_limit_reached()) return;
            Node nd = batch.nodes[i];
            const double active_bound = nd.dual_bound;
            if (batch.status[i] == GBX_NODE_INFEASIBLE || pruned_early_parents_.count(nd.parent_id)) {
                retire(active_bound, false);
                continue;
            }
            std::vector<double> xi(batch.x.begin() + (size_t)i * n, batch.x.begin() + (size_t)(i + 1) * n);
            const double gap = batch.gap[i];
            last_gpu_iterations_.store(batch.iterations[i], std::memory_order_relaxed);
            last_gpu_gap_.store(gap, std::memory_order_relaxed);
            last_gpu_converged_.store(std::isfinite(gap) && gap >= 0.0 && gap < node_tolerance(nd),
                                      std::memory_order_relaxed);
            nd.dual_bound = batch.lower_bound[i];
            bool fresh = false;
            if (batch.best_vertex_val[i] < 1e299 && std::isfinite(batch.best_vertex_val[i])) {
                std::vector<double> bv(batch.best_vertex.begin() + (size_t)i * n,
                                       batch.best_vertex.begin() + (size_t)(i + 1) * n);
                fresh = incumbent_.try_update(batch.best_vertex_val[i], bv);
            }
            const bool certified = std::isfinite(gap) && gap >= 0.0 && gap < node_tolerance(nd);
            if (should_prune(nd)) {
                if (batch.branched_early[i]) {
                    pruned_early_parents_.insert(nd.id);
                    queue_.discard_children(nd.id);
                }
                retire(active_bound, fresh);
                continue;
            }
            if (batch.status[i] >= GBX_NODE_INTEGRAL_UNCONVERGED && !certified) {
                nd.relaxation_x = std::move(xi);
                nd.relaxation_iterations = batch.iterations[i];
                queue_.push(nd);
                active_tasks_.fetch_sub(1, std::memory_order_acq_rel);
                active_bounds_.erase_one(active_bound);
                emit_progress(nodes_done_.load(), fresh);
                continue;
            }
            if (!done_.load(std::memory_order_relaxed) && batch.status[i] < GBX_NODE_INTEGRAL_UNCONVERGED
                    && !batch.branched_early[i]) {
                int nid = next_id_;
                next_id_ += id_stride_;
                for (auto& ch : branch_sel_(nd, nid, xi, prob_.int_vars)) {
                    ch.relaxation_x.clear();
                    ch.relaxation_iterations = 0;
                    if (!should_prune(ch)) queue_.push(ch);
                }
            }
            retire(active_bound, fresh);
        }
        if (active_tasks_.load(std::memory_order_acquire) == 0) finish_if_search_complete();
    }

    // the whole search on the device, from the single root node pushed
    void solve_device_frontier() {
        if (queue_.size() != 1) throw std::invalid_argument("the device frontier starts from exactly one root node");
        const Node root = queue_.pop_batch(1, std::numeric_limits<double>::infinity()).front();
        if (root.relaxation_iterations > 0)
            throw std::invalid_argument("the device frontier cannot resume an interrupted root relaxation");
        gbx_problem pr{};
        pr.n_vars = prob_.n_vars;
        pr.lb = root.lb.data();
        pr.ub = root.ub.data();
        pr.int_vars = prob_.int_vars.data();
        pr.n_int = (int)prob_.int_vars.size();
        gbx_settings s;
        gbx_default_settings(&s);
        s.gpu_batch_size = cfg_.gpu_batch_size;
        s.num_streams = cfg_.num_streams;
        s.gpu_max_iters = cfg_.gpu_max_iters;
        s.gpu_eps = cfg_.gpu_eps;
        s.gpu_eps_decay = cfg_.gpu_eps_decay;
        s.gpu_eps_min = cfg_.gpu_eps_min;
        s.integer_tol = cfg_.integer_tol;
        s.abs_gap_tol = cfg_.abs_gap_tol;
        s.rel_gap_tol = cfg_.rel_gap_tol;
        s.algorithm = alg_;
        s.time_limit_seconds = time_limit_seconds_;
        s.natural_lower_bound = root.dual_bound;
        s.root_initial_point = root.relaxation_x.empty() ? nullptr : root.relaxation_x.data();
        s.branch_k = cfg_.branch_k;
        s.use_cuda_graph = cfg_.use_cuda_graph ? 1 : 0;
        s.device_frontier = 1;
        s.incumbent_cutoff = cfg_.incumbent_cutoff ? 1 : 0;
        s.frontier_capacity = cfg_.frontier_capacity;
        s.frontier_slots = cfg_.frontier_slots;
        s.node_limit = cfg_.node_limit;
        std::vector<double> x(prob_.n_vars);
        gbx_result r{};
        r.x = x.data();
        const int rc = gbx_solve(&pr, &obj_, &lmo_, &s, &r);
        if (rc == GBX_ERR_INVALID) throw std::invalid_argument(gbx_last_error());
        gbx_check(rc, "gbx_solve");
        if (r.has_incumbent) incumbent_.try_update(r.objective, x);
        final_dual_bound_ = r.dual_bound;
        nodes_done_.store(r.nodes_processed);
        reached_tolerance_ = r.reached_tolerance != 0;
        reached_time_limit_ = r.reached_time_limit != 0;
        reached_node_limit_ = r.reached_node_limit != 0;
        batches_launched_ = r.batches;
        // the search ran on the device: one progress report, at its end
        if (progress_cb_)
            progress_cb_(r.nodes_processed, 0, r.dual_bound, incumbent_.get(), r.has_incumbent != 0);
        signal_done();
    }

    void retire(double active_bound, bool fresh) {
        const int iter = nodes_done_.fetch_add(1, std::memory_order_relaxed) + 1;
        active_tasks_.fetch_sub(1, std::memory_order_acq_rel);
        active_bounds_.erase_one(active_bound);
        emit_progress(iter, fresh);
        finish_if_search_complete();
    }

    void gpu_worker() {
        while (!done_.load(std::memory_order_relaxed)) {
            if (finish_if_time_limit_reached() || finish_if_node_limit_reached()) return;
            std::vector<Completed> completed;
            for (Slot* s : ready_slots()) completed.push_back(detach_completed_slot(*s));
            // refill released slots before any CPU work on their results
            fill_free_slots();
            if (queue_.empty() && has_dispatchable_slot()) branch_starved_batches(completed);
            for (auto& b : completed) process_completed_batch(b);
            if (active_tasks_.load(std::memory_order_acquire) == 0 && finish_if_search_complete()) return;
            fill_free_slots();
            bool gpu_active = false;
            for (auto& s : slots_) gpu_active = gpu_active || s.in_use;
            if (!gpu_active) {
                fill_free_slots(true);
                for (auto& s : slots_) gpu_active = gpu_active || s.in_use;
                if (gpu_active) continue;
            }
            if (has_dispatchable_slot() && !queue_.empty()) {
                fill_free_slots(true);
            } else if (gpu_active) {
                std::this_thread::yield();
            } else {
                if (active_tasks_.load(std::memory_order_acquire) == 0 && finish_if_search_complete()) return;
                std::this_thread::yield();
            }
        }
        // batches still in flight when the search completed
        std::vector<Slot*> pending;
        for (auto& s : slots_) if (s.in_use) pending.push_back(&s);
        std::sort(pending.begin(), pending.end(), [](const Slot* a, const Slot* b) { return a->seq < b->seq; });
        for (Slot* s : pending) {
            GBX_CUDA_CHECK(cudaEventSynchronize(s->done));
            auto b = detach_completed_slot(*s);
            process_completed_batch(b);
        }
    }

    Problem prob_;
    gbx_objective obj_;
    LMOSpec lmo_spec_;
    gbx_lmo lmo_{};
    gbx_algorithm alg_;
    BranchStrategy branch_sel_;
    DeviceResidentConfig cfg_;
    double time_limit_seconds_;
    RelaxHooks hooks_;

    ConcurrentQueue queue_;
    ConcurrentBoundSet active_bounds_;
    std::unordered_set<int> pruned_early_parents_;
    AtomicIncumbent incumbent_;
    std::atomic<int> active_tasks_{0};
    int next_id_ = 1;
    int id_stride_ = 8;
    std::atomic<int> nodes_done_{0};
    std::atomic<int> last_gpu_iterations_{0};
    std::atomic<double> last_gpu_gap_{std::numeric_limits<double>::infinity()};
    std::atomic<bool> last_gpu_converged_{false};
    std::atomic<bool> done_{false};
    std::atomic<int> paired_gpu_batches_{0};
    long long batches_launched_ = 0, nodes_launched_ = 0;
    std::uint64_t submit_seq_ = 0;
    double final_dual_bound_ = -std::numeric_limits<double>::infinity();
    bool reached_tolerance_ = false;
    bool reached_time_limit_ = false;
    bool reached_node_limit_ = false;
    Clock::time_point solve_started_{};
    std::function<void(int, int, double, double, bool)> progress_cb_;
    std::function<void(const DRSSchedulingEvent&)> scheduling_cb_;
    BranchBatchHook branch_hook_;
    bool tuned_ = false;

    std::vector<Slot> slots_;
    size_t ws_bytes_ = 0;
    uint8_t* d_flags_ = nullptr;
    uint8_t* d_lmo_is_int_ = nullptr;
};

}  // namespace detail
}  // namespace gpuboscia

// The reference's solver class, with the same constructor and accessors.
template <typename DeviceObjective, typename Algorithm, typename LMO = BoxLMO,
          typename Heuristic = gpuboscia::RoundingHeuristic>
class DeviceResidentHybridSolver : public gpuboscia::detail::BnBEngine {
    static_assert(std::is_same_v<Heuristic, gpuboscia::RoundingHeuristic>,
                  "the GB300 relaxation kernel implements the rounding heuristic only");

public:
    DeviceResidentHybridSolver(const Problem& prob, DeviceObjective obj, Algorithm alg, BranchStrategy branch_sel,
                               DeviceResidentConfig cfg = {}, LMO lmo = {},
                               double time_limit_seconds = std::numeric_limits<double>::infinity(),
                               Heuristic = {})
        : BnBEngine(prob, objective_descriptor(obj), lmo.spec(prob.n_vars), alg.descriptor(),
                    std::move(branch_sel), cfg, time_limit_seconds, hooks_for(obj)) {}

private:
    // built-in kinds go to the library; a user objective (the reference's
    // device-struct extension point) to its template kernel (user_relax.cuh)
    static gbx_objective objective_descriptor(const DeviceObjective& obj) {
        if constexpr (gpuboscia::HasDescriptor<DeviceObjective>::value) {
            return obj.descriptor();
        } else {
            gbx_objective o{};
            o.n = DeviceObjective::n_vars;
            return o;
        }
    }
    static gpuboscia::RelaxHooks hooks_for(const DeviceObjective& obj) {
        if constexpr (gpuboscia::HasDescriptor<DeviceObjective>::value) return {};
        else return gpuboscia::UserRelax<DeviceObjective>::hooks(obj);
    }
};
