// multiblock.cuh -- the reference's include name for its K-CTAs-per-node
// execution (a cooperative barrier per node over global memory). On GB300 a
// node that needs more than one CTA gets a thread-block cluster instead: for
// mixed-precision graph matching over the Birkhoff polytope at orders
// 129..404, four CTAs per node hold slices of the integer oracle costs in
// shared memory and split every Dijkstra step, exchanging minima through
// distributed shared memory (gbx_relax_set_launch_shape persistent = 2, or the
// autotuner's choice). Node vectors that do not fit in shared memory move to
// an L2-resident workspace, and a persistent grid takes nodes from a queue.
// The execution-mode settings are accepted by DeviceResidentConfig.
//
// What user code of the reference names from this header stays available:
// DRS_HAS_MULTIBLOCK_ATOMICS (0: the global-memory node barrier is not a
// backend here, so code that chooses a mode by it takes the single-CTA one)
// and, under nvcc, MultiBlockContext with the reference's public members
// (multiblock.cuh:36-103 of the reference), so that a device objective
// written with an optional grad_multiblock(MultiBlockContext&, ...) member
// still compiles. The relaxation calls grad, never grad_multiblock; a
// context built here describes one CTA: its node barrier is the CTA barrier
// and its sum a CTA reduction.
#pragma once
#include "device_resident_solver.h"

#ifndef DRS_HAS_MULTIBLOCK_ATOMICS
#define DRS_HAS_MULTIBLOCK_ATOMICS 0
#endif

#ifdef __CUDACC__
struct alignas(16) NodeBarrier {
    unsigned int arrived;
    unsigned int generation;
};

class MultiBlockContext {
public:
    unsigned char* lmo_workspace = nullptr;
    double* reduction_partials = nullptr;
    int node_id, block_rank, block_count;
    int thread_rank, threads_per_block, global_tid, total_threads;

    // rank and count describe the CTAs of a node; only one CTA per node is a
    // valid context here (count 1), which every solver path in this library
    // builds: a node that spans CTAs runs as a cluster with its own exchange
    __device__ MultiBlockContext(int node, int rank, int count, NodeBarrier*)
        : node_id(node), block_rank(rank), block_count(count), thread_rank((int)threadIdx.x),
          threads_per_block((int)blockDim.x), global_tid(rank * (int)blockDim.x + (int)threadIdx.x),
          total_threads(count * (int)blockDim.x) {}

    // Sum of one value per thread of the CTA, returned to every thread.
    __device__ double sum(double value) const {
        __shared__ double warp_part[32];
        __shared__ double total;
        for (int o = 16; o > 0; o >>= 1) value += __shfl_down_sync(0xffffffffu, value, o);
        if ((thread_rank & 31) == 0) warp_part[thread_rank >> 5] = value;
        __syncthreads();
        if (thread_rank == 0) {
            double t = 0.0;
            for (int w = 0; w < (threads_per_block + 31) / 32; ++w) t += warp_part[w];
            total = t;
        }
        __syncthreads();
        const double r = total;
        __syncthreads();
        return r;
    }
    __device__ void block_sync() const { __syncthreads(); }
    __device__ void node_sync() const { __syncthreads(); }
};
#endif
