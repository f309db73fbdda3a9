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
#pragma once
#include "device_resident_solver.h"
