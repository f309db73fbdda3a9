// multiblock.cuh -- the reference's include name for its K-CTAs-per-node
// execution. The GB300 kernel needs no separate mode: node vectors that do not
// fit in shared memory move to an L2-resident workspace and a persistent grid
// takes nodes from a queue, chosen per problem shape by the launch autotuner.
// The execution-mode settings are accepted by DeviceResidentConfig.
#pragma once
#include "device_resident_solver.h"
