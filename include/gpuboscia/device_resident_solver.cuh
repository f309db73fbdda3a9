// device_resident_solver.cuh -- the reference's include name; the declarations are in device_resident_solver.h
// (and, under nvcc, the reference's MultiBlockContext name in multiblock.cuh).
#pragma once
#include "device_resident_solver.h"
#ifdef __CUDACC__
#include "multiblock.cuh"
#endif
