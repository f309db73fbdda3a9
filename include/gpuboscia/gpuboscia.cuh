// gpuboscia.cuh -- the reference's include name for the public API. In a
// translation unit compiled by nvcc it also brings the template relaxation of
// user-written device objectives (user_relax.cuh), so a reference program
// whose objective is its own device struct compiles unchanged.
#pragma once
#include "gpuboscia.h"
#ifdef __CUDACC__
#include "multiblock.cuh"
#include "user_relax.cuh"
#endif
