// algorithms.cuh -- the reference's include name; the declarations are in algorithms.h.
#pragma once
#include "algorithms.h"
