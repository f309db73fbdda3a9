// dense_quadratic_objectives.cuh -- the reference's include name; the declarations are in dense_quadratic_objectives.h.
#pragma once
#include "dense_quadratic_objectives.h"
