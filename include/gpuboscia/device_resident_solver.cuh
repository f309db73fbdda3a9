// device_resident_solver.cuh -- the reference's include name; the declarations are in device_resident_solver.h.
#pragma once
#include "device_resident_solver.h"
