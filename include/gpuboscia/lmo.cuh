// lmo.cuh -- the reference's include name; the declarations are in lmo.h.
#pragma once
#include "lmo.h"
