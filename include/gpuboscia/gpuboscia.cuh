// gpuboscia.cuh -- the reference's include name for the public API.
#pragma once
#include "gpuboscia.h"
