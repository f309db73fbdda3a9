// heuristics.h -- incumbent heuristics (reference: include/gpuboscia/heuristics.h:23-35).
#pragma once

namespace gpuboscia {
// Rounds the integer coordinates of the final iterate and scores the result
// on the GPU when it is feasible for the LMO's set. This is the only built-in
// heuristic; it runs inside the relaxation kernel.
struct RoundingHeuristic {};
}  // namespace gpuboscia
