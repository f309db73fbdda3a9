"""GB300-native node relaxation for GPUBoscia's branch and bound.

The compute path is libgpuboscia_gb300.so (hand-written sm_103a CUDA behind
the C ABI of include/gpuboscia_gb300.h). This package builds it in-tree and
mirrors the reference's public API in Python; C++ users include
include/gpuboscia/gpuboscia.h instead.
"""
from . import _abi, instances, scorer
from .api import (BatchRelaxer, BirkhoffLMO, BoxLMO, CardinalityLMO, DenseQuadraticObjective, EqualitySimplexLMO,
                  GraphMatchingObjective, ILSObjective, LinkedCardinalityLMO, Problem, RelaxWorkspace, Result,
                  Settings, UnitSimplexLMO, lmo_batch, node_feasible_batch, objective_gradient_batch,
                  objective_gradient_batch_f32, relax_batch, set_launch_shape, solve)

__all__ = [
    "BatchRelaxer", "BirkhoffLMO", "BoxLMO", "CardinalityLMO", "DenseQuadraticObjective", "EqualitySimplexLMO",
    "GraphMatchingObjective", "ILSObjective", "LinkedCardinalityLMO", "Problem", "RelaxWorkspace", "Result",
    "Settings", "UnitSimplexLMO", "lmo_batch", "node_feasible_batch", "objective_gradient_batch",
    "objective_gradient_batch_f32", "relax_batch", "set_launch_shape", "solve", "instances", "scorer", "_abi",
]
