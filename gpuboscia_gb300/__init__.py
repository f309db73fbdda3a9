"""GB300-native node relaxation for GPUBoscia's branch and bound.

The compute path is libgpuboscia_gb300.so (hand-written sm_103a CUDA behind
the C ABI of include/gpuboscia_gb300.h). This package builds it in-tree and
mirrors the reference's public API in Python; C++ users include
include/gpuboscia/gpuboscia.h instead.
"""
from . import _abi, scorer
from .api import (BirkhoffLMO, BoxLMO, CardinalityLMO, DenseQuadraticObjective, EqualitySimplexLMO, GraphMatchingObjective,
                  ILSObjective, Problem, RelaxWorkspace, Result, Settings, UnitSimplexLMO, lmo_batch,
                  node_feasible_batch, objective_gradient_batch, relax_batch, solve)

__all__ = [
    "BirkhoffLMO", "BoxLMO", "CardinalityLMO", "DenseQuadraticObjective", "EqualitySimplexLMO", "GraphMatchingObjective",
    "ILSObjective", "Problem", "RelaxWorkspace", "Result", "Settings", "UnitSimplexLMO", "lmo_batch",
    "node_feasible_batch", "objective_gradient_batch", "relax_batch", "solve", "scorer", "_abi",
]
