"""The reference's weighted-clique example (examples/weighted_clique.cu): a
convex binary quadratic over the equality simplex sum x = 5 on 20 vertices,
DICG. Its built-in kinds (dense quadratic objective, EqualitySimplexLMO with
integer variables) solve it; the oracle B&B and the device frontier's restated
search reach the optimum found by enumerating all C(20, 5) subsets."""
import itertools

import numpy as np

import _frontier_oracle as F
import _oracle as O
from gpuboscia_gb300 import instances


def _enumerated():
    inst = instances.weighted_clique()
    Q, c = inst.objective.Q, inst.objective.c
    best, arg = np.inf, None
    for S in itertools.combinations(range(20), 5):
        S = list(S)
        v = 0.5 * Q[np.ix_(S, S)].sum() + c[S].sum()
        if v < best:
            best, arg = v, S
    return inst, best, arg


def test_model_is_the_examples():
    inst = instances.weighted_clique()
    Q, c = inst.objective.Q, inst.objective.c
    n, lam = 20, 19.0
    assert np.array_equal(Q, Q.T) and np.all(np.diag(Q) == 2 * lam) and np.all(c == -lam)
    off = Q[~np.eye(n, dtype=bool)]
    assert np.all((off > 0) & (off <= 2))
    # diagonally dominant, hence convex
    assert np.all(np.diag(Q) >= np.abs(Q).sum(1) - np.diag(Q))
    # at a binary point the convexification vanishes: f = 2 sum_{i<j} (1 - w_ij) x_i x_j
    S = [0, 3, 7, 11, 19]
    x = np.zeros(n)
    x[S] = 1
    f = 0.5 * x @ Q @ x + c @ x
    assert abs(f - sum(Q[i, j] for i, j in itertools.combinations(S, 2))) <= 1e-12
    s = inst.settings
    assert s.natural_lower_bound == lam * (25 / 20 - 5)
    assert inst.lmo.equality and inst.lmo.right_side == 5.0


def test_oracle_and_restated_search_reach_the_enumerated_optimum():
    inst, best, arg = _enumerated()
    s = inst.settings
    s.num_streams = 1
    s.time_limit_seconds = 120
    # the example's tolerances (abs 1e-7, rel 1e-3)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    assert not o.reached_time_limit
    assert o.objective - best <= 1e-3 * abs(best) + 1e-7
    assert o.dual_bound <= best + 1e-9
    f = F.solve(inst.problem, inst.objective, inst.lmo, s, 2)
    assert f["objective"] - best <= 1e-3 * abs(best) + 1e-7
    assert f["dual_bound"] <= best + 1e-9
    for x in (o.x, f["x"]):
        x = np.asarray(x)
        assert np.array_equal(x, np.round(x)) and x.sum() == 5
    # closed tolerances: the exact optimum and its subset
    s.rel_gap_tol = 0.0
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    assert abs(o.objective - best) <= 1e-9
    assert sorted(np.nonzero(np.asarray(o.x) > 0.5)[0].tolist()) == arg
