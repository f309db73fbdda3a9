"""Cardinality-linked simplex LMO (the portfolio set) on the CPU: the oracle against
enumeration of every vertex, with forced and forbidden assets and ties. The
set has no counterpart in the reference, so enumeration pins it."""
import itertools

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances


def enumerate_min(g, lb, ub, N, K):
    """min <g, v> over vertices v = (e_a, 1_S): a in S, |S| <= K, forced in S, forbidden out."""
    forced = {j for j in range(N) if lb[N + j] > 0.5}
    forbidden = {j for j in range(N) if ub[N + j] < 0.5}
    free = [j for j in range(N) if j not in forced and j not in forbidden]
    best = np.inf
    for a in range(N):
        if a in forbidden:
            continue
        base = forced | {a}
        if len(base) > K:
            continue
        rest = [j for j in free if j != a]
        for r in range(0, K - len(base) + 1):
            for extra in itertools.combinations(rest, r):
                S = base | set(extra)
                best = min(best, g[a] + sum(g[N + j] for j in S))
    return best


@pytest.mark.parametrize("seed", range(12))
def test_oracle_matches_enumeration(seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    N = int(rng.integers(3, 8))
    K = int(rng.integers(1, N + 1))
    n = 2 * N
    ints = seed % 3 == 0
    lmo = api.CardinalityLMO(N, K)
    for case in range(20):
        g = rng.integers(-3, 4, n).astype(float) if ints else rng.normal(0, 1, n)
        lb, ub = np.zeros(n), np.ones(n)
        for j in range(N):
            u = rng.random()
            if u < 0.15:
                lb[N + j] = 1.0
            elif u < 0.3:
                ub[N + j] = 0.0
        feas = O.feasible(lmo, lb[None], ub[None])[0]
        best = enumerate_min(g, lb, ub, N, K)
        assert bool(feas) == np.isfinite(best), (seed, case)
        if not feas:
            continue
        v = O.lmo_call(lmo, 0, g[None], lb[None], ub[None])[0][0]
        w, z = v[:N], v[N:]
        assert w.sum() == 1.0 and set(np.unique(v)) <= {0.0, 1.0}
        assert (w <= z).all() and z.sum() <= K
        assert (z[lb[N:] > 0.5] == 1).all() and (z[ub[N:] < 0.5] == 0).all()
        assert abs(float(g @ v) - best) <= 1e-12 * max(1.0, abs(best)), (seed, case)


def test_portfolio_instance_shapes():
    inst = instances.portfolio()
    n = 200
    Q = inst.objective.Q
    assert Q.shape == (n, n) and np.allclose(Q, Q.T)
    assert (np.linalg.eigvalsh(Q[:100, :100]) > 0).all()
    assert list(inst.problem.int_vars) == list(range(100, 200))
    lb, ub = instances.portfolio_node_batch(100, 10, 16)
    assert ((lb[:, 100:] > 0.5).sum(1) <= 10).all()
