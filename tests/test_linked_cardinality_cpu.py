"""The sparse-Sharpe linked cardinality set (GBX_LMO_LINKED_CARDINALITY,
examples/sparse_sharpe.cu:266-546) in the oracle, pinned by enumeration: the
forward vertex, the in-face vertex over the minimal face of a point, and the
DICG maximum step; the instance builder on the reference's data shape."""
import itertools
import os
import pathlib

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import api, instances
from _refdata import reference_path

A_, HALF, M = 6, 8, 3            # active assets, padded half, cardinality


def _lmo(rng):
    return api.LinkedCardinalityLMO(rng.uniform(0.5, 3.0, A_), M)


def _vertices(U, lb, ub):
    """All vertices (v, y) of the set intersected with the y bounds."""
    forced = [i for i in range(A_) if lb[HALF + i] > 0.5]
    allowed = [i for i in range(A_) if ub[HALF + i] > 0.5]
    out = []
    for k in range(M + 1):
        for S in itertools.combinations(allowed, k):
            if not set(forced) <= set(S):
                continue
            for vs in itertools.product([0, 1], repeat=len(S)):
                x = np.zeros(2 * HALF)
                for i, on in zip(S, vs):
                    x[HALF + i] = 1.0
                    x[i] = U[i] if on else 0.0
                out.append(x)
    return out


def _bounds(rng):
    lb, ub = np.zeros(2 * HALF), np.zeros(2 * HALF)
    ub[HALF:HALF + A_] = 1.0
    for i in range(A_):
        r = rng.random()
        if r < 0.15:
            lb[HALF + i] = 1.0
        elif r < 0.3:
            ub[HALF + i] = 0.0
    if (lb > 0.5).sum() > M:
        lb[:] = 0.0
    return lb, ub


@pytest.mark.parametrize("seed", range(12))
def test_forward_is_the_enumerated_minimum(seed):
    rng = np.random.default_rng(seed)
    lmo = _lmo(rng)
    lb, ub = _bounds(rng)
    ub[:A_] = lmo.upper
    g = rng.normal(size=(1, 2 * HALF))
    v, _ = O.lmo_call(lmo, 0, g, lb[None], ub[None])
    best = min(float(g[0] @ x) for x in _vertices(lmo.upper, lb, ub))
    assert abs(float(g[0] @ v[0]) - best) <= 1e-12
    assert any(np.array_equal(v[0], x) for x in _vertices(lmo.upper, lb, ub))


def _active_face(x, U, lb, ub):
    """Vertices satisfying, as equalities, every constraint active at x."""
    h = HALF
    keep = []
    for w in _vertices(U, lb, ub):
        ok = True
        for i in range(A_):
            if abs(x[h + i] - lb[h + i]) <= 1e-12 and w[h + i] != lb[h + i]:
                ok = False
            if abs(x[h + i] - ub[h + i]) <= 1e-12 and w[h + i] != ub[h + i]:
                ok = False
            if x[i] == 0.0 and w[i] != 0.0:
                ok = False
            if abs(x[i] - U[i] * x[h + i]) <= 1e-12 and abs(w[i] - U[i] * w[h + i]) > 1e-12:
                ok = False
        if abs(x[h:h + A_].sum() - M) <= 1e-12 and abs(w[h:h + A_].sum() - M) > 1e-12:
            ok = False
        if ok:
            keep.append(w)
    return keep


@pytest.mark.parametrize("seed", range(12))
def test_inface_is_the_minimum_over_the_minimal_face(seed):
    rng = np.random.default_rng(100 + seed)
    lmo = _lmo(rng)
    lb, ub = _bounds(rng)
    ub[:A_] = lmo.upper
    verts = _vertices(lmo.upper, lb, ub)
    pick = rng.choice(len(verts), size=min(3, len(verts)), replace=False)
    lam = rng.dirichlet(np.ones(len(pick)))
    x = sum(l * verts[p] for l, p in zip(lam, pick))
    d = rng.normal(size=(1, 2 * HALF))
    a, _ = O.lmo_call(lmo, 1, d, lb[None], ub[None], x=x[None])
    face = _active_face(x, lmo.upper, lb, ub)
    assert face
    best = min(float(d[0] @ w) for w in face)
    assert abs(float(d[0] @ a[0]) - best) <= 1e-9 * (1 + abs(best))


@pytest.mark.parametrize("seed", range(8))
def test_dicg_step_keeps_feasibility(seed):
    rng = np.random.default_rng(200 + seed)
    lmo = _lmo(rng)
    lb, ub = _bounds(rng)
    ub[:A_] = lmo.upper
    verts = _vertices(lmo.upper, lb, ub)
    pick = rng.choice(len(verts), size=min(4, len(verts)), replace=False)
    x = sum(l * verts[p] for l, p in zip(rng.dirichlet(np.ones(len(pick))), pick))
    g = rng.normal(size=(1, 2 * HALF))
    a, step = O.lmo_call(lmo, 1, g, lb[None], ub[None], x=x[None], want_step=True)
    v, _ = O.lmo_call(lmo, 0, -g, lb[None], ub[None])
    gamma = step[0]
    assert 0.0 <= gamma <= 1.0
    y = x - gamma * (a[0] - v[0])
    U = lmo.upper
    tol = 1e-9
    assert (y[:A_] >= -tol).all() and (y[:A_] <= U * y[HALF:HALF + A_] + tol).all()
    assert (y[HALF:HALF + A_] >= lb[HALF:HALF + A_] - tol).all()
    assert (y[HALF:HALF + A_] <= ub[HALF:HALF + A_] + tol).all()
    assert y[HALF:HALF + A_].sum() <= M + tol


def test_feasibility_counts_mandatory_assets():
    rng = np.random.default_rng(0)
    lmo = _lmo(rng)
    lb = np.zeros((2, 2 * HALF))
    ub = np.ones((2, 2 * HALF))
    lb[0, HALF:HALF + M] = 1.0
    lb[1, HALF:HALF + M + 1] = 1.0
    assert O.feasible(lmo, lb, ub).tolist() == [1, 0]


def test_sparse_sharpe_builder_bounds_the_level_set():
    P = instances.synthetic_gross_returns(120, 30, seed=4)
    inst = instances.sparse_sharpe(P, assets=30, cardinality=4, observations=60, padded=32)
    Q, c = inst.objective.Q, inst.objective.c
    H, mu = Q[:30, :30], -c[:30]
    U = inst.lmo.upper
    # the unconstrained minimiser sits inside the box, at the natural lower bound
    vstar = np.linalg.solve(H, mu)
    assert np.all(vstar <= U + 1e-9)
    f = 0.5 * vstar @ H @ vstar - mu @ vstar
    assert abs(f - inst.settings.natural_lower_bound) <= 1e-9 * (1 + abs(f))
    assert inst.problem.int_vars == list(range(32, 62))


US_ALL = reference_path("DataSets", "US_all_monthly.mat")


@pytest.mark.skipif(not US_ALL.is_file(), reason="reference data set not present")
@pytest.mark.parametrize("assets,card", [(20, 4), (40, 5)])
def test_sparse_sharpe_on_the_reference_returns(assets, card):
    """The example's model on its own data (US_all_monthly.mat, last 60 months,
    the first `assets` columns, epsilon 1e-3): the oracle B&B closes the gap,
    the device frontier's restated search reaches the same optimum, and the
    optimum holds at most `card` assets inside their bounds."""
    import _frontier_oracle as F
    P = instances.load_mat(US_ALL, "data")
    inst = instances.sparse_sharpe(P, assets=assets, cardinality=card, observations=60)
    s = inst.settings
    s.gpu_batch_size = 32
    s.num_streams = 1
    s.gpu_max_iters = 2000
    s.time_limit_seconds = 60
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    assert not o.reached_time_limit
    assert o.dual_bound >= o.objective - max(s.abs_gap_tol, s.rel_gap_tol * abs(o.objective))
    assert s.natural_lower_bound <= o.objective
    f = F.solve(inst.problem, inst.objective, inst.lmo, s, 2)
    assert abs(f["objective"] - o.objective) <= 1e-9 * max(1.0, abs(o.objective))
    h = inst.problem.n_vars // 2
    v, y = o.x[:assets], o.x[h:h + assets]
    assert np.array_equal(y, np.round(y)) and y.sum() <= card
    assert np.all(v >= -1e-12) and np.all(v <= inst.lmo.upper[:assets] * y + 1e-9)
