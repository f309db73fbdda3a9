"""The sparse-Sharpe application (examples/sparse_sharpe.cu:550-799) on the GPU
against the oracle: the linked cardinality LMO (forward, in-face, DICG step,
feasibility) bit for bit, Frank-Wolfe and DICG node relaxations with the LMO's
own rounding candidate bit for bit, the branch and bound on one stream
identical to the oracle's, and the device frontier reaching the same optimum."""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances
from test_gpu_parity import _t, assert_same, run_both
from test_gpu_solve import _same

pytestmark = pytest.mark.gpu


def _instance(assets=40, padded=48, m=5, seed=3):
    P = instances.synthetic_gross_returns(120, assets, seed=seed)
    return instances.sparse_sharpe(P, assets=assets, cardinality=m, observations=60, padded=padded)


def _nodes(inst, count, seed):
    """Node bounds with random y fixings, and points inside each node."""
    rng = np.random.default_rng(seed)
    n = inst.problem.n_vars
    h = n // 2
    k = len(inst.lmo.upper)
    m = inst.lmo.cardinality
    lb = np.tile(inst.problem.lb, (count, 1))
    ub = np.tile(inst.problem.ub, (count, 1))
    for r in range(count):
        forced = rng.choice(k, size=rng.integers(0, m + 1), replace=False)
        lb[r, h + forced] = 1.0
        free = np.setdiff1d(np.arange(k), forced)
        ub[r, h + rng.choice(free, size=rng.integers(0, len(free) // 3 + 1), replace=False)] = 0.0
    return lb, ub


@pytest.mark.parametrize("mode", [0, 1])
def test_lmo_bitwise(cuda_lib, mode):
    inst = _instance()
    lb, ub = _nodes(inst, 64, 1)
    rng = np.random.default_rng(2)
    g = rng.normal(size=lb.shape)
    feas_o = O.feasible(inst.lmo, lb, ub)
    feas_g = api.node_feasible_batch(inst.lmo, _t(lb), _t(ub)).cpu().numpy()
    assert np.array_equal(feas_g, feas_o)
    x = None
    if mode == 1:
        # points of each node: convex combinations of forward vertices
        vs = [O.lmo_call(inst.lmo, 0, rng.normal(size=lb.shape), lb, ub)[0] for _ in range(3)]
        w = rng.dirichlet(np.ones(3), size=lb.shape[0])
        x = sum(w[:, t:t + 1] * vs[t] for t in range(3))
    out, step = api.lmo_batch(inst.lmo, mode, _t(g), _t(lb), _t(ub), _t(x) if x is not None else None,
                              want_step=mode == 1)
    ref, rstep = O.lmo_call(inst.lmo, mode, g, lb, ub, x=x, want_step=mode == 1)
    assert np.array_equal(out.cpu().numpy(), ref)
    if mode == 1:
        assert np.array_equal(step.cpu().numpy(), rstep)


@pytest.mark.parametrize("kind,ls", [(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT), (A.ALG_DICG, A.LS_QUADRATIC_EXACT),
                                     (A.ALG_DICG, A.LS_SECANT), (A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP)])
def test_nodes_bitwise(cuda_lib, kind, ls):
    inst = _instance()
    lb, ub = _nodes(inst, 24, 5)
    flags = np.zeros(inst.problem.n_vars, np.uint8)
    flags[inst.problem.int_vars] = 1
    alg = O.algorithm(kind, ls)
    alg.secant_iters = 16
    g, o = run_both(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, 1e-6, 300, flags, tol=1e-5)
    assert_same(g, o)
    assert (o["best_vertex_val"] < 1e299).any()   # the LMO's rounding candidate scores


def test_branch_and_bound_matches_oracle(cuda_lib):
    inst = _instance(assets=12, padded=16, m=3, seed=7)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 16
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 1e-6
    s.time_limit_seconds = 60
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)
    h = inst.problem.n_vars // 2
    assert (g.x[h:h + 12] > 0.5).sum() <= 3
    s.device_frontier = 1
    d = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert abs(d.objective - g.objective) <= 1e-6 * (1 + abs(g.objective))


def test_reference_shape_solves_with_a_certified_bound(cuda_lib):
    """125 candidate assets, at most 10 (the example's defaults) on synthetic
    returns: an incumbent portfolio and a valid bound within the time limit."""
    inst = _instance(assets=125, padded=125, m=10, seed=11)
    s = inst.settings
    s.time_limit_seconds = 20
    s.gpu_batch_size = 256
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert np.isfinite(r.objective) and r.dual_bound <= r.objective + 1e-9
    v, y = r.x[:125], r.x[125:]
    assert (y > 0.5).sum() <= 10 and (v <= inst.lmo.upper * y + 1e-9).all() and (v >= -1e-12).all()
    assert r.objective < 0.0
