"""The device frontier's search restated on the CPU (tests/_frontier_oracle.py)
reaches the oracle B&B's certified optimum, with one or two batch slots and
with the incumbent cutoff."""
import numpy as np
import pytest

import _frontier_oracle as F
import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances


def _pair(seed, order):
    rng = np.random.Generator(np.random.PCG64(seed))
    return instances.graph_matching(order, instances.gnp_graph(rng, order, 0.5),
                                    instances.gnp_graph(rng, order, 0.5), f"pair{order}_{seed}")


@pytest.mark.parametrize("slots,cutoff", [(1, 0), (2, 0), (2, 1)])
def test_box_qp(slots, cutoff):
    inst = instances.box_qp(n=12, seed=9)
    s = inst.settings
    s.gpu_batch_size = 8
    s.num_streams = 1
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    s.incumbent_cutoff = cutoff
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    f = F.solve(inst.problem, inst.objective, inst.lmo, s, slots)
    assert abs(f["objective"] - o.objective) <= 1e-9
    assert f["dual_bound"] <= o.objective + 1e-9


@pytest.mark.parametrize("slots", [1, 2])
def test_graph_pair(slots):
    inst = _pair(207, 6)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 16
    s.num_streams = 1
    s.gpu_max_iters = 500
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    f = F.solve(inst.problem, inst.objective, inst.lmo, s, slots)
    assert abs(f["objective"] - o.objective) <= 1e-9
    m = 6
    P = f["x"].reshape(m, m)
    assert np.array_equal(P.sum(0), np.ones(m)) and np.array_equal(P.sum(1), np.ones(m))


@pytest.mark.parametrize("slots,cutoff", [(1, 0), (2, 1)])
def test_cardinality_portfolio(slots, cutoff):
    inst = instances.portfolio(assets=8, months=120, cardinality=3, seed=11)
    s = inst.settings
    s.gpu_batch_size = 16
    s.num_streams = 1
    s.gpu_max_iters = 3000
    s.rel_gap_tol = 0.0
    s.incumbent_cutoff = cutoff
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    f = F.solve(inst.problem, inst.objective, inst.lmo, s, slots)
    assert abs(f["objective"] - o.objective) <= 1e-9
    assert f["dual_bound"] <= o.objective + 1e-9
    w, z = f["x"][:8], f["x"][8:]
    assert abs(w.sum() - 1.0) <= 1e-9 and z.sum() <= 3 and np.all(w <= z + 1e-12)


def test_linked_cardinality_sparse_sharpe():
    P = instances.synthetic_gross_returns(months=72, assets=10, seed=5)
    inst = instances.sparse_sharpe(P, assets=10, cardinality=3, observations=60)
    s = inst.settings
    s.gpu_batch_size = 16
    s.num_streams = 1
    s.gpu_max_iters = 2000
    s.time_limit_seconds = 60
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    for slots in (1, 2):
        f = F.solve(inst.problem, inst.objective, inst.lmo, s, slots)
        assert abs(f["objective"] - o.objective) <= 1e-9 * max(1.0, abs(o.objective))
        y = f["x"][inst.problem.n_vars // 2:]
        assert y.sum() <= 3
