"""Whole branch and bound on the GPU (gbx_solve) against the oracle's
single-slot B&B and the reference's known optima."""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu


def test_minimal_example(cuda_lib):
    """examples/minimal.cu: min (x0-.3)^2 + (x1-.7)^2 over binaries -> x = [0, 1], f = .18."""
    obj = api.DenseQuadraticObjective(2 * np.eye(2), np.array([-.6, -1.4]), 1.0, 1.0, .58)
    prob = api.Problem(2, np.zeros(2), np.ones(2), [0, 1])
    s = api.Settings(line_search=A.LS_QUADRATIC_EXACT, natural_lower_bound=0, time_limit_seconds=10)
    r = api.solve(prob, obj, api.BoxLMO(), s)
    assert r.x.tolist() == [0.0, 1.0]
    assert abs(r.objective - .18) < 1e-8


def _same(gpu, ora):
    assert gpu.objective == ora.objective
    assert np.array_equal(gpu.x, ora.x)
    assert gpu.nodes_processed == ora.nodes_processed
    assert gpu.dual_bound == ora.dual_bound
    assert gpu.reached_tolerance == ora.reached_tolerance


@pytest.mark.parametrize("c,lo,hi,alg,ls", [
    ([1.3, 1.6], 0, 3, A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP),
    ([0.7, 1.6, -0.3, 2.8], -1, 4, A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP),
    ([0.7, 1.6, -0.3, 2.8], -1, 4, A.ALG_DICG, A.LS_SAFEGUARDED_SCALED_OPEN_LOOP),
    ([0.7, 1.6, -0.3, 2.8], -1, 4, A.ALG_DICG, A.LS_SECANT),
])
def test_separable_ils_matches_oracle_and_optimum(cuda_lib, c, lo, hi, alg, ls):
    """tests/test_pipeline.cu:647-893: incumbent within 0.02 of the separable optimum."""
    c = np.array(c)
    n = len(c)
    obj = api.ILSObjective(np.eye(n), c, float(c @ c))
    prob = api.Problem(n, np.full(n, float(lo)), np.full(n, float(hi)), list(range(n)))
    s = api.Settings(algorithm=alg, line_search=ls, gpu_batch_size=16, num_streams=1, gpu_max_iters=50000,
                     gpu_eps=1e-6)
    g = api.solve(prob, obj, api.BoxLMO(), s)
    o = O.solve(prob, obj, api.BoxLMO(), s)
    _same(g, o)
    true = sum(min((k - ci) ** 2 for k in range(lo, hi + 1)) for ci in c)
    assert abs(g.objective - true) < 0.02


def test_box_qp_small_matches_oracle(cuda_lib):
    inst = instances.box_qp(n=16, seed=21)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 32
    s.gpu_max_iters = 2000
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)


def test_graph_matching_isomorphic_small(cuda_lib):
    inst = instances.birkhoff_gnp(order=8, seed=3)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 16
    s.gpu_max_iters = 200
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)
    assert g.objective <= 1e-9


def test_multistream_same_optimum(cuda_lib):
    inst = instances.box_qp(n=16, seed=21)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 8
    s.gpu_max_iters = 2000
    one = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.num_streams = 4
    many = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert abs(one.objective - many.objective) <= 1e-9 * max(1.0, abs(one.objective))
    assert many.dual_bound <= many.objective + 1e-9


@pytest.mark.parametrize("seed", [21, 5])
def test_incumbent_cutoff_matches_oracle(cuda_lib, seed):
    """Relaxations stopped at the incumbent (settings.incumbent_cutoff): the
    host-frontier solver and the oracle's B&B stay identical, and reach the
    optimum of the search without the cutoff."""
    inst = instances.box_qp(n=16, seed=seed)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 8
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    ref = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.incumbent_cutoff = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)
    assert abs(g.objective - ref.objective) <= 1e-6
