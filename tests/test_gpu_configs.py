"""The five benchmark configurations at their stated sizes, against the oracle.

* Box BQP, n = 64 (1024-node batches, one stream, FW + quadratic-exact): the
  whole branch and bound closes; the GPU search is the oracle's tree node for
  node (same node count, incumbent, solution and bound).
* G(36, 1/2) pair, order 36: the plain FP64 solve equals the oracle's; mixed
  precision reaches the same optimum 0 with a permutation that maps A onto B.
* Cardinality portfolio, 100 assets, 600 months (64-node batches): the first
  640 nodes of the search equal the oracle's (node limit on both).
* 8-regular order-120 pair: the FP64 relaxation of a batch of open nodes is
  bit-identical to the oracle's (iterate, gap, value, status, best vertex).
* Isomorphic 10-regular order-400 pair: nodes whose fixings name five correct
  pairs reach the isomorphism (value 0, AX = XB) in both precisions, and the
  mixed path's certificate equals the oracle's at the iterate it returns.
"""
import numpy as np
import pytest
import torch

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu


def _same(g, o):
    assert g.nodes_processed == o.nodes_processed
    assert g.objective == o.objective
    assert g.dual_bound == o.dual_bound
    assert np.array_equal(g.x, o.x)
    assert g.reached_node_limit == o.reached_node_limit


def _dev(a, dtype=None):
    return torch.from_numpy(np.array(a, dtype=dtype, order="C", copy=True)).cuda()   # a writable copy


def test_box_bqp64_whole_tree_equals_the_oracle(cuda_lib):
    inst = instances.box_qp(n=64)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 1024
    s.gpu_max_iters = 2000
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)
    assert g.objective == g.dual_bound and g.nodes_processed > 500   # closed, with a real tree
    x = g.x
    assert np.array_equal(x, np.round(x))
    Q, c = inst.objective.Q, inst.objective.c
    assert abs(0.5 * x @ Q @ x + c @ x - g.objective) <= 1e-9 * abs(g.objective)


def test_gnp36_plain_equals_oracle_and_mixed_finds_the_isomorphism(cuda_lib):
    inst = instances.birkhoff_gnp(order=36)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 256
    s.gpu_max_iters = 500
    s.line_search = A.LS_QUADRATIC_EXACT
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)
    assert g.objective == 0.0
    s.precision = A.PRECISION_MIXED
    m = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert m.objective == 0.0 and m.dual_bound == 0.0
    X = m.x.reshape(36, 36)
    assert np.array_equal(X.sum(0), np.ones(36)) and np.array_equal(X.sum(1), np.ones(36))
    Am, Bm = inst.objective.A, inst.objective.B
    assert np.array_equal(Am @ X, X @ Bm)


def test_portfolio100_first_640_nodes_equal_the_oracle(cuda_lib):
    inst = instances.portfolio()
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 64
    s.node_limit = 640
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert o.reached_node_limit and o.nodes_processed >= 640
    _same(g, o)


def test_regular120_fp64_relaxation_bit_exact(cuda_lib):
    inst = instances.birkhoff_regular_perturbed(order=120)
    m, N = 120, 8
    n = m * m
    lb, ub = instances.birkhoff_node_batch(m, N, seed=31)
    eps = np.full(N, 1e-6)
    flags = np.ones(n, np.uint8)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT)
    x = _dev(lb.copy())
    it = _dev(np.zeros(N), np.int32)
    st = _dev(np.zeros(N), np.uint8)
    out = api.relax_batch(inst.objective, inst.lmo, alg, x, _dev(lb), _dev(ub), _dev(eps), it, st, 20, _dev(flags))
    torch.cuda.synchronize()
    ref = O.relax(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, eps, max_iters=20, flags=flags, threads=8)
    assert np.array_equal(x.cpu().numpy(), ref["x"])
    assert np.array_equal(it.cpu().numpy(), ref["iterations"])
    assert np.array_equal(st.cpu().numpy(), ref["status"])
    for k in ("gap", "value", "best_vertex", "best_vertex_val"):
        assert np.array_equal(out[k].cpu().numpy(), ref[k]), k


def _order400_fixed_pairs(inst, rows_per_node):
    m = 400
    col = inst.solution.reshape(m, m).argmax(1)
    N = len(rows_per_node)
    lb, ub = np.zeros((N, m * m)), np.ones((N, m * m))
    for i, rows in enumerate(rows_per_node):
        for r in rows:
            lb[i, r * m + col[r]] = 1.0
    return lb, ub


@pytest.mark.parametrize("precision", [A.PRECISION_MIXED, A.PRECISION_FP64])
def test_regular400_nodes_with_five_correct_pairs_reach_the_isomorphism(cuda_lib, precision):
    inst = instances.birkhoff_regular_isomorphic(order=400)
    m = 400
    lb, ub = _order400_fixed_pairs(inst, [range(5), range(100, 105)])
    N = lb.shape[0]
    alg = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, precision)
    x = _dev(lb.copy())
    it = _dev(np.zeros(N), np.int32)
    st = _dev(np.zeros(N), np.uint8)
    out = api.relax_batch(inst.objective, inst.lmo, alg, x, _dev(lb), _dev(ub), _dev(np.full(N, 1e-9)), it, st, 800,
                          _dev(np.ones(m * m, np.uint8)))
    torch.cuda.synchronize()
    bvv = out["best_vertex_val"].cpu().numpy()
    assert np.all(bvv == 0.0), bvv
    Am, Bm = inst.objective.A, inst.objective.B
    for X in out["best_vertex"].cpu().numpy().reshape(N, m, m):
        assert np.array_equal(X.sum(0), np.ones(m)) and np.array_equal(X.sum(1), np.ones(m))
        assert np.array_equal(Am @ X, X @ Bm)


def test_regular400_mixed_certificate_equals_the_oracle(cuda_lib):
    """The mixed iterations steer; the certificate at the iterate they return
    is FP64 and must be the oracle's to the last bit."""
    inst = instances.birkhoff_regular_isomorphic(order=400)
    m, N = 400, 3
    lb, ub = instances.birkhoff_node_batch(m, N, seed=41)
    eps = np.full(N, 1e-6)
    alg = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_MIXED)
    x = _dev(lb.copy())
    it = _dev(np.zeros(N), np.int32)
    st = _dev(np.zeros(N), np.uint8)
    out = api.relax_batch(inst.objective, inst.lmo, alg, x, _dev(lb), _dev(ub), _dev(eps), it, st, 12,
                          _dev(np.ones(m * m, np.uint8)))
    torch.cuda.synchronize()
    its = it.cpu().numpy()
    assert np.all(its == 12)
    ref = O.relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), x.cpu().numpy(), lb, ub,
                  eps, iterations=its, status=np.full(N, 0x80, np.uint8), max_iters=0,
                  flags=np.ones(m * m, np.uint8), threads=8)
    assert np.array_equal(out["gap"].cpu().numpy(), ref["gap"])
    assert np.array_equal(out["value"].cpu().numpy(), ref["value"])
    assert np.array_equal(st.cpu().numpy(), ref["status"])
