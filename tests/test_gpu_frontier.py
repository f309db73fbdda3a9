"""Branch and bound with the frontier in device memory (settings.device_frontier):
same optima and valid certified bounds as the host-frontier solver and the
oracle's B&B. The trees may differ where the host heap and the device's
(bound, id) order break ties differently, so node counts are not compared
across the two frontiers; a device run is compared with itself for
determinism."""
import math

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu


def _proved(r, tol=1e-6):
    return (not r.reached_time_limit) and math.isfinite(r.objective) and r.dual_bound <= r.objective + 1e-12 \
        and (r.objective - r.dual_bound <= tol or r.objective - r.dual_bound <= tol * abs(r.objective))


def test_minimal_example(cuda_lib):
    """examples/minimal.cu: min (x0-.3)^2 + (x1-.7)^2 over binaries -> x = [0, 1], f = .18."""
    obj = api.DenseQuadraticObjective(2 * np.eye(2), np.array([-.6, -1.4]), 1.0, 1.0, .58)
    prob = api.Problem(2, np.zeros(2), np.ones(2), [0, 1])
    s = api.Settings(line_search=A.LS_QUADRATIC_EXACT, natural_lower_bound=0, time_limit_seconds=10,
                     device_frontier=1)
    r = api.solve(prob, obj, api.BoxLMO(), s)
    assert r.x.tolist() == [0.0, 1.0]
    assert abs(r.objective - .18) < 1e-8


@pytest.mark.parametrize("c,lo,hi,alg,ls", [
    ([1.3, 1.6], 0, 3, A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP),
    ([0.7, 1.6, -0.3, 2.8], -1, 4, A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP),
    ([0.7, 1.6, -0.3, 2.8], -1, 4, A.ALG_DICG, A.LS_SECANT),
])
def test_separable_ils_optimum(cuda_lib, c, lo, hi, alg, ls):
    """tests/test_pipeline.cu:647-893: incumbent within 0.02 of the separable optimum."""
    c = np.array(c)
    n = len(c)
    obj = api.ILSObjective(np.eye(n), c, float(c @ c))
    prob = api.Problem(n, np.full(n, float(lo)), np.full(n, float(hi)), list(range(n)))
    s = api.Settings(algorithm=alg, line_search=ls, gpu_batch_size=16, num_streams=1, gpu_max_iters=50000,
                     gpu_eps=1e-6, device_frontier=1)
    g = api.solve(prob, obj, api.BoxLMO(), s)
    true = sum(min((k - ci) ** 2 for k in range(lo, hi + 1)) for ci in c)
    assert abs(g.objective - true) < 0.02
    assert g.dual_bound <= g.objective + 1e-12
    assert np.array_equal(g.x, np.round(g.x)) and np.all(g.x >= lo) and np.all(g.x <= hi)


@pytest.mark.parametrize("batch,k", [(32, 3), (7, 1), (64, 2)])
def test_box_qp_proves_the_oracle_optimum(cuda_lib, batch, k):
    inst = instances.box_qp(n=16, seed=21)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = batch
    s.branch_k = k
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    s.device_frontier = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(g) and _proved(o)
    assert abs(g.objective - o.objective) <= 1e-6
    assert g.dual_bound <= o.objective + 1e-6
    # the incumbent is integral, in bounds, and its value is the objective
    x = g.x
    assert np.array_equal(x, np.round(x)) and x.min() >= 0 and x.max() <= 1
    Q, c = inst.objective.Q, inst.objective.c
    assert abs(0.5 * x @ Q @ x + c @ x - g.objective) <= 1e-9 * max(1.0, abs(g.objective))


def test_deterministic(cuda_lib):
    inst = instances.box_qp(n=16, seed=5)
    s = inst.settings
    s.gpu_batch_size = 16
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    s.device_frontier = 1
    a = api.solve(inst.problem, inst.objective, inst.lmo, s)
    b = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert a.nodes_processed == b.nodes_processed
    assert a.objective == b.objective and a.dual_bound == b.dual_bound
    assert np.array_equal(a.x, b.x)


def test_graph_without_cuda_graph_replay_is_identical(cuda_lib):
    inst = instances.box_qp(n=12, seed=9)
    s = inst.settings
    s.gpu_batch_size = 8
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    s.device_frontier = 1
    a = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.use_cuda_graph = 0
    b = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert (a.nodes_processed, a.objective, a.dual_bound) == (b.nodes_processed, b.objective, b.dual_bound)
    assert np.array_equal(a.x, b.x)


def _pair(seed, order):
    rng = np.random.Generator(np.random.PCG64(seed))
    return instances.graph_matching(order, instances.gnp_graph(rng, order, 0.5),
                                    instances.gnp_graph(rng, order, 0.5), f"pair{order}_{seed}")


@pytest.mark.parametrize("precision", [A.PRECISION_FP64, A.PRECISION_MIXED])
def test_graph_pair_same_optimum_as_host_frontier(cuda_lib, precision):
    inst = _pair(203, 7)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 64
    s.num_streams = 1
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.precision = precision
    s.time_limit_seconds = 60
    h = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.device_frontier = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(h) and _proved(g)
    assert abs(g.objective - h.objective) <= 1e-6
    m = inst.lmo.order
    P = g.x.reshape(m, m)
    assert np.array_equal(P.sum(0), np.ones(m)) and np.array_equal(P.sum(1), np.ones(m))


def test_isomorphic_graph_reaches_zero(cuda_lib):
    inst = instances.birkhoff_gnp(order=8, seed=3)
    s = inst.settings
    s.gpu_batch_size = 16
    s.gpu_max_iters = 200
    s.device_frontier = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert g.objective <= 1e-9


def test_cardinality_portfolio_same_optimum(cuda_lib):
    inst = instances.portfolio(assets=8, months=120, cardinality=3, seed=11)
    s = inst.settings
    s.gpu_batch_size = 32
    s.num_streams = 1
    s.gpu_max_iters = 3000
    s.rel_gap_tol = 0.0
    s.time_limit_seconds = 60
    h = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.device_frontier = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(h) and _proved(g)
    assert abs(g.objective - h.objective) <= 1e-6


def test_root_initial_point(cuda_lib):
    obj = api.DenseQuadraticObjective(2 * np.eye(2), np.array([-.6, -1.4]), 1.0, 1.0, .58)
    prob = api.Problem(2, np.zeros(2), np.ones(2), [0, 1])
    s = api.Settings(line_search=A.LS_QUADRATIC_EXACT, natural_lower_bound=0, time_limit_seconds=10,
                     device_frontier=1, root_initial_point=np.array([0.5, 0.5]))
    r = api.solve(prob, obj, api.BoxLMO(), s)
    assert r.x.tolist() == [0.0, 1.0]


def test_time_limit_returns_a_valid_bound(cuda_lib):
    inst = _pair(301, 10)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 2
    s.abs_gap_tol = 1e-9
    s.rel_gap_tol = 0.0
    s.time_limit_seconds = 0.01
    s.device_frontier = 1
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert r.reached_time_limit
    assert r.dual_bound <= r.objective


def test_capacity_exceeded_is_reported(cuda_lib):
    inst = _pair(302, 9)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 4
    s.abs_gap_tol = 1e-9
    s.rel_gap_tol = 0.0
    s.time_limit_seconds = 30
    s.device_frontier = 1
    s.frontier_capacity = 33           # one round's children (4 * 2^3) + 1
    with pytest.raises(RuntimeError, match="capacity"):
        api.solve(inst.problem, inst.objective, inst.lmo, s)


def test_rejects_unsupported_settings(cuda_lib):
    inst = instances.box_qp(n=8, seed=1)
    s = inst.settings
    s.device_frontier = 1
    s.gpu_batch_size = 2048
    with pytest.raises(ValueError, match="gpu_batch_size"):
        api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.gpu_batch_size = 16
    s.branch_k = 9
    with pytest.raises(ValueError, match="branch_k"):
        api.solve(inst.problem, inst.objective, inst.lmo, s)


@pytest.mark.parametrize("hidden", [16, 32, 64])
def test_learned_branching_same_optimum_as_host_frontier(cuda_lib, hidden):
    """The scorer inside the device branching kernel: same certified optimum as
    the host engine with the same scorer, and the same node count (a node's
    relaxation, features and scores depend on its bounds alone)."""
    from gpuboscia_gb300 import scorer
    sc = scorer.Scorer(hidden, seed=3)
    inst = _pair(204, 7)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 32
    s.num_streams = 1
    s.gpu_max_iters = 1000
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.precision = A.PRECISION_MIXED
    s.time_limit_seconds = 60
    s.scorer = sc
    h = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.device_frontier = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    g2 = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(h) and _proved(g)
    assert abs(g.objective - h.objective) <= 1e-6
    assert g.nodes_processed == h.nodes_processed
    assert (g2.nodes_processed, g2.objective) == (g.nodes_processed, g.objective)


def test_learned_scorer_bad_descriptor(cuda_lib):
    from gpuboscia_gb300 import scorer
    sc = scorer.Scorer(32, seed=1)
    sc.hidden = 48
    inst = instances.box_qp(n=8, seed=1)
    s = inst.settings
    s.device_frontier = 1
    s.scorer = sc
    with pytest.raises(ValueError, match="scorer"):
        api.solve(inst.problem, inst.objective, inst.lmo, s)


@pytest.mark.parametrize("precision", [A.PRECISION_FP64, A.PRECISION_MIXED])
def test_incumbent_cutoff_same_optimum(cuda_lib, precision):
    inst = _pair(205, 7)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 64
    s.gpu_max_iters = 1000
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.precision = precision
    s.time_limit_seconds = 60
    s.device_frontier = 1
    a = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.incumbent_cutoff = 1
    b = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.device_frontier = 0
    h = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(a) and _proved(b) and _proved(h)
    assert abs(a.objective - b.objective) <= 1e-6 and abs(h.objective - b.objective) <= 1e-6


@pytest.mark.parametrize("precision,learned,cutoff", [(A.PRECISION_FP64, False, 0), (A.PRECISION_MIXED, True, 1)])
def test_two_slots_same_optimum_and_deterministic(cuda_lib, precision, learned, cutoff):
    """frontier_slots = 2 (one batch relaxing while the other is merged) reaches
    the optimum of the one-slot search and repeats itself exactly."""
    from gpuboscia_gb300 import scorer
    inst = _pair(206, 8)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 32
    s.gpu_max_iters = 500
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.precision = precision
    s.scorer = scorer.Scorer(32, seed=2) if learned else None
    s.incumbent_cutoff = cutoff
    s.time_limit_seconds = 60
    s.device_frontier = 1
    s.frontier_slots = 1
    one = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.frontier_slots = 2
    two = api.solve(inst.problem, inst.objective, inst.lmo, s)
    again = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(one) and _proved(two)
    assert abs(one.objective - two.objective) <= 1e-6
    assert (two.nodes_processed, two.objective, two.dual_bound) == (again.nodes_processed, again.objective,
                                                                    again.dual_bound)
    assert np.array_equal(two.x, again.x)
    s.use_cuda_graph = 0
    direct = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert (direct.nodes_processed, direct.objective) == (two.nodes_processed, two.objective)


@pytest.mark.parametrize("problem,slots,cutoff", [("box", 1, 0), ("box", 2, 0), ("box", 2, 1),
                                                  ("graph", 1, 0), ("graph", 2, 1), ("portfolio", 1, 0)])
def test_fp64_search_matches_the_restated_frontier(cuda_lib, problem, slots, cutoff):
    """FP64 node relaxations are bit-identical to the oracle's, and the device
    frontier's rules are deterministic, so the whole device search equals its
    CPU restatement (tests/_frontier_oracle.py): node count, objective,
    certified bound and incumbent."""
    import _frontier_oracle as F
    if problem == "box":
        inst = instances.box_qp(n=12, seed=9)
        s = inst.settings
        s.gpu_batch_size = 8
        s.gpu_max_iters = 2000
        s.rel_gap_tol = 0.0
    elif problem == "graph":
        inst = _pair(207, 6)
        s = inst.settings
        s.algorithm = A.ALG_DICG
        s.line_search = A.LS_QUADRATIC_EXACT
        s.gpu_batch_size = 16
        s.gpu_max_iters = 500
        s.abs_gap_tol = 1e-6
        s.rel_gap_tol = 1e-6
    else:
        inst = instances.portfolio(assets=8, months=120, cardinality=3, seed=11)
        s = inst.settings
        s.gpu_batch_size = 16
        s.gpu_max_iters = 3000
        s.rel_gap_tol = 0.0
    s.incumbent_cutoff = cutoff
    s.time_limit_seconds = 60
    ref = F.solve(inst.problem, inst.objective, inst.lmo, s, slots)
    s.device_frontier = 1
    s.frontier_slots = slots
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert g.nodes_processed == ref["nodes"]
    assert g.objective == ref["objective"]
    assert g.dual_bound == ref["dual_bound"]
    assert g.reached_tolerance == ref["tolerance"]
    assert np.array_equal(g.x, ref["x"])


@pytest.mark.parametrize("device_frontier", [0, 1])
def test_node_limit_stops_with_a_valid_bound(cuda_lib, device_frontier):
    """Settings.node_limit ends the search with the batch that reaches it (both
    frontiers): flagged, at least that many nodes and at most one batch more,
    and the reported bound still below the proved optimum."""
    inst = instances.box_qp(n=40, seed=5)   # a tree of ~90 nodes
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 8
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    s.device_frontier = device_frontier
    whole = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(whole) and not whole.reached_node_limit and whole.nodes_processed > 60
    s.node_limit = 30
    part = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert part.reached_node_limit and not part.reached_tolerance
    assert 30 <= part.nodes_processed <= 30 + 2 * s.gpu_batch_size
    assert part.dual_bound <= whole.objective + 1e-9
    assert part.objective >= whole.objective - 1e-9


def test_round_trace_accounts_for_every_node(cuda_lib):
    """Settings.round_trace: one entry per round of the device search, device
    times from CUDA events, and the rounds' node counts summing to the nodes
    processed."""
    inst = instances.box_qp(n=16, seed=21)
    s = inst.settings
    s.gpu_batch_size = 8
    s.gpu_max_iters = 2000
    s.rel_gap_tol = 0.0
    s.device_frontier = 1
    s.round_trace = 4096
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert _proved(r)
    assert len(r.round_ms) == len(r.round_nodes) > 0
    assert int(r.round_nodes.sum()) == r.nodes_processed
    assert np.all(r.round_ms >= 0) and r.round_ms.sum() > 0
    # a batch of continued nodes only finishes no new node
    assert r.batches >= int(np.count_nonzero(r.round_nodes))


@pytest.mark.parametrize("slots,iters", [(1, 2000), (2, 2000), (2, 4)])
def test_compact_pool_equals_the_fp64_pool(cuda_lib, slots, iters):
    """A binary problem keeps its open nodes' bounds as one byte per variable;
    the same problem with one more integer variable fixed at 2 (zero objective
    weight) must keep FP64 bounds. Both searches are the same tree: node count,
    incumbent, bound and solution agree exactly. A budget of 4 iterations per
    dispatch leaves integral nodes unconverged, so continued nodes (their
    iterates in the separate pool) are exercised as well."""
    inst = instances.box_qp(n=16, seed=21)
    Q, c = inst.objective.Q, inst.objective.c
    n = 16
    Q2 = np.zeros((n + 1, n + 1))
    Q2[:n, :n] = Q
    obj2 = api.DenseQuadraticObjective(Q2, np.concatenate([c, [0.0]]), inst.objective.scale,
                                       inst.objective.linear_scale, inst.objective.constant)
    prob2 = api.Problem(n + 1, np.concatenate([inst.problem.lb, [2.0]]), np.concatenate([inst.problem.ub, [2.0]]),
                        list(inst.problem.int_vars) + [n])
    s = inst.settings
    s.gpu_batch_size = 8
    s.gpu_max_iters = iters
    s.rel_gap_tol = 0.0
    s.device_frontier = 1
    s.frontier_slots = slots
    a = api.solve(inst.problem, inst.objective, inst.lmo, s)
    b = api.solve(prob2, obj2, inst.lmo, s)
    assert _proved(a) and _proved(b)
    assert a.nodes_processed == b.nodes_processed
    assert a.objective == b.objective and a.dual_bound == b.dual_bound
    assert np.array_equal(a.x, b.x[:n]) and b.x[n] == 2.0
