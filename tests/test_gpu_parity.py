"""GPU parity: the FP64 CUDA path against the oracle on the same seeded inputs.

The FP64 kernel and the oracle use the same operation order (256-lane
reductions, explicit fma), so node results must be bit-identical; LMO vertices
and Birkhoff permutations are compared exactly.
"""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu

ALGS = [
    (A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP),
    (A.ALG_FRANK_WOLFE, A.LS_SECANT),
    (A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT),
    (A.ALG_DICG, A.LS_OPEN_LOOP),
    (A.ALG_DICG, A.LS_SCALED_OPEN_LOOP),
    (A.ALG_DICG, A.LS_SAFEGUARDED_SCALED_OPEN_LOOP),
    (A.ALG_DICG, A.LS_SECANT),
    (A.ALG_DICG, A.LS_QUADRATIC_EXACT),
]


def _t(a, dtype=None):
    import torch
    return torch.from_numpy(np.array(a, dtype=dtype, order="C", copy=True)).cuda()   # a writable copy


def gpu_relax(obj, lmo, alg, x, lb, ub, eps, iterations, status, max_iters, flags, tol=1e-6):
    import torch
    X = _t(x)
    it = _t(iterations, np.int32)
    st = _t(status, np.uint8)
    out = api.relax_batch(obj, lmo, alg, X, _t(lb), _t(ub), _t(np.broadcast_to(eps, (x.shape[0],)), np.float64),
                          it, st, max_iters, _t(flags, np.uint8) if flags is not None else None, tol)
    torch.cuda.synchronize()
    return dict(x=X.cpu().numpy(), iterations=it.cpu().numpy(), status=st.cpu().numpy(),
                gap=out["gap"].cpu().numpy(), value=out["value"].cpu().numpy(),
                best_vertex=out["best_vertex"].cpu().numpy(), best_vertex_val=out["best_vertex_val"].cpu().numpy())


def assert_same(g, o, keys=("x", "iterations", "status", "gap", "value", "best_vertex_val")):
    for k in keys:
        a, b = np.asarray(g[k]), np.asarray(o[k])
        assert a.shape == b.shape, k
        same = (a == b) | (np.isnan(a.astype(float)) & np.isnan(b.astype(float)))
        if not same.all():
            bad = np.argwhere(~same)[:5]
            raise AssertionError(f"{k} differs at {bad.tolist()}: gpu={a[tuple(bad[0])]!r} oracle={b[tuple(bad[0])]!r}")
    # best vertex only where a candidate exists
    m = np.asarray(o["best_vertex_val"]) < 1e299
    assert np.array_equal(g["best_vertex"][m], o["best_vertex"][m])


def run_both(obj, lmo, alg, x, lb, ub, eps, max_iters, flags, iterations=None, status=None, tol=1e-6):
    N = x.shape[0]
    iterations = np.zeros(N, np.int32) if iterations is None else iterations
    status = np.zeros(N, np.uint8) if status is None else status
    g = gpu_relax(obj, lmo, alg, x, lb, ub, eps, iterations, status, max_iters, flags, tol)
    o = O.relax(obj, lmo, alg, x, lb, ub, eps, iterations, status, max_iters, flags, tol)
    return g, o


@pytest.mark.parametrize("kind,ls", ALGS)
def test_box_qp_nodes_bitwise(cuda_lib, kind, ls):
    inst = instances.box_qp(n=64)
    lb, ub = instances.box_node_batch(64, 24, seed=7)
    flags = np.ones(64, np.uint8)
    g, o = run_both(inst.objective, inst.lmo, O.algorithm(kind, ls), lb.copy(), lb, ub, 1e-6, 60, flags)
    assert_same(g, o)


@pytest.mark.parametrize("kind,ls", ALGS)
def test_simplex_nodes_bitwise(cuda_lib, kind, ls):
    rng = np.random.default_rng(3)
    n = 40
    M = rng.standard_normal((n, n))
    Q = M.T @ M / n + 0.05 * np.eye(n)
    obj = api.DenseQuadraticObjective(Q, rng.uniform(-1, 1, n))
    ints = list(range(0, n, 2))
    N = 12
    lb = np.zeros((N, n))
    ub = np.full((N, n), 3.0)
    for i in range(N):
        lb[i, ints[i % len(ints)]] = 1.0
    flags = np.zeros(n, np.uint8)
    flags[ints] = 1
    for eq in (False, True):
        lmo = api.UnitSimplexLMO(5.0, ints, eq)
        g, o = run_both(obj, lmo, O.algorithm(kind, ls), lb.copy(), lb, ub, 1e-6, 40, flags)
        assert_same(g, o)


@pytest.mark.parametrize("kind,ls", [a for a in ALGS if a[1] not in (A.LS_SCALED_OPEN_LOOP,)])
def test_birkhoff_graph_matching_bitwise(cuda_lib, kind, ls):
    inst = instances.birkhoff_gnp(order=12, seed=11)
    lb, ub = instances.birkhoff_node_batch(12, 16, seed=5)
    flags = np.ones(144, np.uint8)
    g, o = run_both(inst.objective, inst.lmo, O.algorithm(kind, ls), lb.copy(), lb, ub, 1e-6, 25, flags)
    assert_same(g, o)


def test_birkhoff_order36_dicg_bitwise(cuda_lib):
    inst = instances.birkhoff_gnp()
    lb, ub = instances.birkhoff_node_batch(36, 8, seed=9)
    flags = np.ones(36 * 36, np.uint8)
    g, o = run_both(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), lb.copy(), lb, ub,
                    1e-6, 15, flags)
    assert_same(g, o)


def test_continuation_split_equals_whole(cuda_lib):
    """tests/test_pipeline.cu:1398-1442: 1+1 iterations == 2 iterations, x = 2/3."""
    o = api.ILSObjective(np.eye(2), np.array([.3, .4]), .25)
    flags = np.array([1, 1], np.uint8)
    for kind in (A.ALG_FRANK_WOLFE, A.ALG_DICG):
        alg = O.algorithm(kind, A.LS_OPEN_LOOP)
        z = np.zeros((1, 2)), np.zeros((1, 2)), np.ones((1, 2))
        s1 = gpu_relax(o, api.BoxLMO(), alg, z[0], z[1], z[2], 1e-12, [0], [0], 1, flags)
        assert s1["status"][0] == A.NODE_INTEGRAL_UNCONVERGED
        s2 = gpu_relax(o, api.BoxLMO(), alg, s1["x"], z[1], z[2], 1e-12, s1["iterations"], s1["status"], 1, flags)
        w = gpu_relax(o, api.BoxLMO(), alg, z[0], z[1], z[2], 1e-12, [0], [0], 2, flags)
        assert s2["iterations"][0] == 2
        assert abs(s2["x"][0, 0] - 2.0 / 3.0) < 1e-12
        assert np.array_equal(s2["x"], w["x"]) and s2["gap"][0] == w["gap"][0]


def test_candidate_scores(cuda_lib):
    """tests/test_pipeline.cu:1358-1396: 0.45 from the LMO vertex, 0.09 from rounding."""
    o = api.ILSObjective(np.eye(2), np.array([.3, .4]), .25)
    alg = O.algorithm(A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP)
    r = gpu_relax(o, api.BoxLMO(), alg, np.array([[.6, .4]]), np.zeros((1, 2)), np.ones((1, 2)), 1e-12, [1], [0], 0,
                  np.array([1, 0], np.uint8))
    assert abs(r["best_vertex_val"][0] - 0.45) < 1e-12
    r = gpu_relax(o, api.BoxLMO(), alg, np.array([[.3, .4]]), np.zeros((1, 2)), np.ones((1, 2)), 1e-12, [5], [0], 0,
                  np.array([1, 0], np.uint8))
    assert abs(r["best_vertex_val"][0] - 0.09) < 1e-12
    assert r["best_vertex"][0, 0] == 0.0 and abs(r["best_vertex"][0, 1] - 0.4) < 1e-12


def test_infeasible_before_objective(cuda_lib):
    """tests/test_pipeline.cu:1496-1574: infeasible nodes are rejected with no iteration."""
    o = api.ILSObjective(np.eye(2), np.array([.3, .4]), .25)
    alg = O.algorithm(A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP)
    cases = [
        ([2, 0], [1, 1], [1, 1], api.BoxLMO()),
        ([1.2, 0], [1.8, 1], [1, 0], api.BoxLMO()),
        ([.75, .75], [1, 1], [0, 0], api.EqualitySimplexLMO(1.0, [])),
    ]
    for lb, ub, fl, lmo in cases:
        lb = np.array([lb], float)
        r = gpu_relax(o, lmo, alg, lb.copy(), lb, np.array([ub], float), 1e-12, [0], [0], 1, np.array(fl, np.uint8))
        assert r["status"][0] == A.NODE_INFEASIBLE and r["iterations"][0] == 0 and r["best_vertex_val"][0] >= 1e299
    # Birkhoff order 2 with every row allowed an edge but no perfect matching
    o4 = api.ILSObjective(np.eye(4), np.zeros(4), 0.0)
    lb = np.zeros((1, 4))
    r = gpu_relax(o4, api.BirkhoffLMO(2), alg, lb.copy(), lb, np.array([[1, 0, 1, 0]], float), 1e-12, [0], [0], 1,
                  np.ones(4, np.uint8))
    assert r["status"][0] == A.NODE_INFEASIBLE and r["iterations"][0] == 0


def _lmo_cases(order, cases, seed):
    rng = np.random.default_rng(seed)
    n = order * order
    cost = rng.standard_normal((cases, n))
    lb = np.zeros((cases, n))
    ub = np.ones((cases, n))
    for s in range(cases):
        p = rng.permutation(order)
        for r in range(order):
            for c in range(order):
                if c != p[r] and rng.random() < 0.2:
                    ub[s, r * order + c] = 0.0
        if s % 3:
            r = s % order
            lb[s, r * order + p[r]] = 1.0
    return cost, lb, ub


@pytest.mark.parametrize("order", [7, 36, 120])
def test_birkhoff_lmo_bitwise(cuda_lib, order):
    cost, lb, ub = _lmo_cases(order, 16, order)
    lmo = api.BirkhoffLMO(order)
    g, _ = api.lmo_batch(lmo, 0, _t(cost), _t(lb), _t(ub))
    o, _ = O.lmo_call(lmo, 0, cost, lb, ub)
    assert np.array_equal(g.cpu().numpy(), o)
    # in-face on a convex combination of two permutations, with the maximum step
    rng = np.random.default_rng(order + 1)
    x = np.zeros_like(cost)
    for s in range(len(x)):
        P = np.zeros((order, order))
        P[np.arange(order), rng.permutation(order)] = 0.6
        P[np.arange(order), rng.permutation(order)] += 0.4
        x[s] = P.ravel()
    lb0, ub1 = np.zeros_like(x), np.ones_like(x)
    g, gs = api.lmo_batch(lmo, 1, _t(cost), _t(lb0), _t(ub1), x=_t(x), want_step=True)
    o, os_ = O.lmo_call(lmo, 1, cost, lb0, ub1, x=x, want_step=True)
    assert np.array_equal(g.cpu().numpy(), o)
    assert np.array_equal(gs.cpu().numpy(), os_)


@pytest.mark.parametrize("kind", ["box", "simplex", "eq"])
def test_box_simplex_lmo_bitwise(cuda_lib, kind):
    rng = np.random.default_rng(17)
    n, cases = 200, 32
    d = rng.standard_normal((cases, n))
    d[:, ::7] = 0.0
    lb = np.zeros((cases, n))
    ub = np.full((cases, n), 2.0)
    ints = list(range(0, n, 3))
    if kind == "box":
        lmo = api.BoxLMO()
        lb = rng.integers(-1, 1, (cases, n)).astype(float)
    else:
        lmo = api.UnitSimplexLMO(7.0, ints, kind == "eq")
    x = np.clip(rng.random((cases, n)) * 0.04, 0, None)
    x[:, ::5] = 0.0
    for mode in (0, 1):
        g, gs = api.lmo_batch(lmo, mode, _t(d), _t(lb), _t(ub), x=_t(x), want_step=mode == 1)
        o, os_ = O.lmo_call(lmo, mode, d, lb, ub, x=x, want_step=mode == 1)
        assert np.array_equal(g.cpu().numpy(), o)
        if mode == 1:
            assert np.array_equal(gs.cpu().numpy(), os_)


def _t_at(a, offset):
    """A device copy of `a` that starts `offset` doubles into its allocation
    (offset 1: the buffer is 8-byte but not 16-byte aligned)."""
    import torch
    flat = torch.zeros(a.size + offset, dtype=torch.float64, device="cuda")
    flat[offset:] = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64).ravel()).cuda()
    return flat[offset:].view(*a.shape)


@pytest.mark.parametrize("cases,n,offset", [(1, 1, 0), (3, 7, 0), (3, 7, 1), (5, 4099, 0), (64, 4099, 1),
                                            (512, 2048, 0)])
def test_box_lmo_stream_bitwise(cuda_lib, cases, n, offset):
    """Without the DICG step, a batch of box LMO calls runs as one stream over
    cases*n elements: 16-byte accesses when every buffer is 16-byte aligned,
    one double at a time otherwise, and a lone last element when the count is
    odd. Forward and in-face vertices equal the oracle's bit for bit,
    including directions of -0.0 and iterates just inside and just outside the
    in-face tolerance 1e-6 + 1e-4 |bound|."""
    rng = np.random.default_rng(29 + n + offset)
    d = rng.standard_normal((cases, n))
    d.flat[::5] = 0.0
    d.flat[1::11] = -0.0
    lb = rng.integers(-2, 1, (cases, n)).astype(float)
    ub = lb + rng.integers(0, 3, (cases, n))
    x = lb + rng.random((cases, n)) * (ub - lb)
    pick = rng.random((cases, n))
    x = np.where(pick < 0.15, ub, x)
    x = np.where((pick >= 0.15) & (pick < 0.3), lb, x)
    x = np.where((pick >= 0.3) & (pick < 0.4), ub - 0.5e-6, x)          # inside the upper tolerance
    x = np.where((pick >= 0.4) & (pick < 0.5), lb + 2e-6 + 1e-4 * np.abs(lb), x)   # outside the lower one
    for mode in (0, 1):
        g, step = api.lmo_batch(api.BoxLMO(), mode, _t_at(d, offset), _t_at(lb, offset), _t_at(ub, offset),
                                x=_t_at(x, offset))
        assert step is None
        o, _ = O.lmo_call(api.BoxLMO(), mode, d, lb, ub, x=x)
        assert np.array_equal(g.cpu().numpy(), o), mode
        assert np.array_equal(np.signbit(g.cpu().numpy()), np.signbit(o)), mode


def test_box_lmo_stream_equals_reference_golden(cuda_lib):
    """The committed outputs of the reference's own box oracles at the edges
    of the in-face tolerance (tests/golden/reference_cpu.json, box_edges):
    the stream kernel reproduces them bit for bit, all cases in one batch."""
    import json
    import pathlib
    cases = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_cpu.json").read_text())["box_edges"]
    g, lb, ub, x, fwd, face = (np.array([c[k] for c in cases]) for k in ("g", "lb", "ub", "x", "forward", "inface"))
    for mode, want in ((0, fwd), (1, face)):
        out, _ = api.lmo_batch(api.BoxLMO(), mode, _t(g), _t(lb), _t(ub), x=_t(x))
        got = out.cpu().numpy()
        assert np.array_equal(got, want), mode
        assert np.array_equal(np.signbit(got), np.signbit(want)), mode


def test_node_feasibility_matches_oracle(cuda_lib):
    order = 6
    n = order * order
    rng = np.random.default_rng(5)
    lb = np.zeros((20, n))
    ub = (rng.random((20, n)) < 0.7).astype(float)
    lb[3, 0] = 1.0
    lmo = api.BirkhoffLMO(order)
    g = api.node_feasible_batch(lmo, _t(lb), _t(ub), _t(np.ones(n, np.uint8)))
    o = O.feasible(lmo, lb, ub, np.ones(n, np.uint8))
    assert np.array_equal(g.cpu().numpy(), o)


def test_birkhoff_order64_workspace_path_bitwise(cuda_lib):
    """Order 64 (4096 variables): the node vectors exceed shared memory and live in the
    caller's global workspace; results stay bit-identical to the oracle."""
    import ctypes as C
    inst = instances.birkhoff_gnp(order=64, seed=13)
    keep = api._Keep()
    o = inst.objective.to_c("host", keep)
    lm = inst.lmo.to_c(64 * 64, "host", keep)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT)
    per_node = cuda_lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(alg), 1)
    assert per_node > 4096 * 8 * 4, "order 64 should spill node vectors to the workspace"
    lb, ub = instances.birkhoff_node_batch(64, 4, seed=3)
    g, o_ = run_both(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, 1e-6, 6, np.ones(4096, np.uint8))
    assert_same(g, o_)


def test_birkhoff_order400_nodes_bitwise(cuda_lib):
    """Isomorphic 10-regular graphs on 400 vertices: the FP64 path with the
    zero-skipping gradient and the four-warp Hungarian at 400 free columns."""
    inst = instances.birkhoff_regular_isomorphic(order=400)
    lb, ub = instances.birkhoff_node_batch(400, 2, seed=5)
    flags = np.ones(400 * 400, np.uint8)
    g, o = run_both(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), lb.copy(), lb, ub,
                    1e-6, 2, flags)
    assert_same(g, o)


@pytest.mark.parametrize("kind,ls", [(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT), (A.ALG_DICG, A.LS_QUADRATIC_EXACT),
                                     (A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP)])
@pytest.mark.parametrize("problem", ["box", "graph"])
def test_incumbent_cutoff_nodes_bitwise(cuda_lib, problem, kind, ls):
    """gbx_node_batch.cutoff: nodes whose FW bound clears the incumbent stop
    early; the FP64 kernel and the oracle stop at the same iteration with the
    same certificate."""
    if problem == "box":
        inst = instances.box_qp(n=48)
        lb, ub = instances.box_node_batch(48, 32, seed=11)
        flags = np.ones(48, np.uint8)
        x0 = lb.copy()
    else:
        inst = instances.birkhoff_gnp(order=8, seed=5)
        lb, ub = instances.birkhoff_node_batch(8, 32, seed=4)
        flags = np.ones(64, np.uint8)
        x0 = lb.copy()
    alg = O.algorithm(kind, ls)
    free = O.relax(inst.objective, inst.lmo, alg, x0, lb, ub, 1e-9, max_iters=200, flags=flags)
    bounds = np.where(free["status"] != A.NODE_INFEASIBLE, free["value"] - free["gap"], np.nan)
    cut = float(np.nanpercentile(bounds, 40))
    g = gpu_relax_cut(inst.objective, inst.lmo, alg, x0, lb, ub, 1e-9, 200, flags, cut)
    o = O.relax(inst.objective, inst.lmo, alg, x0, lb, ub, 1e-9, max_iters=200, flags=flags, cutoff=cut)
    assert_same(g, o)
    stopped = o["iterations"] < free["iterations"]
    assert stopped.any()
    # a stopped node's certified bound reaches the cutoff (up to the rounding
    # between the loop's value and the certificate's)
    lo = o["value"] - o["gap"]
    assert np.all(lo[stopped] >= cut - 1e-9 * max(1.0, abs(cut)))


def gpu_relax_cut(obj, lmo, alg, x, lb, ub, eps, max_iters, flags, cutoff):
    import torch
    X = _t(x)
    N = x.shape[0]
    it = _t(np.zeros(N), np.int32)
    st = _t(np.zeros(N), np.uint8)
    out = api.relax_batch(obj, lmo, alg, X, _t(lb), _t(ub), _t(np.full(N, eps), np.float64), it, st, max_iters,
                          _t(flags, np.uint8), 1e-6, cutoff=cutoff)
    torch.cuda.synchronize()
    return dict(x=X.cpu().numpy(), iterations=it.cpu().numpy(), status=st.cpu().numpy(),
                gap=out["gap"].cpu().numpy(), value=out["value"].cpu().numpy(),
                best_vertex=out["best_vertex"].cpu().numpy(), best_vertex_val=out["best_vertex_val"].cpu().numpy())
