"""Mixed-precision relaxation (FP32 gradient, warm-started integer Hungarian,
permutation DICG steps) against the FP64 oracle.

The iterates differ from the FP64 path by design; what must hold:
* the certificate (gap, value, status) at the returned iterate is the exact
  FP64 certificate -- bit-identical to the oracle's evaluated at that iterate;
* every scored vertex is a feasible permutation whose value is exact;
* the certified intervals [f - gap, f] of the mixed and FP64 runs overlap
  (both contain the node optimum);
* branch and bound reaches the same optimum (1e-9 relative).
"""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances
from test_gpu_parity import gpu_relax

pytestmark = pytest.mark.gpu


def mixed(kind=A.ALG_DICG, ls=A.LS_QUADRATIC_EXACT):
    return O.algorithm(kind, ls, precision=A.PRECISION_MIXED)


@pytest.mark.parametrize("kind,ls", [(A.ALG_DICG, A.LS_QUADRATIC_EXACT), (A.ALG_DICG, A.LS_OPEN_LOOP),
                                     (A.ALG_DICG, A.LS_SAFEGUARDED_SCALED_OPEN_LOOP),
                                     (A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT),
                                     (A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP)])
@pytest.mark.parametrize("order", [12, 36])
def test_mixed_certificate_is_exact_fp64(cuda_lib, kind, ls, order):
    inst = instances.birkhoff_gnp(order=order, seed=order + 1)
    n = order * order
    N = 16
    lb, ub = instances.birkhoff_node_batch(order, N, seed=order)
    flags = np.ones(n, np.uint8)
    g = gpu_relax(inst.objective, inst.lmo, mixed(kind, ls), lb.copy(), lb, ub, 1e-6, np.zeros(N, np.int32),
                  np.zeros(N, np.uint8), 40, flags)
    assert (g["iterations"] > 0).all()
    # the oracle's certificate at the GPU's iterate (no further iterations)
    o = O.relax(inst.objective, inst.lmo, O.algorithm(kind, ls), g["x"], lb, ub, 1e-6, g["iterations"],
                np.full(N, A.NODE_INITIAL_POINT_SUPPLIED, np.uint8), 0, flags)
    assert np.array_equal(g["gap"], o["gap"])
    assert np.array_equal(g["value"], o["value"])
    assert np.array_equal(g["status"], o["status"])
    assert (g["gap"] >= 0).all()
    # best vertices are feasible permutations with exact values
    for i in range(N):
        if g["best_vertex_val"][i] >= 1e299:
            continue
        P = g["best_vertex"][i].reshape(order, order)
        assert set(np.unique(P)) <= {0.0, 1.0}
        assert (P.sum(0) == 1).all() and (P.sum(1) == 1).all()
        assert (g["best_vertex"][i] >= lb[i]).all() and (g["best_vertex"][i] <= ub[i]).all()
        assert O.value(inst.objective, g["best_vertex"][i]) == g["best_vertex_val"][i]


def test_mixed_order120_workspace_arrays(cuda_lib):
    """Order 120: the FP32 arrays and the FP64 vectors live in the workspace."""
    inst = instances.birkhoff_regular_perturbed(order=120)
    order, n, N = 120, 120 * 120, 6
    lb, ub = instances.birkhoff_node_batch(order, N, seed=5)
    flags = np.ones(n, np.uint8)
    g = gpu_relax(inst.objective, inst.lmo, mixed(), lb.copy(), lb, ub, 1e-6, np.zeros(N, np.int32),
                  np.zeros(N, np.uint8), 12, flags)
    assert (g["iterations"] > 0).all()
    o = O.relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), g["x"], lb, ub, 1e-6,
                g["iterations"], np.full(N, A.NODE_INITIAL_POINT_SUPPLIED, np.uint8), 0, flags)
    assert np.array_equal(g["gap"], o["gap"])
    assert np.array_equal(g["value"], o["value"])
    assert np.array_equal(g["status"], o["status"])
    X = g["x"].reshape(N, order, order)
    assert np.allclose(X.sum(1), 1.0, atol=1e-9) and np.allclose(X.sum(2), 1.0, atol=1e-9)


def test_mixed_and_fp64_bounds_overlap(cuda_lib):
    inst = instances.birkhoff_gnp()
    N = 12
    lb, ub = instances.birkhoff_node_batch(36, N, seed=21)
    flags = np.ones(36 * 36, np.uint8)
    z = np.zeros(N, np.int32), np.zeros(N, np.uint8)
    m = gpu_relax(inst.objective, inst.lmo, mixed(), lb.copy(), lb, ub, 1e-7, *z, 400, flags)
    f = gpu_relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), lb.copy(), lb, ub, 1e-7,
                  *z, 400, flags)
    for i in range(N):
        lo_m, hi_m = m["value"][i] - m["gap"][i], m["value"][i]
        lo_f, hi_f = f["value"][i] - f["gap"][i], f["value"][i]
        assert m["gap"][i] >= 0 and f["gap"][i] >= 0
        assert max(lo_m, lo_f) <= min(hi_m, hi_f) + 1e-9 * max(1.0, abs(hi_f)), (i, lo_m, hi_m, lo_f, hi_f)


def random_pair(order, seed):
    """Two independent G(order, 1/2) graphs: not isomorphic, optimum > 0."""
    rng = np.random.Generator(np.random.PCG64(seed))
    A_ = instances.gnp_graph(rng, order, 0.5)
    B_ = instances.gnp_graph(rng, order, 0.5)
    return instances.graph_matching(order, A_, B_, f"pair{order}")


@pytest.mark.parametrize("inst", [instances.birkhoff_gnp(order=10, seed=5), random_pair(7, 7)],
                         ids=["isomorphic10", "pair7"])
def test_mixed_solve_reaches_fp64_optimum(cuda_lib, inst):
    order = inst.lmo.order
    s = inst.settings
    s.gpu_batch_size = 64
    s.num_streams = 2
    s.gpu_max_iters = 400
    s.line_search = A.LS_QUADRATIC_EXACT
    s.time_limit_seconds = 120
    plain = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.precision = A.PRECISION_MIXED
    fast = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert not plain.reached_time_limit and not fast.reached_time_limit
    assert abs(plain.objective - fast.objective) <= 1e-9 * max(1.0, abs(plain.objective))
    X = fast.x.reshape(order, order)
    assert (X.sum(0) == 1).all() and (X.sum(1) == 1).all()
    assert fast.dual_bound <= fast.objective + 1e-9


@pytest.mark.parametrize("order", [72, 96])
def test_mixed_tensor_core_bounds_overlap(cuda_lib, order):
    """Orders 65..128 take the tensor-core gradient; certified intervals still overlap FP64's."""
    inst = instances.birkhoff_gnp(order=order, seed=order)
    N = 6
    lb, ub = instances.birkhoff_node_batch(order, N, seed=order + 1)
    flags = np.ones(order * order, np.uint8)
    z = np.zeros(N, np.int32), np.zeros(N, np.uint8)
    m = gpu_relax(inst.objective, inst.lmo, mixed(), lb.copy(), lb, ub, 1e-7, *z, 150, flags)
    f = gpu_relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), lb.copy(), lb, ub, 1e-7,
                  *z, 150, flags)
    o = O.relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), m["x"], lb, ub, 1e-7,
                m["iterations"], np.full(N, A.NODE_INITIAL_POINT_SUPPLIED, np.uint8), 0, flags)
    assert np.array_equal(m["gap"], o["gap"]) and np.array_equal(m["value"], o["value"])
    for i in range(N):
        lo_m, hi_m = m["value"][i] - m["gap"][i], m["value"][i]
        lo_f, hi_f = f["value"][i] - f["gap"][i], f["value"][i]
        assert max(lo_m, lo_f) <= min(hi_m, hi_f) + 1e-9 * max(1.0, abs(hi_f)), (i, lo_m, hi_m, lo_f, hi_f)


def test_mixed_tensor_core_solve_isomorphic72(cuda_lib):
    inst = instances.birkhoff_gnp(order=72, seed=11)
    s = inst.settings
    s.gpu_batch_size = 32
    s.num_streams = 1
    s.gpu_max_iters = 300
    s.line_search = A.LS_QUADRATIC_EXACT
    s.time_limit_seconds = 120
    s.precision = A.PRECISION_MIXED
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert not r.reached_time_limit
    assert r.objective == 0.0
    X = r.x.reshape(72, 72)
    assert (X.sum(0) == 1).all() and (X.sum(1) == 1).all()


def test_mixed_rejects_other_kinds(cuda_lib):
    import ctypes as C
    keep = api._Keep()
    o = api.DenseQuadraticObjective(np.eye(4)).to_c("host", keep)
    lm = api.BoxLMO().to_c(4, "host", keep)
    alg = mixed()
    assert cuda_lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(alg), 4) == 0
    assert b"mixed precision" in cuda_lib.gbx_last_error()
    inst = instances.birkhoff_gnp(order=6, seed=1)
    o = inst.objective.to_c("host", keep)
    lm = inst.lmo.to_c(36, "host", keep)
    alg = O.algorithm(A.ALG_DICG, A.LS_SECANT, precision=A.PRECISION_MIXED)
    assert cuda_lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(alg), 4) == 0
    assert b"secant" in cuda_lib.gbx_last_error()


@pytest.mark.parametrize("order,degree,N,iters", [(180, 8, 4, 10), (400, 10, 3, 4)])
def test_mixed_large_order_costs_in_workspace(cuda_lib, order, degree, N, iters):
    """Orders whose oracle costs exceed shared memory (the 10-regular pair at 400):
    costs and edge codes in the workspace, FP32 gradient over the nonzero
    lists, 16 columns per lane in the integer Hungarian above 256; the
    certificate is still the exact FP64 one at the returned iterate."""
    inst = instances.birkhoff_regular_isomorphic(order=order, degree=degree, seed=order)
    n = order * order
    lb, ub = instances.birkhoff_node_batch(order, N, seed=9)
    flags = np.ones(n, np.uint8)
    g = gpu_relax(inst.objective, inst.lmo, mixed(), lb.copy(), lb, ub, 1e-6, np.zeros(N, np.int32),
                  np.zeros(N, np.uint8), iters, flags)
    assert (g["iterations"] > 0).all()
    o = O.relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), g["x"], lb, ub, 1e-6,
                g["iterations"], np.full(N, A.NODE_INITIAL_POINT_SUPPLIED, np.uint8), 0, flags)
    assert np.array_equal(g["gap"], o["gap"])
    assert np.array_equal(g["value"], o["value"])
    assert np.array_equal(g["status"], o["status"])
    assert (g["gap"] >= 0).all()
    X = g["x"].reshape(N, order, order)
    assert np.allclose(X.sum(1), 1.0, atol=1e-9) and np.allclose(X.sum(2), 1.0, atol=1e-9)
    assert (g["x"] >= lb - 1e-12).all() and (g["x"] <= ub + 1e-12).all()
