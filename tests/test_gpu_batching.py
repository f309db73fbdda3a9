"""Launch shapes of the batched relaxation: the persistent grid (CTAs pulling
nodes from a queue) gives bit-identical node results to one CTA per node; the
tensor-core and SIMT gradients are both valid mixed-precision shapes; the
autotuner restores the batch it times; CUDA-graph replay in the solver gives
the same tree as direct launches."""
import ctypes as C

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances
from test_gpu_parity import gpu_relax

pytestmark = pytest.mark.gpu


def shape(lib, inst, alg, tc, pers):
    keep = api._Keep()
    o = inst.objective.to_c("cuda", keep)
    lm = inst.lmo.to_c(len(inst.problem.lb), "cuda", keep)
    A.check(lib, lib.gbx_relax_set_launch_shape(C.byref(o), C.byref(lm), C.byref(alg), tc, pers),
            "gbx_relax_set_launch_shape")


def run(inst, alg, lb, ub, iters, N):
    flags = np.ones(lb.shape[1], np.uint8)
    return gpu_relax(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, 1e-6, np.zeros(N, np.int32),
                     np.zeros(N, np.uint8), iters, flags)


@pytest.mark.parametrize("prec,order,tc", [(A.PRECISION_FP64, 12, -1), (A.PRECISION_MIXED, 36, 0),
                                           (A.PRECISION_MIXED, 48, 1), (A.PRECISION_MIXED, 96, 1)])
def test_persistent_grid_is_bit_identical(cuda_lib, prec, order, tc):
    inst = instances.birkhoff_gnp(order=order, seed=order)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, precision=prec)
    N = 700 if order <= 48 else 200      # more nodes than resident CTAs: CTAs take several nodes
    lb, ub = instances.birkhoff_node_batch(order, N, seed=3)
    try:
        shape(cuda_lib, inst, alg, tc, 0)
        a = run(inst, alg, lb, ub, 25, N)
        shape(cuda_lib, inst, alg, tc, 1)
        b = run(inst, alg, lb, ub, 25, N)
    finally:
        shape(cuda_lib, inst, alg, -1, 0)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("order", [36, 96])
def test_mixed_relaxation_is_deterministic(cuda_lib, order):
    """Two identical launches give identical nodes (warm-start state included)."""
    inst = instances.birkhoff_gnp(order=order, seed=order + 7)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, precision=A.PRECISION_MIXED)
    N = 600 if order == 36 else 160
    lb, ub = instances.birkhoff_node_batch(order, N, seed=11)
    a = run(inst, alg, lb, ub, 40, N)
    b = run(inst, alg, lb, ub, 40, N)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_tensor_core_and_simt_shapes_both_certify(cuda_lib):
    order, N = 48, 16
    inst = instances.birkhoff_gnp(order=order, seed=2)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, precision=A.PRECISION_MIXED)
    lb, ub = instances.birkhoff_node_batch(order, N, seed=8)
    flags = np.ones(order * order, np.uint8)
    try:
        for tc in (0, 1):
            shape(cuda_lib, inst, alg, tc, 0)
            g = run(inst, alg, lb, ub, 60, N)
            o = O.relax(inst.objective, inst.lmo, O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT), g["x"], lb, ub,
                        1e-6, g["iterations"], np.full(N, A.NODE_INITIAL_POINT_SUPPLIED, np.uint8), 0, flags)
            assert np.array_equal(g["gap"], o["gap"]) and np.array_equal(g["value"], o["value"])
    finally:
        shape(cuda_lib, inst, alg, -1, 0)


def test_autotune_restores_the_batch(cuda_lib):
    import torch
    order, N = 40, 300
    inst = instances.birkhoff_gnp(order=order, seed=4)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, precision=A.PRECISION_MIXED)
    lb, ub = instances.birkhoff_node_batch(order, N, seed=9)
    n = order * order
    T = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a if dt is None else np.asarray(a, dt))).cuda()
    x, dlb, dub, eps = T(lb.copy()), T(lb), T(ub), T(np.full(N, 1e-6))
    it, st = T(np.zeros(N), np.int32), T(np.zeros(N), np.uint8)
    outs = [torch.zeros(N, dtype=torch.float64, device="cuda") for _ in range(3)]
    best = torch.zeros(N, n, dtype=torch.float64, device="cuda")
    b = A.NodeBatch(N, 30, 1e-6, x.data_ptr(), dlb.data_ptr(), dub.data_ptr(), eps.data_ptr(), it.data_ptr(),
                    st.data_ptr(), outs[0].data_ptr(), outs[1].data_ptr(), best.data_ptr(), outs[2].data_ptr(),
                    T(np.ones(n), np.uint8).data_ptr())
    keep = api._Keep()
    o = inst.objective.to_c("cuda", keep)
    lm = inst.lmo.to_c(n, "cuda", keep)
    need = cuda_lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(alg), N)
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    chosen = (C.c_int * 2)()
    s = torch.cuda.current_stream().cuda_stream
    try:
        A.check(cuda_lib, cuda_lib.gbx_relax_autotune(C.byref(o), C.byref(lm), C.byref(alg), C.byref(b),
                                                      ws.data_ptr(), need, s, 2, chosen), "gbx_relax_autotune")
        torch.cuda.synchronize()
        assert np.array_equal(x.cpu().numpy(), lb) and (it.cpu().numpy() == 0).all() and (st.cpu().numpy() == 0).all()
        assert chosen[0] in (0, 1) and chosen[1] in (0, 1)
    finally:
        shape(cuda_lib, inst, alg, -1, 0)


def test_graph_replay_matches_direct_launches(cuda_lib):
    inst = instances.box_qp(n=18, seed=12)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 8
    s.gpu_max_iters = 2000
    s.use_cuda_graph = 1
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    s.use_cuda_graph = 0
    d = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert g.objective == d.objective and g.nodes_processed == d.nodes_processed and g.dual_bound == d.dual_bound
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    assert g.objective == o.objective and g.nodes_processed == o.nodes_processed


def _nodes_per_sm(lib, inst, alg, per_sm):
    keep = api._Keep()
    o = inst.objective.to_c("cuda", keep)
    lm = inst.lmo.to_c(len(inst.problem.lb), "cuda", keep)
    A.check(lib, lib.gbx_relax_set_nodes_per_sm(C.byref(o), C.byref(lm), C.byref(alg), per_sm),
            "gbx_relax_set_nodes_per_sm")


@pytest.mark.parametrize("kind", ["box", "birkhoff", "portfolio"])
def test_fp64_nodes_per_sm_are_bit_identical(cuda_lib, kind):
    """The FP64 kernels compiled for two nodes per SM (128-register cap, the
    default where two fit) and for one give the same nodes bit for bit, with
    more nodes than resident CTAs and against the oracle on a sample."""
    if kind == "box":
        inst = instances.box_qp(n=64, seed=21)
        alg = O.algorithm(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT)
        N, iters = 700, 60
        rng = np.random.default_rng(5)
        lb = np.zeros((N, 64))
        ub = np.ones((N, 64))
        for i in range(N):
            fix = rng.choice(64, 6, replace=False)
            lb[i, fix[:3]] = 1.0
            ub[i, fix[3:]] = 0.0
    elif kind == "birkhoff":
        inst = instances.birkhoff_gnp(order=36, seed=36)
        alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT)
        N, iters = 400, 20
        lb, ub = instances.birkhoff_node_batch(36, N, seed=13)
    else:
        inst = instances.portfolio(assets=100)
        alg = O.algorithm(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT)
        N, iters = 200, 40
        lb, ub = instances.portfolio_node_batch(100, 10, N, seed=9)
    try:
        _nodes_per_sm(cuda_lib, inst, alg, 2)
        a = run(inst, alg, lb, ub, iters, N)
        _nodes_per_sm(cuda_lib, inst, alg, 1)
        b = run(inst, alg, lb, ub, iters, N)
    finally:
        _nodes_per_sm(cuda_lib, inst, alg, -1)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    # a sample against the oracle (the same all-integer flags as run())
    S = 3
    o = O.relax(inst.objective, inst.lmo, alg, lb[:S].copy(), lb[:S], ub[:S], 1e-6, np.zeros(S, np.int32),
                np.zeros(S, np.uint8), iters, np.ones(lb.shape[1], np.uint8))
    for k in ("x", "gap", "value", "status", "iterations"):
        assert np.array_equal(a[k][:S], o[k]), k


@pytest.mark.parametrize("kind", ["portfolio", "box", "portfolio_secant"])
def test_pair_of_ctas_per_node_is_bit_identical(cuda_lib, kind):
    """The dense quadratic objective on a pair of CTAs per node (a two-CTA
    cluster splitting the objective's products, per-lane partial sums exchanged
    through distributed shared memory) gives the nodes of one CTA per node bit
    for bit, and the oracle's on a sample."""
    if kind == "portfolio":
        inst = instances.portfolio(assets=100)
        alg = O.algorithm(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT)
        N, iters = 64, 60
        lb, ub = instances.portfolio_node_batch(100, 10, N, seed=17)
    elif kind == "box":
        inst = instances.box_qp(n=64, seed=23)
        alg = O.algorithm(A.ALG_DICG, A.LS_SECANT)
        N, iters = 40, 40
        lb = np.zeros((N, 64))
        ub = np.ones((N, 64))
        rng = np.random.default_rng(3)
        for i in range(N):
            fix = rng.choice(64, 4, replace=False)
            lb[i, fix[:2]] = 1.0
            ub[i, fix[2:]] = 0.0
    else:   # the secant line search: objective values through the pair's exchanged sums
        inst = instances.portfolio(assets=100)
        alg = O.algorithm(A.ALG_FRANK_WOLFE, A.LS_SECANT)
        N, iters = 32, 30
        lb, ub = instances.portfolio_node_batch(100, 10, N, seed=19)
    try:
        shape(cuda_lib, inst, alg, -1, 0)
        a = run(inst, alg, lb, ub, iters, N)
        shape(cuda_lib, inst, alg, -1, 3)
        b = run(inst, alg, lb, ub, iters, N)
    finally:
        shape(cuda_lib, inst, alg, -1, 0)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    S = 2
    o = O.relax(inst.objective, inst.lmo, alg, lb[:S].copy(), lb[:S], ub[:S], 1e-6, np.zeros(S, np.int32),
                np.zeros(S, np.uint8), iters, np.ones(lb.shape[1], np.uint8))
    for k in ("x", "gap", "value", "status", "iterations"):
        assert np.array_equal(b[k][:S], o[k]), k
