"""The cardinality-constrained portfolio on the GPU against the oracle:
the cardinality LMO and the feasibility test bit for bit, Frank-Wolfe node
relaxations bit for bit, and the whole branch and bound (one stream: the same
tree as the oracle's)."""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances
from test_gpu_parity import _t, assert_same, run_both
from test_gpu_solve import _same

pytestmark = pytest.mark.gpu


def cases(N, K, count, seed, ints):
    rng = np.random.Generator(np.random.PCG64(seed))
    n = 2 * N
    g = rng.integers(-3, 4, (count, n)).astype(float) if ints else rng.normal(0, 1, (count, n))
    lb, ub = np.zeros((count, n)), np.ones((count, n))
    u = rng.random((count, N))
    lb[:, N:][u < 0.08] = 1.0
    ub[:, N:][(u >= 0.08) & (u < 0.3)] = 0.0
    return g, lb, ub


@pytest.mark.parametrize("N,K,ints", [(100, 10, False), (100, 10, True), (37, 5, True), (600, 40, False)])
def test_cardinality_lmo_bitwise(cuda_lib, N, K, ints):
    lmo = api.CardinalityLMO(N, K)
    g, lb, ub = cases(N, K, 48, N + K, ints)
    feas_o = O.feasible(lmo, lb, ub)
    feas_g = api.node_feasible_batch(lmo, _t(lb), _t(ub)).cpu().numpy()
    assert np.array_equal(feas_g, feas_o)
    ok = feas_o.astype(bool)
    out, _ = api.lmo_batch(lmo, 0, _t(g[ok]), _t(lb[ok]), _t(ub[ok]))
    ref, _ = O.lmo_call(lmo, 0, g[ok], lb[ok], ub[ok])
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("ls", [A.LS_QUADRATIC_EXACT, A.LS_OPEN_LOOP, A.LS_SECANT])
def test_portfolio_nodes_bitwise(cuda_lib, ls):
    inst = instances.portfolio()
    lb, ub = instances.portfolio_node_batch(100, 10, 24, seed=3)
    flags = np.r_[np.zeros(100), np.ones(100)].astype(np.uint8)
    g, o = run_both(inst.objective, inst.lmo, O.algorithm(A.ALG_FRANK_WOLFE, ls), np.clip(lb, 0, None), lb, ub,
                    1e-6, 150, flags)
    assert_same(g, o)


def test_portfolio_rejects_dicg(cuda_lib):
    import ctypes as C
    inst = instances.portfolio(assets=8, months=60, cardinality=2)
    keep = api._Keep()
    o = inst.objective.to_c("cuda", keep)
    lm = inst.lmo.to_c(16, "cuda", keep)
    alg = O.algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT)
    assert cuda_lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(alg), 4) == 0
    assert b"Frank-Wolfe" in cuda_lib.gbx_last_error()


def test_portfolio_solve_matches_oracle(cuda_lib):
    inst = instances.portfolio(assets=12, months=120, cardinality=3, seed=31)
    s = inst.settings
    s.num_streams = 1
    s.gpu_batch_size = 16
    s.gpu_max_iters = 3000
    s.rel_gap_tol = 1e-4
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    _same(g, o)
    w, z = g.x[:12], g.x[12:]
    assert abs(w.sum() - 1) <= 1e-9 and z.sum() <= 3 and (w <= z + 1e-9).all()
