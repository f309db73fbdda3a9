"""Objective gradients through gbx_objective_gradient_batch against the oracle.

FP64: bit-identical to the oracle's gradient (the relaxation's own code).
Mixed (graph matching): BF16 tensor-core products with FP32 accumulation for
orders 65..128 (X and R split into hi + lo BF16), FP32 SIMT below. The
tolerance is stated on the max-norm: |g_mixed - g_fp64|_inf <= 2e-5 * |g_fp64|_inf.
"""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu

MIXED_TOL = 2e-5


def points(order, cases, seed):
    """Doubly-stochastic-ish iterates: convex combinations of a few permutations plus noise."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = order * order
    X = np.zeros((cases, n))
    for k in range(cases):
        w = rng.dirichlet(np.ones(4))
        M = np.zeros((order, order))
        for t in range(4):
            M[np.arange(order), rng.permutation(order)] += w[t]
        X[k] = (M + 1e-3 * rng.random((order, order))).ravel()
    return X


def gpu_grad(obj, X, precision):
    import torch
    return api.objective_gradient_batch(obj, torch.from_numpy(X).cuda(), precision).cpu().numpy()


@pytest.mark.parametrize("order", [12, 36, 72, 120, 128])
def test_fp64_gradient_bitwise(cuda_lib, order):
    inst = instances.birkhoff_gnp(order=order, seed=order)
    X = points(order, 3, order)
    g = gpu_grad(inst.objective, X, A.PRECISION_FP64)
    for k in range(X.shape[0]):
        assert np.array_equal(g[k], O.grad(inst.objective, X[k]))


def test_fp64_dense_gradient_bitwise(cuda_lib):
    inst = instances.box_qp(n=64)
    rng = np.random.Generator(np.random.PCG64(3))
    X = rng.random((5, 64))
    g = gpu_grad(inst.objective, X, A.PRECISION_FP64)
    for k in range(5):
        assert np.array_equal(g[k], O.grad(inst.objective, X[k]))


@pytest.mark.parametrize("order", [36, 65, 96, 120, 128])
def test_mixed_gradient_error(cuda_lib, order):
    inst = instances.birkhoff_regular_perturbed(order=order) if order == 120 else \
        instances.birkhoff_gnp(order=order, seed=order + 3)
    X = points(order, 4, order + 1)
    g = gpu_grad(inst.objective, X, A.PRECISION_MIXED)
    for k in range(X.shape[0]):
        ref = O.grad(inst.objective, X[k])
        err = np.max(np.abs(g[k] - ref)) / np.max(np.abs(ref))
        assert err <= MIXED_TOL, (order, k, err)


def test_mixed_gradient_rejects(cuda_lib):
    import torch
    inst = instances.box_qp(n=16)
    with pytest.raises(RuntimeError, match="mixed gradient"):
        api.objective_gradient_batch(inst.objective, torch.zeros(1, 16, dtype=torch.float64).cuda(),
                                     A.PRECISION_MIXED)


@pytest.mark.parametrize("order,cases", [(36, 1), (96, 5), (120, 300), (128, 700)])
def test_pipelined_f32_gradient_error(cuda_lib, order, cases):
    """gbx_objective_gradient_batch_f32: the persistent pipelined kernel (several
    points per CTA, both operand buffers reused) against the FP64 oracle."""
    import torch
    inst = instances.birkhoff_gnp(order=order, seed=order + 9)
    X = points(order, cases, order + 2)
    g = api.objective_gradient_batch_f32(inst.objective, torch.from_numpy(X).cuda()).cpu().numpy()
    for k in sorted({0, cases // 2, cases - 1}):
        ref = O.grad(inst.objective, X[k].astype(np.float32).astype(np.float64))
        err = np.max(np.abs(g[k] - ref)) / np.max(np.abs(ref))
        assert err <= MIXED_TOL, (order, k, err)


def test_pipelined_f32_gradient_rejects(cuda_lib):
    import torch
    inst = instances.birkhoff_gnp(order=130, seed=1)
    with pytest.raises(RuntimeError, match="order 128"):
        api.objective_gradient_batch_f32(inst.objective, torch.zeros(1, 130 * 130).cuda())
