"""Learned branching scorer on the GPU: forward (FP32 and BF16) and the
listwise-loss gradient of the CUDA kernels against the float64 numpy oracle
(oracle/scorer_oracle.py), determinism, and training on strong-branching
labels produced by the library's own relaxations.

Tolerances: FP32 forward 1e-5 relative to max |z|; BF16 inference against the
oracle run on BF16-rounded weights, 1e-4; gradient 1e-4 relative to max |g|.
"""
import os
import sys

import numpy as np
import pytest

from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import instances, scorer

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import scorer_oracle as SO  # noqa: E402

pytestmark = pytest.mark.gpu
F = A.SCORER_FEATURES


def bf16_round(a):
    import torch
    return torch.from_numpy(np.asarray(a, np.float32)).to(torch.bfloat16).to(torch.float32).numpy()


def batch(seed, rows=300, groups=17):
    rng = np.random.Generator(np.random.PCG64(seed))
    X = rng.normal(0, 1, (rows, F)).astype(np.float32)
    cuts = np.sort(rng.choice(np.arange(1, rows), groups - 1, replace=False))
    gp = np.concatenate([[0], cuts, [rows]]).astype(np.int32)
    t = rng.random(rows).astype(np.float32)
    for g in range(groups):
        t[gp[g]:gp[g + 1]] /= t[gp[g]:gp[g + 1]].sum()
    return X, gp, t


@pytest.mark.parametrize("hidden", [16, 32, 64])
def test_forward_matches_oracle(cuda_lib, hidden):
    sc = scorer.Scorer(hidden, seed=hidden)
    X, _, _ = batch(1)
    p = sc.numpy()
    z32 = sc.forward(X).cpu().numpy()
    ref, _ = SO.forward(p, X, F, hidden)
    assert np.max(np.abs(z32 - ref)) <= 1e-5 * max(1.0, np.max(np.abs(ref)))
    zb = sc.forward(X, bf16=True).cpu().numpy()
    refb, _ = SO.forward(bf16_round(p), X, F, hidden)
    assert np.max(np.abs(zb - refb)) <= 1e-4 * max(1.0, np.max(np.abs(refb)))


@pytest.mark.parametrize("hidden", [16, 32, 64])
def test_gradient_matches_oracle(cuda_lib, hidden):
    sc = scorer.Scorer(hidden, seed=7)
    X, gp, t = batch(2, rows=517, groups=31)
    g, loss = sc.gradient(X, gp, t)
    g = g.cpu().numpy()
    L, gref = SO.loss_and_grad(sc.numpy(), X, gp, t, F, hidden)
    assert abs(loss.item() - L) <= 1e-4 * max(1.0, abs(L))
    assert np.max(np.abs(g - gref)) <= 1e-4 * max(1.0, np.max(np.abs(gref)))
    g2, _ = sc.gradient(X, gp, t)
    assert np.array_equal(g, g2.cpu().numpy())   # fixed reduction order


def test_adam_matches_reference_update(cuda_lib):
    sc = scorer.Scorer(32, seed=3)
    X, gp, t = batch(3)
    p0 = sc.numpy().astype(np.float64)
    g, _ = sc.gradient(X, gp, t)
    gh = g.cpu().numpy().astype(np.float64)
    sc.adam(g, lr=1e-2)
    m = 0.1 * gh
    v = 0.001 * gh * gh
    ref = p0 - 1e-2 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    assert np.max(np.abs(sc.numpy() - ref)) <= 1e-6
    assert np.array_equal(sc.params_bf16.float().cpu().numpy(), bf16_round(sc.numpy()))


def test_training_on_strong_branching_labels(cuda_lib):
    inst = instances.box_qp(n=20, seed=11)
    data = scorer.collect_strong_branching(inst, max_nodes=12, max_candidates=20)
    assert data.groups >= 4
    for g in range(data.groups):
        seg = data.target[data.group_ptr[g]:data.group_ptr[g + 1]]
        assert abs(seg.sum() - 1.0) < 1e-5 and (seg >= 0).all()
    sc = scorer.Scorer(32, seed=1)
    losses = sc.train(data, epochs=300, lr=3e-3)
    assert losses[-1] < 0.8 * losses[0]


def random_pair(order, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return instances.graph_matching(order, instances.gnp_graph(rng, order, 0.5), instances.gnp_graph(rng, order, 0.5),
                                    f"pair{order}_{seed}")


def solve(inst, sc):
    from gpuboscia_gb300 import api
    s = inst.settings
    s.gpu_batch_size = 32
    s.num_streams = 1
    s.gpu_max_iters = 1000
    s.line_search = A.LS_QUADRATIC_EXACT
    s.time_limit_seconds = 60
    s.scorer = sc
    return api.solve(inst.problem, inst.objective, inst.lmo, s)


def test_learned_branching_gain_on_held_out_pairs(cuda_lib):
    """Train on strong-branching labels of four order-7 graph pairs, then solve
    six other pairs to certified optimality with and without the scorer: the
    same optimum every time, fewer nodes in total with it (one stream, so both
    trees are deterministic)."""
    data = scorer.Dataset.concat([scorer.collect_strong_branching(random_pair(7, 100 + k), max_nodes=30,
                                                                  max_candidates=32) for k in range(4)])
    sc = scorer.Scorer(32, seed=0)
    sc.train(data, epochs=400, lr=3e-3)
    plain = learned = 0
    for k in range(6):
        inst = random_pair(7, 200 + k)
        r0 = solve(inst, None)
        r1 = solve(inst, sc)
        for r in (r0, r1):   # finished, and the FW bound certifies the optimum
            assert not r.reached_time_limit and r.dual_bound >= r.objective - 1e-9
        assert r1.objective == r0.objective
        plain += r0.nodes_processed
        learned += r1.nodes_processed
    print(f"nodes to certified optimum: most fractional {plain}, learned {learned}")
    assert learned < plain
