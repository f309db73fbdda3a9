"""The incumbent cutoff (gbx_node_batch.cutoff) in the oracle, on the CPU:
an infinite cutoff is the reference's behaviour bit for bit; a finite one
only shortens relaxations, and a node it stops has a certified bound
f(x) - gap at or above the cutoff."""
import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import instances


def _box():
    inst = instances.box_qp(n=24, seed=4)
    lb, ub = instances.box_node_batch(24, 16, seed=2)
    return inst, lb, ub, np.ones(24, np.uint8)


def _graph():
    inst = instances.birkhoff_gnp(order=7, seed=2)
    lb, ub = instances.birkhoff_node_batch(7, 16, seed=3)
    return inst, lb, ub, np.ones(49, np.uint8)


@pytest.mark.parametrize("make", [_box, _graph])
@pytest.mark.parametrize("kind,ls", [(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT), (A.ALG_DICG, A.LS_QUADRATIC_EXACT)])
def test_cutoff_rule(make, kind, ls):
    inst, lb, ub, flags = make()
    alg = O.algorithm(kind, ls)
    free = O.relax(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, 1e-9, max_iters=300, flags=flags)
    inf = O.relax(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, 1e-9, max_iters=300, flags=flags,
                  cutoff=float("inf"))
    for k in ("x", "iterations", "status", "gap", "value", "best_vertex_val"):
        assert np.array_equal(free[k], inf[k]), k
    ok = free["status"] != A.NODE_INFEASIBLE
    bounds = (free["value"] - free["gap"])[ok]
    for q in (10, 50, 90):
        cut = float(np.percentile(bounds, q))
        r = O.relax(inst.objective, inst.lmo, alg, lb.copy(), lb, ub, 1e-9, max_iters=300, flags=flags, cutoff=cut)
        assert (r["iterations"] <= free["iterations"]).all()
        stopped = r["iterations"] < free["iterations"]
        lo = r["value"] - r["gap"]
        assert np.all(lo[stopped] >= cut - 1e-9 * max(1.0, abs(cut)))
        # nodes the cutoff did not stop ran exactly as without it
        same = ~stopped
        assert np.array_equal(r["x"][same], free["x"][same])
