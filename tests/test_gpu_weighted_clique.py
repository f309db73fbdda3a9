"""The reference's weighted-clique example (examples/weighted_clique.cu) solved
on the GPU: 20 vertices, exactly 5 chosen, DICG over the equality simplex with
integer variables. One stream repeats the oracle's B&B exactly; the example's
own settings (two streams) and the device frontier reach the enumerated optimum
within the example's tolerances."""
import itertools

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import api, instances

pytestmark = pytest.mark.gpu


def _best(inst):
    Q, c = inst.objective.Q, inst.objective.c
    return min(0.5 * Q[np.ix_(S, S)].sum() + c[list(S)].sum() for S in itertools.combinations(range(20), 5))


def test_one_stream_repeats_the_oracle(cuda_lib):
    inst = instances.weighted_clique()
    s = inst.settings
    s.num_streams = 1
    s.time_limit_seconds = 120
    g = api.solve(inst.problem, inst.objective, inst.lmo, s)
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    assert g.objective == o.objective
    assert g.dual_bound == o.dual_bound
    assert g.nodes_processed == o.nodes_processed
    assert np.array_equal(g.x, o.x)


@pytest.mark.parametrize("device_frontier", [0, 1])
def test_examples_settings_reach_the_optimum(cuda_lib, device_frontier):
    inst = instances.weighted_clique()
    best = _best(inst)
    s = inst.settings
    s.time_limit_seconds = 120
    s.device_frontier = device_frontier
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert not r.reached_time_limit
    assert r.objective - best <= 1e-3 * abs(best) + 1e-7
    assert r.dual_bound <= best + 1e-9
    assert np.array_equal(r.x, np.round(r.x)) and r.x.sum() == 5
