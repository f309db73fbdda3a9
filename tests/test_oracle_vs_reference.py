"""The oracle's LMOs and host rules against the reference project's own CPU
functions: through the committed fixtures (tests/golden/reference_cpu.json,
made by tests/golden/make_golden.py) and, where the reference tree was present
at build time, live against oracle/_ref on fresh random cases."""
import json
import math
import pathlib

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import api

GOLDEN = json.loads((pathlib.Path(__file__).parent / "golden" / "reference_cpu.json").read_text())


def test_birkhoff_hungarian_matches_reference_bitwise():
    """BirkhoffLMO::compute_v_cpu / compute_inface_v_cpu (lmo.cuh:958-1171), ties to the lowest column."""
    for c in GOLDEN["birkhoff"]:
        order = c["order"]
        n = order * order
        lmo = api.BirkhoffLMO(order)
        cost, lb, ub, x = (np.array([c[k]]) for k in ("cost", "lb", "ub", "x"))
        fwd, _ = O.lmo_call(lmo, 0, cost, lb, ub)
        assert np.array_equal(fwd[0], np.array(c["forward"])), f"order {order} forward"
        face, _ = O.lmo_call(lmo, 1, cost, np.zeros((1, n)), np.ones((1, n)), x=x)
        assert np.array_equal(face[0], np.array(c["inface"])), f"order {order} in-face"


def test_box_lmo_matches_reference():
    for c in GOLDEN["box"]:
        g, lb, ub, x = (np.array([c[k]]) for k in ("g", "lb", "ub", "x"))
        fwd, _ = O.lmo_call(api.BoxLMO(), 0, g, lb, ub)
        assert np.array_equal(fwd[0], c["forward"])
        face, step = O.lmo_call(api.BoxLMO(), 1, g, lb, ub, x=x, want_step=True)
        assert np.array_equal(face[0], c["inface"])
        assert step[0] == max(0.0, c["step"])


def test_box_lmo_tolerance_edges_match_reference():
    """BoxLMO::compute_v_cpu / compute_inface_v_cpu (lmo.cuh:225-262) with
    iterates on, just inside, exactly at and just beyond the in-face
    tolerance 1e-6 + 1e-4 |bound| of either bound, and directions of +0.0 and
    -0.0: the oracle's vertices equal the reference's bit for bit (sign bits
    included)."""
    for c in GOLDEN["box_edges"]:
        g, lb, ub, x = (np.array([c[k]]) for k in ("g", "lb", "ub", "x"))
        fwd, _ = O.lmo_call(api.BoxLMO(), 0, g, lb, ub)
        assert np.array_equal(fwd[0], c["forward"])
        assert np.array_equal(np.signbit(fwd[0]), np.signbit(c["forward"]))
        face, _ = O.lmo_call(api.BoxLMO(), 1, g, lb, ub, x=x)
        assert np.array_equal(face[0], c["inface"])
        assert np.array_equal(np.signbit(face[0]), np.signbit(c["inface"]))


def test_simplex_lmo_matches_reference():
    for c in GOLDEN["simplex"]:
        lmo = api.UnitSimplexLMO(c["rhs"], c["ints"], bool(c["equality"]))
        g, lb, ub, x = (np.array([c[k]]) for k in ("g", "lb", "ub", "x"))
        fwd, _ = O.lmo_call(lmo, 0, g, lb, ub)
        assert np.array_equal(fwd[0], c["forward"]), c
        face, step = O.lmo_call(lmo, 1, g, lb, ub, x=x, want_step=True)
        assert np.array_equal(face[0], c["inface"]), c
        assert abs(step[0] - max(0.0, min(1.0, c["step"]))) <= 1e-12, (step[0], c["step"])


def test_host_rules_match_reference():
    """gap_utils.h and line_search_options.h through the fixture tables."""
    from gpuboscia_gb300 import _abi  # noqa: F401  (tables only)
    lib = O.lib()
    assert lib is not None
    for b, i, ga, gr, t1, t2 in GOLDEN["gaps"]:
        ours_abs = math.inf if (i >= math.inf or b <= -math.inf) else abs(i - b)
        if not (math.isnan(b) or math.isnan(i)):
            assert ours_abs == ga or (math.isinf(ours_abs) and math.isinf(ga))
        if not (math.isfinite(b) and math.isfinite(i)):
            assert math.isinf(gr)
    for d, tol in GOLDEN["depth_tol"]:
        assert tol == (max(1e-3, 1e-6) if d <= 0 else max(1e-6, 1e-3 * 0.8 ** d))


def test_quadratic_exact_step_table():
    for g, c, m, expect in GOLDEN["quad_step"]:
        if m <= 0:
            ours = 0.0
        elif c > 0:
            ours = 0.0 if g <= 0 else min(g / c, m)
        else:
            ours = m if -g + 0.5 * c * m < 0 else 0.0
        assert ours == expect


def test_branch_pow2_children():
    """branching.h:80-118 through the fixture; the C++ header is checked in test_host_cpp."""
    for c in GOLDEN["branch_pow2"]:
        x = np.array(c["x"])
        n = len(x)
        fr = x - np.floor(x)
        dist = np.minimum(fr, 1 - fr)
        cand = [i for i in range(n) if dist[i] > 1e-6]
        vars_ = sorted(cand, key=lambda i: -dist[i])[: c["k"]]
        assert len(c["lb"]) == 2 ** len(vars_)


@pytest.mark.skipif(O.ref() is None, reason="reference tree not available at build time")
def test_live_random_birkhoff_against_reference():
    R = O.ref()
    rng = np.random.default_rng(99)
    for order in (4, 7, 12, 36):
        n = order * order
        lmo = api.BirkhoffLMO(order)
        for _ in range(6):
            cost = rng.integers(-6, 7, n) / 4.0
            ub = (rng.random(n) > 0.1).astype(float)
            p = rng.permutation(order)
            ub[np.arange(order) * order + p] = 1.0
            lb = np.zeros(n)
            out = np.zeros(n)
            R.ref_birkhoff_lmo(order, 0, cost.ctypes.data, None, lb.ctypes.data, ub.ctypes.data, out.ctypes.data)
            ours, _ = O.lmo_call(lmo, 0, cost[None], lb[None], ub[None])
            assert np.array_equal(ours[0], out)


@pytest.mark.skipif(O.ref() is None, reason="reference tree not available at build time")
def test_live_birkhoff_inface_forced_forbidden_against_reference():
    """BirkhoffLMO::compute_v_cpu / compute_inface_v_cpu (lmo.cuh:958-1171) on
    heavy ties (costs in quarters, some -0.0), forbidden entries, a few forced
    pairs and iterates that mix up to three permutations: the oracle's
    forward and in-face vertices equal the reference's bit for bit."""
    R = O.ref()
    rng = np.random.default_rng(5)
    calls = 0
    for _ in range(300):
        order = int(rng.choice([3, 4, 5, 6, 7, 8, 12, 16]))
        n = order * order
        cost = rng.integers(-3, 4, n) / 4.0
        cost[rng.random(n) < 0.1] = -0.0
        lb, ub = np.zeros(n), np.ones(n)
        p = rng.permutation(order)
        forbid = rng.random(n) < 0.25
        forbid[np.arange(order) * order + p] = False
        ub[forbid] = 0.0
        for i in range(order):
            if rng.random() < 0.15:
                lb[i * order + p[i]] = 1.0
        x = np.zeros(n)
        for w in rng.dirichlet(np.ones(3)):
            q = p.copy()
            a, b = rng.choice(order, 2, replace=False)
            q[a], q[b] = p[b], p[a]
            allowed = all(ub[i * order + q[i]] > 0 for i in range(order)) and lb[a * order + p[a]] == 0 \
                and lb[b * order + p[b]] == 0
            for i, col in enumerate(q if allowed else p):
                x[i * order + col] += w
        lmo = api.BirkhoffLMO(order)
        for mode in (0, 1):
            out = np.zeros(n)
            rc = R.ref_birkhoff_lmo(order, mode, cost.ctypes.data, x.ctypes.data if mode else None, lb.ctypes.data,
                                    ub.ctypes.data, out.ctypes.data)
            assert rc == 0
            ours, _ = O.lmo_call(lmo, mode, cost[None], lb[None], ub[None], x=x[None] if mode else None)
            assert np.array_equal(ours[0], out), (order, mode)
            calls += 1
    assert calls == 600


@pytest.mark.skipif(O.ref() is None, reason="reference tree not available at build time")
@pytest.mark.parametrize("order", [32, 33, 97, 120, 129, 400])
def test_live_large_order_birkhoff_against_reference(order):
    """The orders of the reference's LMO benchmark check (32, 33, 97, 129)
    and the order-120 and order-400 workloads: forward and in-face vertices under 30 %
    forbidden arcs, a few forced pairs and tied costs, bit-identical to the
    reference's CPU Hungarian."""
    R = O.ref()
    rng = np.random.default_rng(order)
    n = order * order
    lmo = api.BirkhoffLMO(order)
    for _ in range(4):
        cost = rng.integers(-8, 9, n) / 4.0
        lb, ub = np.zeros(n), np.ones(n)
        p = rng.permutation(order)
        forbid = rng.random(n) < 0.3
        forbid[np.arange(order) * order + p] = False
        ub[forbid] = 0.0
        lb[np.arange(order) * order + p] = (rng.random(order) < 0.05).astype(float)
        x = np.zeros(n)
        for w in (0.6, 0.4):
            q = p.copy()
            a, b = rng.choice(order, 2, replace=False)
            if ub[a * order + p[b]] > 0 and ub[b * order + p[a]] > 0 and lb[a * order + p[a]] == 0 \
                    and lb[b * order + p[b]] == 0:
                q[a], q[b] = p[b], p[a]
            x[np.arange(order) * order + q] += w
        for mode in (0, 1):
            out = np.zeros(n)
            assert R.ref_birkhoff_lmo(order, mode, cost.ctypes.data, x.ctypes.data if mode else None,
                                      lb.ctypes.data, ub.ctypes.data, out.ctypes.data) == 0
            ours, _ = O.lmo_call(lmo, mode, cost[None], lb[None], ub[None], x=x[None] if mode else None)
            assert np.array_equal(ours[0], out), mode
