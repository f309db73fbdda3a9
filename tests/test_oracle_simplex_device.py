"""The bounded-simplex oracles follow the reference's DEVICE algorithm, which
its relaxation kernel runs, and that algorithm is not its CPU one in one
case.

UnitSimplexLMO::parallel_greedy_allocate_cooperative (lmo.cuh:529-610) sorts
the eligible coordinates by (gradient, index), exclusive-scans their
capacities (an integer coordinate's residual interval, a continuous one's the
whole remaining mass) and gives each coordinate min(max(remaining - prefix,
0), capacity), floored for integer coordinates where the caller asks
(compute_v in the equality form, compute_inface_v always; lmo.cuh:785-860).
The CPU oracle compute_v_cpu (lmo.cuh:399-450) instead walks the coordinates
and subtracts what each one actually took. The two agree unless an integer
coordinate is floored below its capacity ahead of another eligible
coordinate: the scan still charges the full capacity, so the later
coordinate sees less mass than is left, and in the equality form the vertex
can miss the right-hand side (rhs 1.5: [1, 0] on the device, [1, 0.5] on the
CPU). The oracle restates the device algorithm (the CUDA kernels are
checked against the oracle); the committed golden cases from the CPU
functions use integral right-hand sides, where the two agree. This file
checks both statements on CPU."""
import math

import numpy as np
import pytest

import _oracle as O
from gpuboscia_gb300 import api


def _greedy(grad, ub, out, fixed, remaining, is_int, force_full, floor_int, eq):
    """parallel_greedy_allocate_cooperative restated sequentially (exact here:
    the capacities are binary fractions, so the scan's order cannot round)."""
    elig = [j for j in range(len(grad)) if (fixed is None or not fixed[j]) and (force_full or grad[j] <= 0.0)]
    elig.sort(key=lambda j: (grad[j], j))
    prefix, adds = 0.0, []
    for j in elig:
        cap = max(ub[j] - out[j], 0.0) if is_int[j] else remaining
        add = min(max(remaining - prefix, 0.0), cap)
        if floor_int and is_int[j]:
            add = math.floor(add + (1e-9 if eq else 0.0))
        adds.append((j, add))
        prefix += cap
    for j, add in adds:
        out[j] += add


def device_forward(grad, lb, ub, is_int, rhs, eq):
    """UnitSimplexLMO::compute_v (lmo.cuh:785-809)."""
    v = np.where(is_int, lb, 0.0).astype(float)
    _greedy(grad, ub, v, None, rhs - v.sum(), is_int, eq, eq, eq)
    return v


def device_inface(grad, x, lb, ub, is_int, rhs, eq, atol=1e-6, rtol=1e-4):
    """UnitSimplexLMO::compute_inface_v (lmo.cuh:811-860)."""
    n = len(grad)
    a = np.zeros(n)
    fixed = [False] * n
    for j in range(n):
        lower = lb[j] if is_int[j] else 0.0
        a[j] = lower
        if abs(x[j] - lower) <= atol + rtol * max(abs(x[j]), abs(lower)):
            fixed[j] = True
        elif is_int[j] and abs(x[j] - ub[j]) <= atol + rtol * max(abs(x[j]), abs(ub[j])):
            fixed[j] = True
            a[j] = ub[j]
    xm = float(np.sum(x))
    force = eq or abs(xm - rhs) <= atol + rtol * max(abs(xm), abs(rhs))
    _greedy(grad, ub, a, fixed, rhs - float(np.sum(a)), is_int, force, True, eq)
    return a


def _cases(seed, count, fractional):
    """Random bounded-simplex cases with many gradient ties, some integer
    coordinates forced to 1 and a feasible iterate x."""
    rng = np.random.default_rng(seed)
    for _ in range(count):
        n = int(rng.integers(2, 40))
        eq = int(rng.integers(0, 2))
        k = int(rng.integers(0, n + 1))
        ints = sorted(rng.choice(n, k, replace=False).tolist())
        rhs = float(rng.integers(1, 12)) + (0.5 if fractional else 0.0)
        g = rng.integers(-2, 3, n) / 8.0
        lb = np.zeros(n)
        ub = np.where(np.isin(np.arange(n), ints), rng.integers(1, 4, n), rhs).astype(float)
        s = 0.0
        for j in ints:
            if rng.random() < 0.2 and s + 1 <= rhs:
                lb[j] = 1.0
                s += 1
        x = lb.copy()
        rest = (rhs - s) if eq else (rhs - s) * rng.random()
        for j in rng.permutation([j for j in range(n) if ub[j] > lb[j]]):
            if rest <= 0:
                break
            add = min(ub[j] - x[j], rest) if rng.random() < 0.5 else min(ub[j] - x[j], rest, float(rng.integers(0, 3)))
            x[j] += add
            rest -= add
        if eq and rest > 1e-12:
            continue
        yield n, eq, ints, rhs, g, lb, ub, x


@pytest.mark.parametrize("fractional", [False, True])
def test_oracle_is_the_device_algorithm(fractional):
    calls = 0
    for n, eq, ints, rhs, g, lb, ub, x in _cases(11 + fractional, 600, fractional):
        is_int = np.isin(np.arange(n), ints)
        lmo = api.UnitSimplexLMO(rhs, ints, bool(eq))
        fwd, _ = O.lmo_call(lmo, 0, g[None], lb[None], ub[None])
        assert np.array_equal(fwd[0], device_forward(g, lb, ub, is_int, rhs, eq)), (n, eq, ints, rhs)
        face, _ = O.lmo_call(lmo, 1, g[None], lb[None], ub[None], x=x[None])
        assert np.array_equal(face[0], device_inface(g, x, lb, ub, is_int, rhs, eq)), (n, eq, ints, rhs)
        calls += 2
    assert calls > 1000


def test_device_and_cpu_algorithms_differ_on_a_floored_integer():
    """rhs 1.5, x0 integer (residual interval 2) ahead of the continuous x1."""
    g, lb, ub = np.array([-1.0, 0.0]), np.zeros(2), np.array([2.0, 1.5])
    is_int = np.array([True, False])
    assert np.array_equal(device_forward(g, lb, ub, is_int, 1.5, 1), [1.0, 0.0])
    fwd, _ = O.lmo_call(api.UnitSimplexLMO(1.5, [0], True), 0, g[None], lb[None], ub[None])
    assert np.array_equal(fwd[0], [1.0, 0.0])
    R = O.ref()
    if R is not None:   # the reference's CPU oracle fills the remainder
        out = np.zeros(2)
        iv = np.array([0], dtype=np.int32)
        R.ref_simplex_lmo(1, 0, 2, 1.5, iv.ctypes.data, 1, g.ctypes.data, None, lb.ctypes.data, ub.ctypes.data,
                          out.ctypes.data, None)
        assert np.array_equal(out, [1.0, 0.5])


@pytest.mark.skipif(O.ref() is None, reason="reference tree not available at build time")
def test_integral_right_sides_agree_with_the_reference_cpu_functions():
    """Where no integer coordinate is floored below its capacity (integral
    right-hand sides), the reference's CPU oracles equal the oracle: forward
    and in-face vertices over random tie-heavy cases."""
    R = O.ref()
    calls = 0
    for n, eq, ints, rhs, g, lb, ub, x in _cases(7, 600, False):
        lmo = api.UnitSimplexLMO(rhs, ints, bool(eq))
        iv = np.array(ints, dtype=np.int32)
        for mode in (0, 1):
            out = np.zeros(n)
            R.ref_simplex_lmo(eq, mode, n, rhs, iv.ctypes.data if ints else None, len(ints), g.ctypes.data,
                              x.ctypes.data if mode else None, lb.ctypes.data, ub.ctypes.data, out.ctypes.data, None)
            o, _ = O.lmo_call(lmo, mode, g[None], lb[None], ub[None], x=x[None] if mode else None)
            assert np.array_equal(o[0], out), (mode, n, eq, ints, rhs)
            calls += 1
    assert calls > 1000
