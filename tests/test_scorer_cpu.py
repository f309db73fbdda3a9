"""Learned branching scorer on the CPU: the numpy oracle's gradient against
finite differences, and the host feature function through the C ABI."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import scorer_oracle as SO  # noqa: E402

F = 16


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(1))
    H = 8
    count = H * F + H + H * H + H + H + 1
    p = rng.normal(0, 0.5, count)
    X = rng.normal(0, 1, (11, F))
    gp = np.array([0, 4, 5, 11])
    t = rng.random(11)
    for g in range(3):
        t[gp[g]:gp[g + 1]] /= t[gp[g]:gp[g + 1]].sum()
    L, g = SO.loss_and_grad(p, X, gp, t, F, H)
    h = 1e-6
    for idx in rng.choice(count, 40, replace=False):
        q = p.copy(); q[idx] += h
        Lp, _ = SO.loss_and_grad(q, X, gp, t, F, H)
        q[idx] -= 2 * h
        Lm, _ = SO.loss_and_grad(q, X, gp, t, F, H)
        assert abs((Lp - Lm) / (2 * h) - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])), idx


def test_branch_features_known_answer():
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import scorer
    lib_path = A.LIB_PATH
    if not lib_path.exists():
        pytest.skip("library not built")
    # Birkhoff order 3: rows (.5,.5,0), (.5,.25,.25), (0,.25,.75); x[0][0] is a candidate
    x = np.array([.5, .5, 0, .5, .25, .25, 0, .25, .75])
    lb = np.zeros(9)
    ub = np.ones(9)
    ub[2] = 0.0
    f = scorer.features(x, lb, ub, 3, 5, 0.2, 1.8, [0, 4])
    assert f.shape == (2, 16)
    np.testing.assert_allclose(f[0, :6], [0.5, 0.5, 0.5, 5 / 64, 0.2 / 2.8, 1.0], rtol=1e-6)
    # row 0 has two fractional entries, column 0 has two; row max .5, column max .5
    np.testing.assert_allclose(f[0, 6:15], [2 / 3, 2 / 3, .5, .5, 1, 1, 1, 1, 2 / 3], rtol=1e-6)
    # x[1][1] = .25: row 1 all three fractional, column 1 three fractional, maxima .5 and .5
    np.testing.assert_allclose(f[1, [0, 6, 7, 8, 9, 10, 11, 12, 13]], [.25, 1, 1, .5, .5, 0, 0, .5, .5], rtol=1e-6)


def test_scorer_entry_points_check_their_inputs():
    """features(), Scorer.forward and Scorer.gradient refuse inputs the
    library would read past (short bounds, candidate indices out of range,
    rows without F features, group offsets that do not span the rows) before
    any device work."""
    import pytest
    from gpuboscia_gb300 import scorer
    x, lb, ub = np.full(6, 0.5), np.zeros(6), np.ones(6)
    with pytest.raises(ValueError, match="same length"):
        scorer.features(x, lb[:5], ub, 0, 1, 0.1, 1.0, [0])
    with pytest.raises(ValueError, match="out of range"):
        scorer.features(x, lb, ub, 0, 1, 0.1, 1.0, [6])
    with pytest.raises(ValueError, match="out of range"):
        scorer.features(x, lb, ub, 0, 1, 0.1, 1.0, [-1])
    F = scorer.F
    sc = scorer.Scorer.__new__(scorer.Scorer)   # the checks run before the parameters are needed
    with pytest.raises(ValueError, match="features must be"):
        sc.forward(np.zeros((4, F - 1), np.float32))
    rows = 5
    X, t = np.zeros((rows, F), np.float32), np.full(rows, 0.2, np.float32)
    for gp in ([0, 2, 4], [1, 2, 5], [0, 3, 2, 5], []):
        with pytest.raises(ValueError, match="group_ptr"):
            sc.gradient(X, np.asarray(gp, np.int32), t)
    with pytest.raises(ValueError, match="target"):
        sc.gradient(X, np.asarray([0, 2, 5], np.int32), t[:4])
    # a well-formed batch passes the host checks
    assert scorer._check_groups(X, np.asarray([0, 2, 2, 5], np.int32), t).tolist() == [0, 2, 2, 5]
