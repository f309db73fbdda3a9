"""Generate tests/golden/reference_cpu.json from the reference project's own
CPU functions (oracle/_ref/libgbref.so, built by oracle/build.sh from the
reference headers).

Inputs are exact binary fractions (integers / 8) so the JSON round trip is
lossless and equal costs occur often, which exercises the lowest-index
tie-break of the Hungarian oracle. Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parent.parent))

import _oracle as O  # noqa: E402


def frac(rng, shape, lo=-40, hi=40):
    return rng.integers(lo, hi + 1, size=shape) / 8.0


def birkhoff_cases(rng, order, cases):
    out = []
    n = order * order
    for s in range(cases):
        cost = frac(rng, n)
        lb = np.zeros(n)
        ub = np.ones(n)
        p = rng.permutation(order)
        for r in range(order):
            for c in range(order):
                if c != p[r] and rng.random() < 0.15:
                    ub[r * order + c] = 0.0
        if s % 3:
            r = int(rng.integers(0, order))
            lb[r * order + p[r]] = 1.0
        # a point of the face: convex combination of two feasible permutations
        q = p.copy()
        i, j = rng.choice(order, 2, replace=False)
        forced_rows = {r for r in range(order) if lb[r * order + p[r]] > 0.5}
        if i not in forced_rows and j not in forced_rows and ub[i * order + p[j]] and ub[j * order + p[i]]:
            q[i], q[j] = p[j], p[i]
        x = np.zeros(n)
        x[np.arange(order) * order + p] += 0.625
        x[np.arange(order) * order + q] += 0.375
        out.append(dict(order=order, cost=cost.tolist(), lb=lb.tolist(), ub=ub.tolist(), x=x.tolist()))
    return out


def main():
    R = O.ref()
    if R is None:
        raise SystemExit("oracle/_ref/libgbref.so is missing: run oracle/build.sh where the reference exists")
    rng = np.random.default_rng(20261203)
    doc = {"generator": "tests/golden/make_golden.py", "source": "reference CPU functions via oracle/ref_shim.cu"}

    bk = []
    for order, cases in ((3, 6), (5, 8), (7, 20), (8, 6), (12, 6), (36, 3)):
        for c in birkhoff_cases(rng, order, cases):
            n = order * order
            cost, lb, ub, x = (np.array(c[k]) for k in ("cost", "lb", "ub", "x"))
            fwd = np.zeros(n)
            R.ref_birkhoff_lmo(order, 0, cost.ctypes.data, None, lb.ctypes.data, ub.ctypes.data, fwd.ctypes.data)
            face = np.zeros(n)
            zl = np.zeros(n)
            on = np.ones(n)
            R.ref_birkhoff_lmo(order, 1, cost.ctypes.data, x.ctypes.data, zl.ctypes.data, on.ctypes.data,
                               face.ctypes.data)
            c["forward"] = fwd.tolist()
            c["inface"] = face.tolist()
            bk.append(c)
    doc["birkhoff"] = bk

    bx = []
    for s in range(10):
        n = 24
        g = frac(rng, n)
        g[::5] = 0.0
        lb = rng.integers(-2, 1, n).astype(float)
        ub = lb + rng.integers(0, 3, n)
        x = lb + (ub - lb) * rng.integers(0, 9, n) / 8.0
        fwd = np.zeros(n)
        R.ref_box_lmo(0, n, g.ctypes.data, None, lb.ctypes.data, ub.ctypes.data, fwd.ctypes.data, None)
        face = np.zeros(n)
        step = np.zeros(1)
        R.ref_box_lmo(1, n, g.ctypes.data, x.ctypes.data, lb.ctypes.data, ub.ctypes.data, face.ctypes.data,
                      step.ctypes.data)
        bx.append(dict(g=g.tolist(), lb=lb.tolist(), ub=ub.tolist(), x=x.tolist(), forward=fwd.tolist(),
                       inface=face.tolist(), step=float(step[0])))
    doc["box"] = bx

    sx = []
    for s in range(16):
        n = 10
        eq = s % 2
        ints = sorted(rng.choice(n, 6, replace=False).tolist())
        rhs = float(rng.integers(4, 9))
        g = frac(rng, n)
        lb = np.zeros(n)
        lb[ints[0]] = 1.0
        ub = np.where(np.isin(np.arange(n), ints), rng.integers(1, 4, n), rhs).astype(float)
        x = np.zeros(n)
        x[ints[0]] = 1.0
        # integral point of the set, then an interior shift of mass to a continuous coordinate
        rest = rhs - 1.0 if eq else rhs - 2.0
        k = [j for j in range(n) if j not in ints][0]
        x[k] = rest
        iv = np.array(ints, dtype=np.int32)
        fwd = np.zeros(n)
        R.ref_simplex_lmo(eq, 0, n, rhs, iv.ctypes.data, len(ints), g.ctypes.data, None, lb.ctypes.data,
                          ub.ctypes.data, fwd.ctypes.data, None)
        face = np.zeros(n)
        step = np.zeros(1)
        R.ref_simplex_lmo(eq, 1, n, rhs, iv.ctypes.data, len(ints), g.ctypes.data, x.ctypes.data, lb.ctypes.data,
                          ub.ctypes.data, face.ctypes.data, step.ctypes.data)
        sx.append(dict(equality=eq, ints=ints, rhs=rhs, g=g.tolist(), lb=lb.tolist(), ub=ub.tolist(), x=x.tolist(),
                       forward=fwd.tolist(), inface=face.tolist(), step=float(step[0])))
    doc["simplex"] = sx

    inf = float("inf")
    nan = float("nan")
    gaps = []
    for b, i in [(9.0, 10.0), (0.25, 0.75), (-10.0, -9.0), (0.0, 0.0), (0.0, 1.0), (-1.0, 0.0), (99.0, 100.0),
                 (-1.0, 1.0), (inf, 1.0), (1.0, inf), (-inf, 1.0), (nan, 1.0)]:
        gaps.append([b, i, R.ref_gap_absolute(b, i), R.ref_gap_relative(b, i),
                     R.ref_gap_within_tolerance(b, i, 0.01, 0.01), R.ref_gap_within_tolerance(b, i, 0.0, 0.105)])
    doc["gaps"] = gaps
    doc["certified"] = [[a, b, c, R.ref_certified_fw_lower_bound(a, b, c)]
                        for a, b, c in [(-7, 10, 3), (-7, 10, -1e-12), (-7, 10, nan), (-7, inf, 1), (5, 10, 1)]]
    doc["depth_tol"] = [[d, R.ref_depth_dependent_tolerance(1e-3, 0.8, 1e-6, d)] for d in (0, 1, 2, 5, 30, 1000)]
    doc["quad_step"] = [[g, c, m, R.ref_quadratic_exact_step(g, c, m)]
                        for g, c, m in [(3, 6, 1), (3, 2, .25), (-3, 6, 1), (3, 0, 1), (0, 0, 1), (-1, -4, 1),
                                        (3, 6, 0), (3e-100, 6e-100, 1), (7, 28, 1)]]
    br = []
    for x, k in [([1.5, 2.5, 3.9], 3), ([1.0, 2.5, 3.0], 3), ([0.3, 0.7, 0.5, 0.9], 2)]:
        n = len(x)
        xv = np.array(x)
        lb = np.zeros(n)
        ub = np.full(n, 5.0)
        iv = np.arange(n, dtype=np.int32)
        ol = np.zeros(8 * n)
        ou = np.zeros(8 * n)
        cnt = R.ref_branch_pow2(n, lb.ctypes.data, ub.ctypes.data, xv.ctypes.data, iv.ctypes.data, n, k, 1e-6,
                                ol.ctypes.data, ou.ctypes.data)
        br.append(dict(x=x, k=k, lb=ol[:cnt * n].reshape(cnt, n).tolist(), ub=ou[:cnt * n].reshape(cnt, n).tolist()))
    doc["branch_pow2"] = br

    # the box oracles at the edges of the in-face tolerance 1e-6 + 1e-4 |bound|
    # and with signed-zero directions (own generator: the cases above stay as they were)
    re_ = np.random.default_rng(4242)
    be = []
    for s in range(8):
        n = 48
        g = frac(re_, n)
        g[::4] = 0.0
        g[2::8] = -0.0
        lb = re_.integers(-3, 2, n).astype(float)
        ub = lb + re_.integers(0, 3, n)
        tu = 1e-6 + 1e-4 * np.abs(ub)
        tl = 1e-6 + 1e-4 * np.abs(lb)
        pick = re_.integers(0, 8, n)
        x = np.choose(pick, [ub, lb, ub - 0.5 * tu, lb + 0.5 * tl, ub - tu, lb + tl, ub - 2.0 * tu,
                             lb + 2.0 * tl])
        fwd = np.zeros(n)
        R.ref_box_lmo(0, n, g.ctypes.data, None, lb.ctypes.data, ub.ctypes.data, fwd.ctypes.data, None)
        face = np.zeros(n)
        R.ref_box_lmo(1, n, g.ctypes.data, x.ctypes.data, lb.ctypes.data, ub.ctypes.data, face.ctypes.data, None)
        be.append(dict(g=g.tolist(), lb=lb.tolist(), ub=ub.tolist(), x=x.tolist(), forward=fwd.tolist(),
                       inface=face.tolist()))
    doc["box_edges"] = be

    out = HERE / "reference_cpu.json"
    out.write_text(json.dumps(doc, allow_nan=True, separators=(",", ":")))
    print(out, out.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
