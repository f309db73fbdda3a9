"""ctypes binding of the test oracle (oracle/fw_oracle.cpp) and of the
reference project's own CPU functions (oracle/_ref/libgbref.so, present only
where the reference tree was available at build time).

Test infrastructure only: the product package never imports this module.
"""
from __future__ import annotations

import ctypes as C
import math
import pathlib
import subprocess

import numpy as np

from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api

ROOT = pathlib.Path(__file__).resolve().parent.parent
ORACLE_SO = ROOT / "oracle" / "_build" / "liboracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libgbref.so"

_lib = None
_ref = None


def build():
    src = ROOT / "oracle" / "fw_oracle.cpp"
    if not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["bash", str(ROOT / "oracle" / "build.sh")], check=True)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(ORACLE_SO))
        P = C.POINTER
        L.oracle_relax_batch.argtypes = [P(A.Objective), P(A.LMO), P(A.Algorithm), P(A.NodeBatch), C.c_int]
        L.oracle_lmo_batch.argtypes = [P(A.LMO), C.c_int, C.c_int] + [C.c_void_p] * 6
        L.oracle_node_feasible_batch.argtypes = [P(A.LMO), C.c_int] + [C.c_void_p] * 4
        L.oracle_solve.argtypes = [P(A.Problem), P(A.Objective), P(A.LMO), P(A.Settings), P(A.Result)]
        L.oracle_objective_value.restype = C.c_double
        L.oracle_objective_value.argtypes = [P(A.Objective), C.c_void_p]
        L.oracle_objective_grad.argtypes = [P(A.Objective), C.c_void_p, C.c_void_p]
        L.oracle_objective_curvature.restype = C.c_double
        L.oracle_objective_curvature.argtypes = [P(A.Objective), C.c_void_p]
        L.oracle_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def ref():
    """The reference's CPU functions, or None when they were not built."""
    global _ref
    if _ref is None and REF_SO.exists():
        R = C.CDLL(str(REF_SO))
        d = C.c_double
        R.ref_birkhoff_lmo.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 5
        R.ref_simplex_lmo.argtypes = [C.c_int, C.c_int, C.c_int, d, C.c_void_p, C.c_int] + [C.c_void_p] * 6
        R.ref_box_lmo.argtypes = [C.c_int, C.c_int] + [C.c_void_p] * 6
        for f in ("ref_certified_fw_lower_bound", "ref_gap_relative", "ref_gap_absolute", "ref_quadratic_exact_step"):
            getattr(R, f).restype = d
            getattr(R, f).argtypes = [d, d, d] if f in ("ref_certified_fw_lower_bound", "ref_quadratic_exact_step") else [d, d]
        R.ref_gap_within_tolerance.argtypes = [d, d, d, d]
        R.ref_depth_dependent_tolerance.restype = d
        R.ref_depth_dependent_tolerance.argtypes = [d, d, d, C.c_int]
        R.ref_branch_pow2.argtypes = [C.c_int] + [C.c_void_p] * 3 + [C.c_void_p, C.c_int, C.c_int, d, C.c_void_p, C.c_void_p]
        _ref = R
    return _ref


def _p(a):
    return a.ctypes.data if a is not None else None


def algorithm(kind=A.ALG_DICG, ls=A.LS_OPEN_LOOP, secant_iters=4, secant_tol=1e-10, secant_denom_eps=1e-14,
              precision=A.PRECISION_FP64) -> A.Algorithm:
    return A.Algorithm(kind, ls, secant_iters, secant_tol, secant_denom_eps, precision)


def relax(objective, lmo, alg: A.Algorithm, x, lb, ub, eps, iterations=None, status=None, max_iters=100,
          flags=None, tol=1e-6, threads=1, cutoff=None):
    """oracle_relax_batch over host arrays; returns a dict of outputs (x, iterations, status, gap, value,
    best_vertex, best_vertex_val)."""
    L = lib()
    keep = api._Keep()
    x = np.array(x, dtype=np.float64, order="C", copy=True)
    N, n = x.shape
    lb = np.ascontiguousarray(lb, dtype=np.float64)
    ub = np.ascontiguousarray(ub, dtype=np.float64)
    eps = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, dtype=np.float64), (N,)))
    it = np.zeros(N, np.int32) if iterations is None else np.array(iterations, dtype=np.int32, copy=True)
    st = np.zeros(N, np.uint8) if status is None else np.array(status, dtype=np.uint8, copy=True)
    fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
    out = dict(x=x, iterations=it, status=st, gap=np.zeros(N), value=np.zeros(N), best_vertex=np.zeros((N, n)),
               best_vertex_val=np.zeros(N))
    o = objective.to_c("host", keep)
    lm = lmo.to_c(n, "host", keep)
    b = A.NodeBatch(N, max_iters, tol, _p(x), _p(lb), _p(ub), _p(eps), _p(it), _p(st), _p(out["gap"]),
                    _p(out["value"]), _p(out["best_vertex"]), _p(out["best_vertex_val"]), _p(fl))
    if cutoff is not None:
        cut = np.array([float(cutoff)])
        keep.items.append(cut)
        b.cutoff = _p(cut)
    rc = L.oracle_relax_batch(C.byref(o), C.byref(lm), C.byref(alg), C.byref(b), threads)
    if rc != 0:
        raise RuntimeError(L.oracle_last_error().decode())
    return out


def lmo_call(lmo, mode, direction, lb, ub, x=None, want_step=False):
    L = lib()
    keep = api._Keep()
    d = np.ascontiguousarray(direction, dtype=np.float64)
    cases, n = d.shape
    lm = lmo.to_c(n, "host", keep)
    out = np.zeros((cases, n))
    step = np.zeros(cases) if want_step else None
    xx = np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
    rc = L.oracle_lmo_batch(C.byref(lm), cases, mode, _p(d), _p(xx), _p(np.ascontiguousarray(lb, dtype=np.float64)),
                            _p(np.ascontiguousarray(ub, dtype=np.float64)), _p(out), _p(step))
    assert rc == 0
    return out, step


def feasible(lmo, lb, ub, flags=None):
    L = lib()
    keep = api._Keep()
    lb = np.ascontiguousarray(lb, dtype=np.float64)
    ub = np.ascontiguousarray(ub, dtype=np.float64)
    cases, n = lb.shape
    lm = lmo.to_c(n, "host", keep)
    out = np.zeros(cases, np.uint8)
    fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint8)
    L.oracle_node_feasible_batch(C.byref(lm), cases, _p(lb), _p(ub), _p(fl), _p(out))
    return out


def value(objective, x):
    keep = api._Keep()
    o = objective.to_c("host", keep)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    return lib().oracle_objective_value(C.byref(o), _p(xx))


def grad(objective, x):
    keep = api._Keep()
    o = objective.to_c("host", keep)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    g = np.zeros_like(xx)
    lib().oracle_objective_grad(C.byref(o), _p(xx), _p(g))
    return g


def solve(problem, objective, lmo, settings: api.Settings | None = None) -> api.Result:
    """Single-slot deterministic B&B (num_streams = 1)."""
    L = lib()
    settings = settings or api.Settings()
    keep = api._Keep()
    n = problem.n_vars
    o = objective.to_c("host", keep)
    lm = lmo.to_c(n, "host", keep)
    s = settings.to_c(keep)
    pr = api.problem_to_c(problem, keep)
    x = np.zeros(n)
    r = A.Result()
    r.x = x.ctypes.data
    rc = L.oracle_solve(C.byref(pr), C.byref(o), C.byref(lm), C.byref(s), C.byref(r))
    if rc != 0:
        raise ValueError(L.oracle_last_error().decode())
    return api.Result(r.objective, x if r.has_incumbent else np.zeros(0), r.dual_bound, r.nodes_processed,
                      r.elapsed_seconds, bool(r.reached_tolerance), bool(r.reached_time_limit),
                      bool(r.reached_node_limit), int(r.batches))


INF = math.inf
