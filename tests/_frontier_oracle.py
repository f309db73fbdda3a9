"""Test infrastructure: the device frontier's search (gpuboscia_gb300/csrc/frontier.cu)
restated on the CPU over the oracle's node relaxation (bit-identical to the FP64
kernel), so a device-frontier solve can be compared node for node.

Rules restated (one or two batch slots):
* the frontier is sorted by (bound, id); a round pops its first min(B, open) entries;
* a node's tolerance is the host's depth_dependent_tolerance, its cutoff (when
  enabled) the incumbent at its pop;
* branch_pow2 variables: the k most fractional integer variables above the
  tolerance, ties to the lower index;
* in batch order: the incumbent is the running minimum of the candidates'
  values (strict improvement), the certified bound max(inherited, f - gap) when
  the gap is finite and non-negative, a node is pruned at bound >= incumbent,
  an unconverged integral node continues from its iterate, a fractional one
  branches (children ids next_id + c, next_id advancing by max(8, 2^k) per
  branched node);
* the merge keeps entries below the incumbent; the search ends when nothing is
  open or in flight, or when the live bound is within the gap tolerances.
"""
from __future__ import annotations

import math

import numpy as np

import _oracle as O
from gpuboscia_gb300 import _abi as A


def _depth_tol(s, d):
    if d <= 0:
        return max(s.gpu_eps, s.gpu_eps_min)
    return max(s.gpu_eps_min, s.gpu_eps * math.pow(s.gpu_eps_decay, d))


def _within(bound, inc, abs_tol, rel_tol):
    if not (math.isfinite(bound) and math.isfinite(inc)):
        return False
    if abs(inc - bound) <= abs_tol:
        return True
    scale = min(abs(bound), abs(inc))
    return scale != 0.0 and (inc - bound) / scale <= rel_tol


def solve(problem, objective, lmo, s, slots: int = 1):
    n = problem.n_vars
    k = s.branch_k
    stride = max(8, 1 << k)
    flags = np.zeros(n, np.uint8)
    flags[list(problem.int_vars)] = 1
    int_vars = sorted(int(j) for j in problem.int_vars)
    alg = s.algorithm_c()
    root_x = None if s.root_initial_point is None else np.asarray(s.root_initial_point, np.float64)
    # open node: (bound, id, lb, ub, x or None, iterations, depth)
    frontier = [(s.natural_lower_bound, 0, np.asarray(problem.lb, np.float64).copy(),
                 np.asarray(problem.ub, np.float64).copy(), root_x, 0, 0)]
    inc, inc_x, next_id, done_nodes = math.inf, None, 1, 0
    inflight = [None, None]   # per slot: (nodes, relaxation outputs)

    def relax(batch, cut):
        N = len(batch)
        lb = np.stack([b[2] for b in batch])
        ub = np.stack([b[3] for b in batch])
        x = np.stack([b[4] if b[4] is not None else b[2] for b in batch])
        it = np.array([b[5] for b in batch], np.int32)
        st = np.array([A.NODE_INITIAL_POINT_SUPPLIED if b[4] is not None else 0 for b in batch], np.uint8)
        eps = np.array([_depth_tol(s, b[6]) for b in batch])
        return O.relax(objective, lmo, alg, x, lb, ub, eps, it, st, s.gpu_max_iters, flags, s.integer_tol,
                       cutoff=cut if s.incumbent_cutoff else None), eps

    def branch_vars(xv):
        cands = []
        for j in int_vars:
            fr = xv[j] - math.floor(xv[j])
            d = min(fr, 1.0 - fr)
            if d > s.integer_tol:
                cands.append((-d, j))
        cands.sort()
        return [j for _, j in cands[:k]]

    def finish(q):
        nonlocal inc, inc_x, next_id, done_nodes, frontier
        if inflight[q] is None:
            return []
        batch, (out, eps) = inflight[q]
        inflight[q] = None
        N = len(batch)
        cands = [v if (v < 1e299 and math.isfinite(v)) else math.inf for v in out["best_vertex_val"]]
        inc0 = inc
        run, incs = inc0, []
        for c in cands:
            run = min(run, c)
            incs.append(run)
        entries, n_cont, n_branched = [], 0, 0
        for i, b in enumerate(batch):
            st = int(out["status"][i])
            if st == A.NODE_INFEASIBLE:
                continue
            gap, val = float(out["gap"][i]), float(out["value"][i])
            lower = b[0]
            if math.isfinite(val) and math.isfinite(gap) and gap >= 0.0:
                lower = max(b[0], val - gap)
            certified = math.isfinite(gap) and gap >= 0.0 and gap < eps[i]
            if not lower < incs[i]:
                continue
            xi = out["x"][i]
            if st >= A.NODE_INTEGRAL_UNCONVERGED:
                if not certified:
                    entries.append((lower, b[1], b[2], b[3], xi.copy(), int(out["iterations"][i]), b[6]))
                    n_cont += 1
                continue
            vars_ = branch_vars(xi)
            if not vars_:
                continue
            base = next_id + n_branched * stride
            n_branched += 1
            for c in range(1 << len(vars_)):
                clb, cub = b[2].copy(), b[3].copy()
                for bit, v in enumerate(vars_):
                    if c >> bit & 1:
                        clb[v] = math.ceil(xi[v])
                    else:
                        cub[v] = math.floor(xi[v])
                entries.append((lower, base + c, clb, cub, None, 0, b[6] + 1))
        next_id += n_branched * stride
        done_nodes += N - n_cont
        final = incs[-1] if incs else inc0
        if final < inc0:
            src = cands.index(final)
            inc, inc_x = final, out["best_vertex"][src].copy()
        return entries

    for r in range(100000):
        q = 0 if slots == 1 else r & 1
        N = min(s.gpu_batch_size, len(frontier))
        popped, frontier = frontier[:N], frontier[N:]
        if N:
            inflight[q] = (popped, relax(popped, inc))
        other = q if slots == 1 else q ^ 1
        entries = finish(other)
        frontier = sorted(frontier + entries, key=lambda e: (e[0], e[1]))
        frontier = [e for e in frontier if e[0] < inc]
        still = slots == 2 and inflight[q] is not None
        bound = min(frontier[0][0], inc) if frontier else inc
        if still:
            bound = min(bound, popped[0][0])
        if not frontier and not still:
            return dict(objective=inc, dual_bound=inc, nodes=done_nodes, x=inc_x, tolerance=False)
        if _within(bound, inc, s.abs_gap_tol, s.rel_gap_tol):
            return dict(objective=inc, dual_bound=bound, nodes=done_nodes, x=inc_x, tolerance=True)
    raise RuntimeError("frontier restatement did not finish")
