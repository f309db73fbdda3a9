"""Branch and bound over several GPUs: one process per GPU, each relaxing its
own part of the frontier, with every exchange on the host.

Nodes are independent relaxations, so the data path has no collective: each
rank pops its best nodes, relaxes them in one batched call (``gbx_relax_batch``
on its own GPU) and branches. After every round the ranks exchange, through
``torch.distributed`` (NCCL between GPUs, gloo on CPU):

* the incumbent: all-reduce MIN of its value, then the winning rank's x;
* the live bound: all-reduce MIN of the best open bound, and the total number
  of open nodes (termination when the frontier is empty everywhere or the
  certified gap closes);
* work: ranks with an empty frontier take nodes from the fullest ranks
  (work stealing), so the search never idles a GPU while nodes are open.

A rank that fails (raises, dies, never joins) makes the next collective of its
peers fail within the process group's timeout; they raise
``RankFailure`` instead of waiting. Only the certified FW bound (value - gap of
a node whose gap is finite and non-negative) prunes, as in the single-GPU
solver (with ``settings.incumbent_cutoff`` each relaxation stops once that
bound reaches the shared incumbent); branching is branch_pow2 over the most fractional variables, or over
the learned scorer's choice when one is given.
"""
from __future__ import annotations

import dataclasses
import heapq
import math
from typing import Callable, List, Optional

import numpy as np

from . import _abi as A


class RankFailure(RuntimeError):
    """A peer rank failed or stopped answering; the search cannot continue."""


@dataclasses.dataclass
class Node:
    bound: float
    seq: int
    lb: np.ndarray
    ub: np.ndarray
    depth: int
    x: Optional[np.ndarray] = None       # warm start (continuation)
    iterations: int = 0

    def __lt__(self, other):
        return (self.bound, self.seq) < (other.bound, other.seq)


@dataclasses.dataclass
class DistributedResult:
    objective: float
    x: Optional[np.ndarray]
    dual_bound: float
    nodes_processed: int          # this rank
    nodes_total: int              # all ranks
    rounds: int
    stolen: int                   # nodes this rank received from others


# relax(lbs, ubs, xs, eps, iterations, status[, cutoff=incumbent]) -> dict(x, gap, value, status,
#                                                     iterations, best_vertex, best_vertex_val)
# (cutoff is passed only when settings.incumbent_cutoff is set)
RelaxFn = Callable[..., dict]


def gpu_relax_fn(objective, lmo, settings, integer_flags):
    """The product relaxation: gbx_relax_batch on this rank's GPU."""
    import torch
    from . import api
    alg = settings.algorithm_c()
    flags = torch.from_numpy(np.ascontiguousarray(integer_flags, np.uint8)).cuda()

    def relax(lbs, ubs, xs, eps, iterations, status, cutoff=None):
        T = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a if dt is None else np.asarray(a, dt))).cuda()
        x = T(xs)
        it = T(iterations, np.int32)
        st = T(status, np.uint8)
        out = api.relax_batch(objective, lmo, alg, x, T(lbs), T(ubs), T(eps), it, st, settings.gpu_max_iters, flags,
                              settings.integer_tol, cutoff=cutoff)
        torch.cuda.synchronize()
        return dict(x=x.cpu().numpy(), gap=out["gap"].cpu().numpy(), value=out["value"].cpu().numpy(),
                    status=st.cpu().numpy(), iterations=it.cpu().numpy(),
                    best_vertex=out["best_vertex"].cpu().numpy(),
                    best_vertex_val=out["best_vertex_val"].cpu().numpy())
    return relax


def _gap_ok(bound, inc, abs_tol, rel_tol):
    if not math.isfinite(inc) or bound == -math.inf:
        return False
    g = abs(inc - bound)
    return g <= abs_tol or g / max(abs(inc), 1e-12) <= rel_tol


def _most_fractional(x, int_vars, k, tol):
    fr = x[int_vars] - np.floor(x[int_vars])
    dist = np.minimum(fr, 1 - fr)
    idx = np.argsort(-dist, kind="stable")
    return [int(int_vars[i]) for i in idx[:k] if dist[i] > tol]


def solve(problem, settings, relax: RelaxFn, group=None, branch_vars: Optional[Callable] = None,
          max_rounds: int = 100000) -> DistributedResult:
    """Run the distributed search on this rank (call it on every rank)."""
    import torch
    import torch.distributed as dist

    def coll(fn, *a, **kw):
        try:
            return fn(*a, group=group, **kw)
        except Exception as e:   # noqa: BLE001 -- any transport error means a lost peer
            raise RankFailure(f"collective {fn.__name__} failed: {e}") from e

    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    n = problem.n_vars
    int_vars = np.asarray(list(problem.int_vars), np.int64)
    B = settings.gpu_batch_size
    k = settings.branch_k
    tol = settings.integer_tol
    queue: List[Node] = []
    seq = 0
    if rank == 0:
        queue.append(Node(settings.natural_lower_bound, 0, np.asarray(problem.lb, np.float64).copy(),
                          np.asarray(problem.ub, np.float64).copy(), 0))
    seq = rank + 1
    inc_val, inc_x = math.inf, None
    processed = stolen = rounds = 0
    total_processed = 0
    global_bound = settings.natural_lower_bound

    def push(node):
        nonlocal seq
        node.seq = seq
        seq += world
        heapq.heappush(queue, node)

    while rounds < max_rounds:
        rounds += 1
        # ---- relax a batch of this rank's best open nodes
        batch = []
        while queue and len(batch) < B:
            nd = heapq.heappop(queue)
            if nd.bound >= inc_val - settings.abs_gap_tol:
                continue
            batch.append(nd)
        if batch:
            N = len(batch)
            lbs = np.stack([b.lb for b in batch])
            ubs = np.stack([b.ub for b in batch])
            xs = np.stack([b.x if b.x is not None else np.clip(b.lb, None, None) for b in batch])
            its = np.array([b.iterations for b in batch], np.int32)
            sts = np.array([A.NODE_INITIAL_POINT_SUPPLIED if b.x is not None else 0 for b in batch], np.uint8)
            eps = np.array([max(settings.gpu_eps_min, settings.gpu_eps * settings.gpu_eps_decay ** b.depth)
                            for b in batch])
            # with the incumbent cutoff a node stops iterating once its FW bound
            # reaches the shared incumbent: it is pruned below all the same
            cut = {"cutoff": inc_val} if getattr(settings, "incumbent_cutoff", 0) and math.isfinite(inc_val) else {}
            r = relax(lbs, ubs, xs, eps, its, sts, **cut)
            processed += N
            for i, nd in enumerate(batch):
                bv = r["best_vertex_val"][i]
                if bv < 1e299 and math.isfinite(bv) and bv < inc_val:
                    inc_val, inc_x = float(bv), r["best_vertex"][i].copy()
                st = int(r["status"][i])
                if st == A.NODE_INFEASIBLE:
                    continue
                gap, val = r["gap"][i], r["value"][i]
                bound = nd.bound
                if math.isfinite(gap) and gap >= 0:
                    bound = max(bound, float(val - gap))
                certified = math.isfinite(gap) and 0 <= gap < eps[i]
                if bound >= inc_val - settings.abs_gap_tol:
                    continue
                if st >= A.NODE_INTEGRAL_UNCONVERGED:
                    if not certified:   # continue the same node from its iterate
                        push(Node(bound, 0, nd.lb, nd.ub, nd.depth, r["x"][i].copy(), int(r["iterations"][i])))
                    continue
                xi = r["x"][i]
                vars_ = branch_vars(nd, xi) if branch_vars else _most_fractional(xi, int_vars, k, tol)
                for mask in range(1 << len(vars_)):
                    clb, cub = nd.lb.copy(), nd.ub.copy()
                    for b_, v in enumerate(vars_):
                        if mask >> b_ & 1:
                            clb[v] = math.ceil(xi[v])
                        else:
                            cub[v] = math.floor(xi[v])
                    push(Node(bound, 0, clb, cub, nd.depth + 1))
        # ---- exchange: incumbent, bound, frontier size
        t = torch.tensor([inc_val, float(rank)], dtype=torch.float64)
        allv = [torch.zeros(2, dtype=torch.float64) for _ in range(world)]
        coll(dist.all_gather, allv, t)
        vals = [(float(v[0]), int(v[1])) for v in allv]
        best_val, owner = min(vals)
        if best_val < math.inf:
            xs_obj = [inc_x if rank == owner else None]
            coll(dist.broadcast_object_list, xs_obj, src=owner)
            inc_val, inc_x = best_val, np.asarray(xs_obj[0])
        local_bound = queue[0].bound if queue else math.inf
        for nd in queue:
            local_bound = min(local_bound, nd.bound)
        st = torch.tensor([local_bound, float(len(queue)), float(processed)], dtype=torch.float64)
        gathered = [torch.zeros(3, dtype=torch.float64) for _ in range(world)]
        coll(dist.all_gather, gathered, st)
        sizes = [int(g_[1]) for g_ in gathered]
        total_processed = int(sum(int(g_[2]) for g_ in gathered))
        gb = min(float(g_[0]) for g_ in gathered)
        global_bound = min(gb, inc_val)
        if sum(sizes) == 0 or _gap_ok(global_bound, inc_val, settings.abs_gap_tol, settings.rel_gap_tol):
            break
        # ---- work stealing: idle ranks take nodes from the fullest one
        idle = [q for q in range(world) if sizes[q] == 0]
        donor = int(np.argmax(sizes))
        if idle and sizes[donor] >= 2:
            give = []
            if rank == donor:
                share = sizes[donor] // (len(idle) + 1)
                queue.sort()
                keep, give = [], []
                for j, nd in enumerate(queue):   # alternate so donor and takers get good nodes
                    (give if (j % (len(idle) + 1)) and len(give) < share * len(idle) else keep).append(nd)
                queue[:] = keep
                heapq.heapify(queue)
            obj = [give if rank == donor else None]
            coll(dist.broadcast_object_list, obj, src=donor)
            if rank in idle:
                mine = obj[0][idle.index(rank)::len(idle)]
                for nd in mine:
                    push(nd)
                stolen += len(mine)
    return DistributedResult(inc_val, inc_x, global_bound, processed, total_processed, rounds, stolen)
