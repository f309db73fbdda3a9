#!/usr/bin/env python
"""Benchmark of the node-relaxation hot path on GB300, on the metric's own
configuration.

Default workload: Birkhoff graph matching on an isomorphic pair of 10-regular
graphs on 400 vertices (160,000 binary variables, B = P A P'), branch and bound
with 1024-node batches, mixed precision, the learned branching scorer, the
device frontier and the incumbent cutoff. A step is one round of that search
(pop a batch, relax it, branch and merge the batch of the round before), timed
on the device by CUDA events on the search's stream; the first rounds grow the
frontier to full batches and are the warm-up, the last --steps rounds are timed.
value = B&B nodes per second over the timed rounds (whole batches resident in
HBM); e2e = nodes per second of the whole gbx_solve call through the Python API
(instance uploaded from host arrays, incumbent read back).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload NAME]

Other workloads (`--workload`): birkhoff_regular120 (the same search on the
order-120 pair, 256-node batches) and, one relaxation launch per step,
birkhoff_gnp36, box_qp64 and portfolio100.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time to certified 1e-6 gap & B&B nodes/s: batched+learned vs plain, 1 GB300"

WORKLOADS = {
    # name: instance family and size, nodes per batch, algorithm (0 FW, 1 DICG), line search (4 quadratic
    # exact), FW iterations per dispatch, and the measurement: "bnb" times rounds of a gbx_solve search,
    # "relax" times one gbx_relax_batch launch over a synthetic batch of open nodes
    "birkhoff_regular400": dict(kind="birkhoff", order=400, nodes=1024, alg=1, ls=4, iters=20, mode="bnb"),
    "birkhoff_regular120": dict(kind="birkhoff", order=120, nodes=256, alg=1, ls=4, iters=100, mode="bnb"),
    "birkhoff_gnp36": dict(kind="birkhoff", order=36, nodes=256, alg=1, ls=4, iters=100, mode="relax"),
    "box_qp64": dict(kind="box", n=64, nodes=1024, alg=0, ls=4, iters=200, mode="relax"),
    "portfolio100": dict(kind="portfolio", n=200, nodes=64, alg=0, ls=4, iters=500, mode="relax"),
}
DEFAULT_WORKLOAD = "birkhoff_regular400"
BRANCH_K = 3   # branch_pow2's default: 8 children per branched node


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def workload_flags(name, n):
    """Integer flags of the workload's variables (the portfolio's z only)."""
    flags = np.ones(n, np.uint8)
    if WORKLOADS[name]["kind"] == "portfolio":
        flags[: n // 2] = 0
    return flags


def make_instance(name):
    from gpuboscia_gb300 import instances
    w = WORKLOADS[name]
    if w["kind"] == "box":
        return instances.box_qp(n=w["n"])
    if w["kind"] == "portfolio":
        return instances.portfolio(assets=w["n"] // 2)
    if name.startswith("birkhoff_gnp"):
        return instances.birkhoff_gnp(order=w["order"])
    if w["order"] == 400:
        return instances.birkhoff_regular_isomorphic(order=w["order"])
    return instances.birkhoff_regular_perturbed(order=w["order"])


def make_workload(name, nodes, rank):
    """The instance and a batch of open nodes with uneven fixings and
    depth-dependent tolerances (lb, ub, eps)."""
    from gpuboscia_gb300 import instances
    w = WORKLOADS[name]
    inst = make_instance(name)
    if w["kind"] == "box":
        lb, ub = instances.box_node_batch(w["n"], nodes, seed=4242 + rank)
    elif w["kind"] == "portfolio":
        lb, ub = instances.portfolio_node_batch(w["n"] // 2, 10, nodes, seed=4242 + rank)
    else:
        lb, ub = instances.birkhoff_node_batch(w["order"], nodes, seed=4242 + rank)
    rng = np.random.Generator(np.random.PCG64(77 + rank))
    depth = rng.integers(0, 13, nodes)
    eps = np.maximum(1e-6, 1e-3 * 0.8 ** depth)
    return inst, lb, ub, eps


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index, period_ms=50):
        self.dev = device_index
        self.period = period_ms
        self.proc = None

    def __enter__(self):
        import select
        self.first = ""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", str(self.period)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            # the timed region starts once sampling runs (the first sample is the state entering it)
            if select.select([self.proc.stdout], [], [], 5.0)[0]:
                self.first = self.proc.stdout.readline()
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.text = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.text, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.text, _ = self.proc.communicate()
            self.text = self.first + self.text

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (getattr(self, "text", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(inst, lb, ub, eps, alg_kind, ls, iters, budget_s=12.0, flags=None):
    """The oracle on the machine's host cores over a bounded sample of the batch."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    threads = os.cpu_count() or 1
    n = lb.shape[1]
    flags = np.ones(n, np.uint8) if flags is None else flags
    alg = O.algorithm(alg_kind, ls)
    count = min(len(lb), max(threads, 8))
    t0 = time.perf_counter()
    O.relax(inst.objective, inst.lmo, alg, lb[:count].copy(), lb[:count], ub[:count], eps[:count],
            max_iters=iters, flags=flags, threads=threads)
    dt = time.perf_counter() - t0
    done = count
    while dt < budget_s and done < len(lb):
        c2 = min(len(lb) - done, count)
        t1 = time.perf_counter()
        O.relax(inst.objective, inst.lmo, alg, lb[done:done + c2].copy(), lb[done:done + c2], ub[done:done + c2],
                eps[done:done + c2], max_iters=iters, flags=flags, threads=threads)
        dt += time.perf_counter() - t1
        done += c2
    return done / dt, threads, done, dt


def ref_sample_nodes(args):
    """Nodes of the CPU samples: one batch's worth, at most 32 at order 400."""
    w = WORKLOADS[args.workload]
    return min(args.nodes, 32) if w.get("order", 0) >= 400 else args.nodes


def run_reference(args, rank, world):
    """--impl reference: the oracle port of the reference's relaxation on the
    host cores (a B&B node is one relaxation; the host bookkeeping around it is
    negligible at these sizes)."""
    if rank != 0:
        return
    inst, lb, ub, eps = make_workload(args.workload, ref_sample_nodes(args), 0)
    w = WORKLOADS[args.workload]
    for _ in range(args.warmup):
        cpu_sample(inst, lb, ub, eps, w["alg"], w["ls"], args.iters, budget_s=0.0,
                   flags=workload_flags(args.workload, lb.shape[1]))
    vals, times, done = [], [], 0
    for _ in range(args.steps):
        v, threads, done, dt = cpu_sample(inst, lb, ub, eps, w["alg"], w["ls"], args.iters, budget_s=args.ref_budget,
                                          flags=workload_flags(args.workload, lb.shape[1]))
        vals.append(v)
        times.append(dt)
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "nodes/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * statistics.mean(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(config_dict(args), precision="fp64 (CPU oracle)"),
            "cpu_baseline": {"value": value, "unit": "nodes/s", "cores": threads, "kind": "port",
                             "sample": f"{done} open nodes of the workload per step (uneven fixings), "
                                       f"relaxed with {args.iters} iterations max each"},
            "e2e": {"value": value, "unit": "nodes/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_dict(args):
    w = WORKLOADS[args.workload]
    d = {"workload": args.workload}
    if w["kind"] == "birkhoff":
        d.update(order=w["order"], variables=w["order"] ** 2)
    else:
        d.update(variables=w["n"])
    d.update({"nodes_per_batch": args.nodes, "max_iters_per_dispatch": args.iters,
              "algorithm": "DICG" if w["alg"] == 1 else "Frank-Wolfe", "line_search": "quadratic_exact",
              "precision": args.precision})
    if w["mode"] == "bnb":
        d.update({"step": "one round of the branch-and-bound search (a batch popped, relaxed, branched, merged)",
                  "search": "device frontier, learned branching scorer (branch_pow2, k=3), incumbent cutoff",
                  "l2": "inputs larger than L2 (each round streams its batch's node vectors)"})
    else:
        d["l2"] = "flushed between timed steps (256 MiB write)"
    if getattr(args, "launch_shape", "auto") != "auto":
        d["launch_shape"] = args.launch_shape
    if getattr(args, "oracle_warps", -1) != -1:
        d["oracle_warps"] = args.oracle_warps
        if getattr(args, "tuned_shape", None):
            d["tuned_shape"] = {"tensor_core": args.tuned_shape[0], "persistent": args.tuned_shape[1]}
    return d


# ---------------------------------------------------------------- learned scorer and graph pairs
def _pair(seed, order=9):
    from gpuboscia_gb300 import instances
    rng = np.random.Generator(np.random.PCG64(seed))
    return instances.graph_matching(order, instances.gnp_graph(rng, order, 0.5),
                                    instances.gnp_graph(rng, order, 0.5), f"pair{order}_{seed}")


def _trained_scorer():
    """The learned scorer: strong-branching labels of four G(9, 1/2) pairs (seeds
    100-103, disjoint from the held-out pairs 200-203), 400 Adam epochs. Its 16
    features do not depend on the order, so the same network ranks candidates
    at every order."""
    from gpuboscia_gb300 import scorer
    data = scorer.Dataset.concat([scorer.collect_strong_branching(_pair(100 + k), max_nodes=30, max_candidates=64)
                                  for k in range(4)])
    sc = scorer.Scorer(32, seed=0)
    sc.train(data, epochs=400, lr=3e-3)
    return sc


def _solve_timed(inst, prec, scorer_obj, batch, streams, limit, device_frontier=0, cutoff=0, iters=500,
                 node_limit=0, trace=0, capacity=0, autotune=1):
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api
    s = inst.settings
    s.gpu_batch_size = batch
    s.num_streams = streams
    s.gpu_max_iters = iters
    s.line_search = A.LS_QUADRATIC_EXACT
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.time_limit_seconds = limit
    s.precision = prec
    s.scorer = scorer_obj
    s.device_frontier = device_frontier
    s.incumbent_cutoff = cutoff
    s.node_limit = node_limit
    s.round_trace = trace
    s.frontier_capacity = capacity
    s.autotune = autotune
    t0 = time.perf_counter()
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    wall = time.perf_counter() - t0
    gap = abs(r.objective - r.dual_bound) if math.isfinite(r.objective) else math.inf
    certified = bool(not r.reached_time_limit and not r.reached_node_limit
                     and (gap <= 1e-6 or gap <= 1e-6 * abs(r.objective)))
    return wall, r, certified


def _solve_summary(wall, r, cert):
    return {"seconds": wall, "nodes": r.nodes_processed, "nodes_per_s": r.nodes_processed / wall,
            "batches": r.batches, "objective": r.objective, "dual_bound": r.dual_bound, "certified": cert,
            "time_limit": bool(r.reached_time_limit), "node_limit": bool(r.reached_node_limit)}


# time-to-gap configurations over the held-out pairs:
# precision, learned scorer, batch, streams, device frontier, incumbent cutoff
PAIR_CONFIGS = {
    "plain_fp64": (0, False, 64, 1, 0, 0),
    "mixed": (1, False, 64, 1, 0, 0),
    "mixed_learned": (1, True, 64, 1, 0, 0),
    "mixed_learned_256x4": (1, True, 256, 4, 0, 0),
    "device_frontier_mixed_1024": (1, False, 1024, 1, 1, 0),
    "device_frontier_mixed_learned_1024": (1, True, 1024, 1, 1, 0),
    "full_stack": (1, True, 1024, 1, 1, 1),
}


def _solve_pairs(name, sc, limit):
    prec, use, batch, streams, dev, cut = PAIR_CONFIGS[name]
    tot_s, tot_n, cert = 0.0, 0, True
    for k in range(4):
        wall, r, c = _solve_timed(_pair(200 + k), prec, sc if use else None, batch, streams, limit, dev, cut)
        tot_s += wall
        tot_n += r.nodes_processed
        cert = cert and c
    return {"seconds": tot_s, "nodes": tot_n, "certified": cert}


def certified_cases(sc, limit):
    """Instances whose 1e-6 gap closes within a bench run, plain against the
    full stack: the order-36 G(36, 1/2) pair (the root's LMO vertex is the
    isomorphism) and four held-out G(9, 1/2) pairs (non-isomorphic: the tree
    branches, ~3-4k nodes each)."""
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import instances
    out = {}
    gnp = instances.birkhoff_gnp(order=36)
    for name, prec in (("plain_fp64", A.PRECISION_FP64), ("mixed", A.PRECISION_MIXED)):
        wall, r, cert = _solve_timed(gnp, prec, None, 256, 2, limit)
        out.setdefault("gnp36", {})[name] = _solve_summary(wall, r, cert)
    pairs = {"instances": "4 held-out G(9,1/2) pairs; batch 64 x 1 stream, host frontier, unless named; "
                          "full_stack = mixed + learned + device frontier (1024-node rounds) + incumbent cutoff"}
    for name in PAIR_CONFIGS:
        pairs[name] = _solve_pairs(name, sc, limit)
    pairs["full_vs_plain"] = pairs["plain_fp64"]["seconds"] / max(pairs["full_stack"]["seconds"], 1e-9)
    out["graph_pairs"] = pairs
    return out


# ---------------------------------------------------------------- relaxation arms on one batch
def relax_arms(inst, lb, ub, eps, w, iters, check_nodes=4):
    """The same open nodes relaxed by the plain FP64 method and by mixed
    precision at the same iteration budget (one gbx_relax_batch launch each,
    CUDA events on the launching stream): nodes/s, mean certified bound
    f(x) - gap, converged fraction. The mixed certificate of a sample of nodes
    is re-evaluated by the oracle at the returned iterate (an FP64 certificate:
    the error is that of the GPU's FP64 arithmetic against the oracle's)."""
    import torch
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    dev = torch.device("cuda")
    N, n = lb.shape
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_lb, d_ub, d_eps = T(lb), T(ub), T(eps)
    d_flags = T(np.ones(n, np.uint8))
    stream = torch.cuda.current_stream()
    out = {}
    for name, prec in (("plain_fp64", A.PRECISION_FP64), ("mixed", A.PRECISION_MIXED)):
        alg = A.Algorithm(w["alg"], w["ls"], 4, 1e-10, 1e-14, prec)
        x = d_lb.clone()
        it = torch.zeros(N, dtype=torch.int32, device=dev)
        st = torch.zeros(N, dtype=torch.uint8, device=dev)
        rl = api.BatchRelaxer(inst.objective, inst.lmo, alg, x, d_lb, d_ub, d_eps, it, st, iters, d_flags, 1e-6,
                              stream)
        rl.launch()   # warm-up (module load, launch attributes)
        x.copy_(d_lb)
        it.zero_()
        st.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        rl.launch()
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        val, gap, stat = rl.value.cpu().numpy(), rl.gap.cpu().numpy(), st.cpu().numpy()
        ok = np.isfinite(gap) & (stat != 2)
        out[name] = {"nodes": N, "ms": ms, "nodes_per_s": N / (ms / 1000.0),
                     "node_iterations": int(it.sum().item()),
                     "mean_certified_bound": float(np.mean((val - gap)[ok])) if ok.any() else None,
                     "converged_fraction": float(np.isin(stat, (1, 4)).mean())}
        if name == "mixed" and check_nodes > 0:
            import _oracle as O
            k = min(check_nodes, N)
            oalg = O.algorithm(w["alg"], w["ls"])
            xs = x.cpu().numpy()[:k]
            ref = O.relax(inst.objective, inst.lmo, oalg, xs, lb[:k], ub[:k], eps[:k],
                          iterations=it.cpu().numpy()[:k], status=np.full(k, 0x80, np.uint8), max_iters=0,
                          threads=os.cpu_count() or 1)
            out[name]["certificate_check"] = {
                "nodes": k, "max_abs_gap_error": float(np.max(np.abs(ref["gap"] - gap[:k]))),
                "max_abs_value_error": float(np.max(np.abs(ref["value"] - val[:k])))}
    return out


def cluster_arms(inst, w, lb, ub, eps, iters, sizes=(1, 38, 152)):
    """Large orders, mixed precision: one CTA per node (two nodes per SM) with
    each integer oracle on four warps (the default) or on one warp, and the
    cluster shape (four CTAs per node, the oracle costs split across their
    shared memories), on the first N nodes of the batch, one launch each (CUDA
    events). Identical results; the question is time per launch."""
    import torch
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api
    m = w["order"]
    n = m * m
    alg = A.Algorithm(w["alg"], w["ls"], 4, 1e-10, 1e-14, A.PRECISION_MIXED)
    out = {}
    try:
        for N in sizes:
            if N > lb.shape[0]:
                continue
            row = {}
            for name, shape, ow in (("one_cta", 0, -1), ("one_cta_one_warp_oracles", 0, 1), ("cluster4", 2, -1)):
                api.set_launch_shape(inst.objective, inst.lmo, alg, n, -1, shape, oracle_warps=ow)
                T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
                d_lb, d_ub, d_eps = T(lb[:N]), T(ub[:N]), T(eps[:N])
                flags = T(np.ones(n, np.uint8))
                x = d_lb.clone()
                it = torch.zeros(N, dtype=torch.int32, device="cuda")
                st = torch.zeros(N, dtype=torch.uint8, device="cuda")
                rl = api.BatchRelaxer(inst.objective, inst.lmo, alg, x, d_lb, d_ub, d_eps, it, st, iters, flags, 1e-6,
                                      torch.cuda.current_stream())
                rl.launch()
                x.copy_(d_lb)
                it.zero_()
                st.zero_()
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                rl.launch()
                b.record()
                torch.cuda.synchronize()
                ms = a.elapsed_time(b)
                row[name] = {"ms": ms, "nodes_per_s": N / (ms / 1000.0), "x_sum": float(x.sum().item())}
            row["same_iterates"] = len({r["x_sum"] for r in row.values()}) == 1
            out[f"nodes_{N}"] = row
    finally:
        api.set_launch_shape(inst.objective, inst.lmo, alg, n, -1, 0)
    return out


# ---------------------------------------------------------------- the search (bnb mode)
def _host_available_bytes():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return 0


def run_bnb(args, rank, world):
    """Rounds of the full-stack search on the workload's instance (see the
    module docstring), plus the plain method, the relaxation arms, the other
    large configuration and the certified cases on the same GPU."""
    import torch
    from gpuboscia_gb300 import _abi as A

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    w = WORKLOADS[args.workload]
    order, B, I = w["order"], args.nodes, args.iters
    n = order * order
    inst = make_instance(args.workload)
    t0 = time.perf_counter()
    sc = _trained_scorer()
    train_s = time.perf_counter() - t0

    # ramp: the search grows 1, 8, 64, ... nodes per round until batches are full
    ramp, g = 0, 1
    while g < B:
        ramp += g
        g <<= BRANCH_K
    warm_rounds = max(args.warmup, 3)
    limit = ramp + (warm_rounds + args.steps + 1) * B
    # open nodes the pool must hold: each processed node opens 2^k children
    capacity = limit * (1 << BRANCH_K) + 2 * B + 1

    # the full stack once for module loading and graph capture (untimed)
    _solve_timed(inst, A.PRECISION_MIXED, sc, B, 1, math.inf, 1, 1, I, node_limit=1)
    with ClockSampler(torch.cuda.current_device(), period_ms=200) as clk:
        torch.cuda.synchronize()
        wall, r, cert = _solve_timed(inst, A.PRECISION_MIXED, sc, B, 1, math.inf, 1, 1, I, node_limit=limit,
                                     trace=4096, capacity=capacity)
        torch.cuda.synchronize()
    ms, nodes = r.round_ms.astype(np.float64), r.round_nodes.astype(np.int64)
    full = np.nonzero(nodes == B)[0]
    timed = full[-args.steps:] if len(full) >= args.steps else full
    if len(timed) == 0:
        raise RuntimeError("the search ended before a full batch")
    first_timed = int(timed[0])
    t_local = torch.tensor([float(ms[timed].sum())], dtype=torch.float64, device="cuda")
    n_local = float(nodes[timed].sum())
    if world > 1:
        torch.distributed.all_reduce(t_local, op=torch.distributed.ReduceOp.MAX)
    total_ms = float(t_local.item())
    value = n_local * world / (total_ms / 1000.0)
    main = _solve_summary(wall, r, cert)
    main.update(rounds=len(ms), warmup_rounds=first_timed, timed_rounds=len(timed),
                round_ms_mean=float(ms[timed].mean()))

    # whole calls with the same node budget: the plain method (the reference's
    # configuration: FP64, host frontier, most fractional, no cutoff, no tuner)
    # against the full stack. The host frontier keeps every open node's bounds
    # in host memory (two FP64 vectors): the budget stays within a quarter of
    # the host's available memory
    small = ramp + B
    per_node = (1 << BRANCH_K) * 2 * n * 8
    avail = _host_available_bytes()
    if avail and small * per_node > avail // 4:
        small = max(ramp, int(avail // 4 // per_node))
    wall_f, r_f, c_f = _solve_timed(inst, A.PRECISION_MIXED, sc, B, 1, math.inf, 1, 1, I, node_limit=small,
                                    capacity=capacity)
    wall_p, r_p, c_p = _solve_timed(inst, A.PRECISION_FP64, None, B, 1, math.inf, 0, 0, I, node_limit=small,
                                    autotune=0)
    plain = _solve_summary(wall_p, r_p, c_p)
    full_small = _solve_summary(wall_f, r_f, c_f)

    # e2e: the main search's whole call through the Python API (instance from host arrays)
    h2d = 2 * n * 8 + 2 * n * 8 + len(inst.problem.int_vars) * 4    # A, B, root lb, ub, integer indices
    d2h = n * 8                                                       # the incumbent
    e2e_value = r.nodes_processed / wall

    other = {}
    if args.workload == "birkhoff_regular400" and args.other_limit > 0:
        # the order-120 pair (non-isomorphic 8-regular graphs), 256-node batches, a fixed time budget
        inst4 = make_instance("birkhoff_regular120")
        w4 = WORKLOADS["birkhoff_regular120"]
        o4 = {}
        for name, prec, scx, devf, cut in (("plain_fp64", A.PRECISION_FP64, None, 0, 0),
                                           ("full_stack", A.PRECISION_MIXED, sc, 1, 1)):
            wl, rr, cc = _solve_timed(inst4, prec, scx, w4["nodes"], 1, args.other_limit, devf, cut, w4["iters"],
                                      autotune=0)
            o4[name] = _solve_summary(wl, rr, cc)
        o4["full_vs_plain_nodes_per_s"] = o4["full_stack"]["nodes_per_s"] / max(o4["plain_fp64"]["nodes_per_s"], 1e-9)
        o4["note"] = (f"time budget {args.other_limit:g} s per arm, {w4['iters']} iterations per dispatch; "
                      "for two d-regular graphs the doubly stochastic J/n gives AX = XB, so every FW bound is 0 "
                      "while the optimum is positive: the gap cannot close by this method")
        other["birkhoff_regular120"] = o4
        # the box BQP (n = 64): time to a certified gap through gbx_solve, the reference's
        # configuration (host frontier, 64-node batches, one stream) against 1024-node
        # device-frontier rounds with the incumbent cutoff; FP64 both (bit-exact relaxations)
        from gpuboscia_gb300 import instances as I_
        ob = {}
        for name, batch, devf, cut in (("plain_fp64", 64, 0, 0), ("batched_fp64", 1024, 1, 1)):
            instb = I_.box_qp(n=64)
            wl, rr, cc = _solve_timed(instb, A.PRECISION_FP64, None, batch, 1, args.other_limit, devf, cut, 2000,
                                      autotune=0)
            ob[name] = _solve_summary(wl, rr, cc)
        ob["batched_vs_plain_seconds"] = ob["plain_fp64"]["seconds"] / max(ob["batched_fp64"]["seconds"], 1e-9)
        ob["note"] = "box BQP n = 64, whole tree to a certified 1e-6 gap, 2000 iterations per dispatch"
        other["box_qp64"] = ob
        # the cardinality portfolio (100 assets, 600 months): B&B nodes/s over a fixed time
        # budget, 64-node batches on one stream against four streams
        op = {}
        for name, streams in (("plain_fp64", 1), ("four_streams_fp64", 4)):
            instp = I_.portfolio()
            wl, rr, cc = _solve_timed(instp, A.PRECISION_FP64, None, 64, streams, args.other_limit / 2, 0, 0, 500,
                                      autotune=0)
            op[name] = _solve_summary(wl, rr, cc)
        op["four_streams_vs_plain_nodes_per_s"] = (op["four_streams_fp64"]["nodes_per_s"]
                                                   / max(op["plain_fp64"]["nodes_per_s"], 1e-9))
        op["note"] = (f"portfolio, 100 assets, cardinality 10, 64-node batches, time budget {args.other_limit / 2:g} s "
                      "per arm: one 64-node launch fills 64 of 152 SMs, several streams overlap batches")
        other["portfolio100"] = op

    _, lb_r, ub_r, eps_r = make_workload(args.workload, min(args.relax_nodes, B), rank)
    arms = relax_arms(inst, lb_r, ub_r, eps_r, w, I, check_nodes=args.check_nodes)
    if 128 < order <= 404 and args.cluster_arms:
        arms["cluster_vs_one_cta"] = cluster_arms(inst, w, lb_r, ub_r, eps_r, I)
    cases = certified_cases(sc, args.ttg_limit) if args.ttg_limit > 0 else None
    if rank != 0:
        return

    hbm_peak, bf16_peak, peak_kind = load_peaks()
    mx = arms["mixed"]
    # the relaxation kernel's algorithmic bytes: the iteration's m*m arrays
    # streamed once each -- FP32 iterate read, FP32 gradient written and read,
    # integer oracle costs written and read (20 m^2 bytes per node-iteration)
    per_it = 20.0 * order * order
    achieved = mx["node_iterations"] * per_it / (mx["ms"] / 1000.0) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak, "traffic": None, "peak_kind": peak_kind,
                "kernel": "relax_kernel<GRAPH_MATCHING,BIRKHOFF,mixed>",
                "work": f"{mx['node_iterations']} node-iterations x 20*{order}^2 bytes in "
                        f"{mx['ms']:.1f} ms ({mx['nodes']} nodes, one launch)",
                "note": "latency-bound: the two exact integer Hungarians per iteration are a dependent chain of "
                        "Dijkstra steps; the gradient runs in FP32 over the graphs' nonzero lists (no tensor "
                        "cores at this order)"}
    cpu_v, cores, done, dt = cpu_sample(inst, lb_r[:ref_sample_nodes(args)], ub_r[:ref_sample_nodes(args)],
                                        eps_r[:ref_sample_nodes(args)], w["alg"], w["ls"], I,
                                        budget_s=args.cpu_budget)
    ttg = {args.workload: {
        "plain_fp64": plain, "full_stack": full_small, "full_stack_long": main,
        "certified": bool(main["certified"] or full_small["certified"]),
        "note": ("the optimum is 0 and every FW bound is 0 (J/n is a fractional isomorphism of two regular "
                 "graphs), so the gap closes only when an LMO vertex is the isomorphism itself; at the root the "
                 "iterate's mass on it stays at 1/order, and only nodes whose fixings already name two correct "
                 "pairs reach it within a few hundred iterations")}}
    if cases:
        ttg.update(cases)
    line = {"metric": METRIC, "value": value, "unit": "nodes/s", "n_gpus": world, "steps": len(timed),
            "warmup": first_timed, "ms_per_step": total_ms / len(timed), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f64", "data": "synthetic",
            "config": config_dict(args),
            "e2e": {"value": e2e_value, "unit": "nodes/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "what": "whole gbx_solve call of the timed search (ramp rounds included) through the Python "
                            "API, instance uploaded from host arrays, incumbent read back"},
            "roofline": roofline,
            "cpu_baseline": {"value": cpu_v, "unit": "nodes/s", "cores": cores, "kind": "port",
                             "sample": f"{done} open nodes of the workload (uneven fixings), {I} iterations max "
                                       f"each, {dt:.1f} s"},
            "clocks": clk.summary(),
            # per round: select, gather, relax, learned branching, decide, expand, merge, status
            "gpu_launches": 8 * len(timed),
            "full_vs_plain_nodes_per_s": full_small["nodes_per_s"] / max(plain["nodes_per_s"], 1e-9),
            "plain_fp64": plain, "full_stack_same_budget": full_small, "search": main,
            "relax_arms": arms, "other_configs": other, "time_to_gap": ttg,
            "scorer_training_seconds": train_s}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- one relaxation launch (relax mode)
def time_plain(args, inst, lb, x0, d_lb, d_ub, d_eps, d_flags, flush, w, stream):
    """The plain method (FP64 gradient and Hungarian) on the same batch, for the ratio."""
    import torch
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api
    N = lb.shape[0]
    alg = A.Algorithm(w["alg"], w["ls"], 4, 1e-10, 1e-14, A.PRECISION_FP64)
    x = torch.empty_like(x0)
    it = torch.zeros(N, dtype=torch.int32, device=x0.device)
    st = torch.zeros(N, dtype=torch.uint8, device=x0.device)
    relaxer = api.BatchRelaxer(inst.objective, inst.lmo, alg, x, d_lb, d_ub, d_eps, it, st, args.iters, d_flags,
                               1e-6, stream)
    x.copy_(x0)
    relaxer.launch()
    times = []
    for k in range(args.plain_steps):
        flush.fill_(float(k))
        x.copy_(x0)
        it.zero_()
        st.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        relaxer.launch()
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    ms = sum(times) / len(times)
    return {"value": N / (ms / 1000.0), "unit": "nodes/s", "ms_per_step": ms, "steps": len(times),
            "node_iterations_per_step": int(it.sum().item())}


def run_relax(args, rank, world):
    """A step is one gbx_relax_batch launch over the workload's batch of open
    nodes, up to --iters iterations each; value = node relaxations per second."""
    import torch
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda")
    inst, lb, ub, eps = make_workload(args.workload, args.nodes, rank)
    w = WORKLOADS[args.workload]
    birkhoff = w["kind"] == "birkhoff"
    order = w.get("order", 0)
    N, n = lb.shape
    prec = A.PRECISION_MIXED if args.precision == "mixed" else A.PRECISION_FP64
    alg = A.Algorithm(w["alg"], w["ls"], 4, 1e-10, 1e-14, prec)
    T = lambda a, t=None: torch.from_numpy(np.ascontiguousarray(a if t is None else np.asarray(a, t))).to(dev)
    d_lb, d_ub, d_eps = T(lb), T(ub), T(eps)
    d_flags = T(workload_flags(args.workload, n), np.uint8)
    x0 = d_lb.clone()
    x = torch.empty_like(x0)
    it = torch.zeros(N, dtype=torch.int32, device=dev)
    st = torch.zeros(N, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    if args.launch_shape in ("tc", "simt"):
        api.set_launch_shape(inst.objective, inst.lmo, alg, n, 1 if args.launch_shape == "tc" else 0, 0)
    elif args.launch_shape == "cluster":
        api.set_launch_shape(inst.objective, inst.lmo, alg, n, -1, 2)
    elif args.launch_shape == "pair":
        api.set_launch_shape(inst.objective, inst.lmo, alg, n, -1, 3)
    if args.oracle_warps != -1:
        api.set_launch_shape(inst.objective, inst.lmo, alg, n, -1, 2 if args.launch_shape == "cluster" else 0,
                             oracle_warps=args.oracle_warps)
    relaxer = api.BatchRelaxer(inst.objective, inst.lmo, alg, x, d_lb, d_ub, d_eps, it, st, args.iters, d_flags,
                               1e-6, stream)
    if args.launch_shape == "tuned":
        x.copy_(x0)
        it.zero_()
        st.zero_()
        args.tuned_shape = relaxer.autotune()   # before the warm-up, on this batch
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        x.copy_(x0)
        it.zero_()
        st.zero_()
        relaxer.launch()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.fill_(float(k))
            x.copy_(x0)
            it.zero_()
            st.zero_()
            ev[k][0].record(stream)
            relaxer.launch()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    times = [a.elapsed_time(b) for a, b in ev]
    kernel_ms = sum(times) / len(times)
    node_iters = int(it.sum().item())
    statuses = st.cpu().numpy()
    t_local = torch.tensor([sum(times)], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(t_local, op=torch.distributed.ReduceOp.MAX)
    total_ms = float(t_local.item())
    value = N * args.steps * world / (total_ms / 1000.0)

    # e2e through the C ABI with pinned host buffers
    h = {k: v.pin_memory() for k, v in dict(x=torch.from_numpy(lb.copy()), lb=torch.from_numpy(lb),
                                                 ub=torch.from_numpy(ub), eps=torch.from_numpy(eps),
                                                 it=torch.zeros(N, dtype=torch.int32),
                                                 st=torch.zeros(N, dtype=torch.uint8)).items()}
    ho = {k: torch.empty(s, dtype=dt).pin_memory() for k, s, dt in
          (("x", (N, n), torch.float64), ("gap", (N,), torch.float64), ("value", (N,), torch.float64),
           ("bvv", (N,), torch.float64), ("bv", (N, n), torch.float64), ("it", (N,), torch.int32),
           ("st", (N,), torch.uint8))}
    h2d = sum(v.numel() * v.element_size() for v in h.values())
    d2h = sum(v.numel() * v.element_size() for v in ho.values())

    def e2e_step():
        x.copy_(h["x"], non_blocking=True)
        d_lb.copy_(h["lb"], non_blocking=True)
        d_ub.copy_(h["ub"], non_blocking=True)
        d_eps.copy_(h["eps"], non_blocking=True)
        it.copy_(h["it"], non_blocking=True)
        st.copy_(h["st"], non_blocking=True)
        relaxer.launch()
        ho["x"].copy_(x, non_blocking=True)
        ho["gap"].copy_(relaxer.gap, non_blocking=True)
        ho["value"].copy_(relaxer.value, non_blocking=True)
        ho["bvv"].copy_(relaxer.best_vertex_val, non_blocking=True)
        ho["bv"].copy_(relaxer.best_vertex, non_blocking=True)
        ho["it"].copy_(it, non_blocking=True)
        ho["st"].copy_(st, non_blocking=True)
        stream.synchronize()

    e2e_step()
    e2e_times = []
    for k in range(args.steps):
        flush.fill_(float(k))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_times.append(time.perf_counter() - t0)
    e2e_local = torch.tensor([sum(e2e_times)], dtype=torch.float64, device=dev)
    if world > 1:
        torch.distributed.all_reduce(e2e_local, op=torch.distributed.ReduceOp.MAX)
    e2e_value = N * args.steps * world / float(e2e_local.item())

    plain = None
    if args.plain_steps > 0 and prec != A.PRECISION_FP64 and birkhoff:
        plain = time_plain(args, inst, lb, x0, d_lb, d_ub, d_eps, d_flags, flush, w, stream)
    if rank != 0:
        return
    hbm_peak, bf16_peak, peak_kind = load_peaks()
    grads = node_iters + N  # iterations plus the final certificate gradient of each node
    if birkhoff and prec == A.PRECISION_MIXED and order > 64:
        # the mixed gradient runs on the tensor cores (orders 65..128 by default)
        flops = grads * 8.0 * order ** 3
        achieved_tf = flops / (kernel_ms / 1000.0) / 1e12
        roofline = {"bound": "tensor", "achieved": achieved_tf, "peak": bf16_peak, "unit": "TFLOP/s",
                    "frac": achieved_tf / bf16_peak, "traffic": None, "peak_kind": peak_kind,
                    "kernel": "relax_kernel<GRAPH_MATCHING,BIRKHOFF,mixed>",
                    "work": f"{grads} gradients x 8*{order}^3 flop per launch"}
    elif birkhoff:
        # FP32 SIMT or FP64 gradient: the iteration's m*m arrays streamed once each
        per_it = 20.0 * order * order
        achieved = node_iters * per_it / (kernel_ms / 1000.0) / 1e9
        roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved / hbm_peak, "traffic": None, "peak_kind": peak_kind,
                    "kernel": "relax_kernel<GRAPH_MATCHING,BIRKHOFF,%s>" % args.precision,
                    "work": f"{node_iters} node-iterations x 20*{order}^2 bytes per launch"}
    else:
        # the box / simplex LMO phase: g, lb, ub in and v out, 32 bytes per variable per call
        lmo_bytes = grads * 32.0 * n
        achieved_gbs = lmo_bytes / (kernel_ms / 1000.0) / 1e9
        roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                    "frac": achieved_gbs / hbm_peak, "traffic": None, "peak_kind": peak_kind,
                    "kernel": "relax_kernel<DENSE_QUADRATIC,%s>" % ("BOX" if w["kind"] == "box" else "CARDINALITY"),
                    "work": f"{grads} LMO calls x 32*{n} bytes per launch"}
    cpu_v, cores, done, dt = cpu_sample(inst, lb, ub, eps, w["alg"], w["ls"], args.iters, budget_s=args.cpu_budget,
                                        flags=workload_flags(args.workload, n))
    line = {"metric": METRIC, "value": value, "unit": "nodes/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if prec == A.PRECISION_FP64 else "bf16+f64",
            "data": "synthetic", "config": config_dict(args),
            "e2e": {"value": e2e_value, "unit": "nodes/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roofline,
            "cpu_baseline": {"value": cpu_v, "unit": "nodes/s", "cores": cores, "kind": "port",
                             "sample": f"{done} of {N} nodes of the same batch, {args.iters} iterations max, "
                                       f"{dt:.1f} s"},
            # relax_kernel, plus sparse_build_kernel for graph matching
            "clocks": clk.summary(), "gpu_launches": (2 if birkhoff else 1) * args.steps,
            "node_iterations_per_step": node_iters,
            "plain_fp64": plain,
            "status_counts": {str(s): int((statuses == s).sum()) for s in np.unique(statuses)}}
    print(json.dumps(line), flush=True)


def run_gradient(args):
    """--mode gradient: the batched graph-matching gradient entry points alone
    (for profiling), on a G(order, 1/2) pair and --cases random points:
    --gradient f32 times gbx_objective_gradient_batch_f32 (the pipelined
    tensor-core kernel), mixed times gbx_objective_gradient_batch with FP64
    points in mixed precision. One JSON line (not the benchmark's line)."""
    import torch
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api, instances
    m, N = args.order, args.cases
    inst = instances.birkhoff_gnp(order=m, seed=5)
    rng = np.random.Generator(np.random.PCG64(9))
    x = torch.from_numpy(rng.random((N, m * m))).cuda()
    xf = x.float()
    call = ((lambda: api.objective_gradient_batch_f32(inst.objective, xf)) if args.gradient == "f32"
            else (lambda: api.objective_gradient_batch(inst.objective, x, A.PRECISION_MIXED)))
    for _ in range(args.warmup):
        call()
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        call()
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    t = statistics.mean(ms)
    print(json.dumps({"mode": "gradient", "entry": args.gradient, "order": m, "cases": N, "ms": t,
                      "tflops_algorithmic": N * 8.0 * m ** 3 / (t / 1000.0) / 1e12}), flush=True)


def run_lmo(args):
    """--mode lmo: the batched box LMO (gbx_lmo_batch) alone, for profiling
    its HBM stream: --cases rows of --lmo-n variables, --lmo-mode 0 (forward:
    direction, lb, ub in, the vertex out, 32 bytes per variable) or 1 (in-face:
    x in as well, 40 bytes). Every array is larger than L2 at the default
    sizes (4096 x 8192 doubles = 268 MB), so no flush is needed between calls.
    One JSON line (not the benchmark's line) with the algorithmic GB/s against
    the measured copy bandwidth; the result is checked against the same
    formula in numpy on a sample of rows. The timed region is one call of the
    Python API: the output's allocation and zero fill (8 more bytes per
    variable), the kernel, and the call's stream synchronisation; the
    kernel's own duration is what ncu reports for box_lmo_stream_kernel."""
    import torch
    from gpuboscia_gb300 import api
    N, n, mode = args.cases, args.lmo_n, args.lmo_mode
    rng = np.random.Generator(np.random.PCG64(13))
    d = torch.from_numpy(rng.standard_normal((N, n))).cuda()
    lb = torch.from_numpy(rng.integers(-1, 1, (N, n)).astype(np.float64)).cuda()
    ub = lb + 1.0
    x = (lb + torch.from_numpy(rng.random((N, n))).cuda().round()) if mode == 1 else None
    lmo = api.BoxLMO()
    call = lambda: api.lmo_batch(lmo, mode, d, lb, ub, x=x)
    for _ in range(max(args.warmup, 3)):
        out, _ = call()
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        out, _ = call()
        b.record()
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    rows = slice(0, min(N, 64))
    want = np.where(d[rows].cpu().numpy() > 0.0, lb[rows].cpu().numpy(), ub[rows].cpu().numpy())
    if mode == 1:   # x sits on a bound everywhere here: the in-face vertex keeps it
        want = x[rows].cpu().numpy()
    ok = bool(np.array_equal(out[rows].cpu().numpy(), want))
    t = statistics.mean(ms)
    per = 40 if mode == 1 else 32
    gbs = N * n * per / (t / 1000.0) / 1e9
    hbm, _, kind = load_peaks()
    print(json.dumps({"mode": "lmo", "lmo": "box", "lmo_mode": mode, "cases": N, "n": n, "ms": t,
                      "bytes_per_variable": per, "gbs_algorithmic": gbs, "hbm_peak_gbs": hbm,
                      "peak_kind": kind, "frac": gbs / hbm, "sample_rows_equal": ok,
                      "l2": "every array larger than L2 (no flush)"}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--nodes", type=int, default=None)
    ap.add_argument("--iters", type=int, default=None)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--plain-steps", type=int, default=2,
                    help="relax mode: timed steps of the plain FP64 method on the same batch (0 skips it)")
    ap.add_argument("--ttg-limit", type=float, default=30.0,
                    help="bnb mode: time limit of each certified time-to-gap solve in seconds (0 skips them)")
    ap.add_argument("--other-limit", type=float, default=10.0,
                    help="bnb mode: time budget of each order-120 search arm in seconds (0 skips them)")
    ap.add_argument("--relax-nodes", type=int, default=152,
                    help="bnb mode: open nodes of the relaxation-arm comparison (one wave of 152 SMs)")
    ap.add_argument("--cluster-arms", type=int, default=1,
                    help="bnb mode, orders 129..404: time the cluster shape against one CTA per node (0 skips)")
    ap.add_argument("--check-nodes", type=int, default=4,
                    help="bnb mode: nodes whose mixed certificate the oracle re-evaluates")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--ref-budget", type=float, default=8.0)
    ap.add_argument("--launch-shape", default="auto", choices=["auto", "tc", "simt", "tuned", "cluster", "pair"],
                    help="relax mode, mixed Birkhoff: the default rule, tensor-core gradient, FP32 SIMT "
                         "gradient (over the nonzero lists for sparse graphs above order 64), the "
                         "autotuner's choice on the batch (gbx_relax_autotune), a cluster of four CTAs "
                         "per node (orders 129..404), or a pair of CTAs per node (FP64 dense quadratic)")
    ap.add_argument("--oracle-warps", type=int, default=-1, choices=[-1, 1, 4],
                    help="relax mode, mixed Birkhoff orders 129..512: warps per integer oracle (-1 default: 4)")
    ap.add_argument("--solve", default=None, choices=sorted(PAIR_CONFIGS),
                    help="only solve the held-out graph pairs with this time-to-gap configuration "
                         "(one JSON line; for profiling the search)")
    ap.add_argument("--mode", default=None, choices=["bnb", "relax", "gradient", "lmo"],
                    help="override the workload's measurement (relax: one relaxation launch per step; "
                         "gradient: the batched gradient entry points alone; lmo: the batched box LMO "
                         "alone; both for profiling)")
    ap.add_argument("--order", type=int, default=128, help="gradient mode: graph order")
    ap.add_argument("--cases", type=int, default=4096, help="gradient mode: points per call")
    ap.add_argument("--gradient", default="f32", choices=["f32", "mixed"], help="gradient mode: entry point")
    ap.add_argument("--lmo-n", type=int, default=8192, help="lmo mode: variables per row")
    ap.add_argument("--lmo-mode", type=int, default=0, choices=[0, 1], help="lmo mode: forward (0) or in-face (1)")
    args = ap.parse_args()
    if args.mode in ("gradient", "lmo"):
        from gpuboscia_gb300 import build
        build.build()
        if args.mode == "lmo":
            run_lmo(args)
        else:
            run_gradient(args)
        return
    if args.solve:
        from gpuboscia_gb300 import build
        build.build()
        sc = _trained_scorer() if PAIR_CONFIGS[args.solve][1] else None
        # warm-up: module loading and the first-batch launch-shape tuning stay out of the timed solves
        prec, use, batch, streams, dev, cut = PAIR_CONFIGS[args.solve]
        _solve_timed(_pair(300, 6), prec, sc if use else None, batch, streams, 10.0, dev, cut)
        print(json.dumps({"solve": args.solve, **_solve_pairs(args.solve, sc, args.ttg_limit or 60.0)}))
        return
    w = WORKLOADS[args.workload]
    mode = args.mode or w["mode"]
    if w["kind"] != "birkhoff":
        args.precision = "fp64"   # mixed precision covers graph matching over Birkhoff only
        mode = "relax"
    args.nodes = args.nodes or w["nodes"]
    args.iters = args.iters or w["iters"]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "gb300":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        from gpuboscia_gb300 import build
        if rank == 0:
            build.build()
        if world > 1:
            import torch
            torch.distributed.barrier()
        if mode == "bnb":
            run_bnb(args, rank, world)
        else:
            run_relax(args, rank, world)
    if world > 1 and args.impl == "gb300":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
