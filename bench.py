#!/usr/bin/env python
"""Benchmark of the node-relaxation hot path on GB300.

A step is one batched relaxation launch: every open B&B node of a synthetic
batch (uneven fixings, depth-dependent FW tolerances) is relaxed by FW/DICG
for up to --iters iterations. value = node relaxations per second with the
batch resident in HBM; e2e = the same through the C ABI with the node data
in pinned host memory (H2D and D2H inside the timed region).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
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
    # name: instance family and size, nodes per batch, algorithm, line search, iterations per launch
    "birkhoff_gnp36": dict(kind="birkhoff", order=36, nodes=256, alg=1, ls=4, iters=100),
    "birkhoff_regular120": dict(kind="birkhoff", order=120, nodes=256, alg=1, ls=4, iters=20),
    # isomorphic 10-regular pair on 400 vertices (B = P A P'); mixed precision keeps the oracle costs in the
    # workspace and runs the FP32 gradient over the nonzero lists at this order
    "birkhoff_regular400": dict(kind="birkhoff", order=400, nodes=152, alg=1, ls=4, iters=5),
    # the 64-variable box BQP (1024-node batches) and the 100-asset cardinality portfolio
    # (64 nodes per launch): Frank-Wolfe, FP64
    "box_qp64": dict(kind="box", n=64, nodes=1024, alg=0, ls=4, iters=200),
    "portfolio100": dict(kind="portfolio", n=200, nodes=64, alg=0, ls=4, iters=500),
}


# dram__bytes_read.sum + dram__bytes_write.sum of the relaxation kernel per node,
# from the committed ncu captures (profiles/: 256 nodes at order 36, 152 nodes at
# order 120); independent of the iteration count, scaled by the nodes of a launch
TRAFFIC_PER_NODE = {("birkhoff_gnp36", "mixed"): 8247552 / 256,
                    ("birkhoff_regular120", "mixed"): (139682816 + 191056640) / 152}


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


def make_workload(name, nodes, rank):
    from gpuboscia_gb300 import instances
    w = WORKLOADS[name]
    if w["kind"] == "box":
        inst = instances.box_qp(n=w["n"])
        lb, ub = instances.box_node_batch(w["n"], nodes, seed=4242 + rank)
    elif w["kind"] == "portfolio":
        inst = instances.portfolio(assets=w["n"] // 2)
        lb, ub = instances.portfolio_node_batch(w["n"] // 2, 10, nodes, seed=4242 + rank)
    else:
        order = w["order"]
        if name.startswith("birkhoff_gnp"):
            inst = instances.birkhoff_gnp(order=order)
        elif order == 400:
            inst = instances.birkhoff_regular_isomorphic(order=order)
        else:
            inst = instances.birkhoff_regular_perturbed(order=order)
        lb, ub = instances.birkhoff_node_batch(order, nodes, seed=4242 + rank)
    rng = np.random.Generator(np.random.PCG64(77 + rank))
    depth = rng.integers(0, 13, nodes)
    eps = np.maximum(1e-6, 1e-3 * 0.8 ** depth)
    return inst, lb, ub, eps


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        import select
        self.first = ""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
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


def run_reference(args, rank, world):
    """--impl reference: the oracle port of the reference's relaxation on the host cores."""
    if rank != 0:
        return
    inst, lb, ub, eps = make_workload(args.workload, args.nodes, 0)
    w = WORKLOADS[args.workload]
    for _ in range(args.warmup):
        cpu_sample(inst, lb, ub, eps, w["alg"], w["ls"], args.iters, budget_s=0.0,
                   flags=workload_flags(args.workload, lb.shape[1]))
    vals, times = [], []
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
                             "sample": f"{done} of {args.nodes} nodes per step, {args.iters} iterations max"},
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
              "precision": args.precision, "l2": "flushed between timed steps (256 MiB write)"})
    if getattr(args, "launch_shape", "auto") != "auto":
        d["launch_shape"] = args.launch_shape
        if getattr(args, "tuned_shape", None):
            d["tuned_shape"] = {"tensor_core": args.tuned_shape[0], "persistent": args.tuned_shape[1]}
    return d


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


def _solve_timed(inst, prec, scorer_obj, batch, streams, limit, device_frontier=0, cutoff=0):
    from gpuboscia_gb300 import _abi as A
    from gpuboscia_gb300 import api
    s = inst.settings
    s.gpu_batch_size = batch
    s.num_streams = streams
    s.gpu_max_iters = 500   # the reference's graph-matching example (examples/main.cu:218)
    s.line_search = A.LS_QUADRATIC_EXACT
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.time_limit_seconds = limit
    s.precision = prec
    s.scorer = scorer_obj
    s.device_frontier = device_frontier
    s.incumbent_cutoff = cutoff
    t0 = time.perf_counter()
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    wall = time.perf_counter() - t0
    gap = abs(r.objective - r.dual_bound) if math.isfinite(r.objective) else math.inf
    certified = bool(not r.reached_time_limit and (gap <= 1e-6 or gap <= 1e-6 * abs(r.objective)))
    return wall, r, certified


def time_to_gap(args, inst):
    """Wall time of gpuboscia::solve (through gbx_solve) from entry to the certified
    1e-6 gap. (1) The workload's instance, plain FP64 against mixed precision.
    (2) Held-out G(9, 1/2) graph pairs (non-isomorphic, the tree branches):
    plain (FP64 gradients, most-fractional branching) against mixed precision
    and mixed precision + the learned scorer (trained first on strong-branching
    labels of four other pairs); same engine settings for all."""
    from gpuboscia_gb300 import _abi as A
    out = {}
    for name, prec in (("plain_fp64", A.PRECISION_FP64), ("mixed", A.PRECISION_MIXED)):
        wall, r, cert = _solve_timed(inst, prec, None, 256, 2, args.ttg_limit)
        out[name] = {"seconds": wall, "nodes": r.nodes_processed, "objective": r.objective,
                     "dual_bound": r.dual_bound, "certified": cert, "time_limit": bool(r.reached_time_limit)}

    t0 = time.perf_counter()
    sc = _trained_scorer()
    train_s = time.perf_counter() - t0
    pairs = {"instances": "4 held-out G(9,1/2) pairs; batch 64 x 1 stream, host frontier, unless named; "
                          "full_stack = mixed + learned + device frontier (1024-node rounds) + incumbent cutoff",
             "scorer_training_seconds": train_s}
    for name in PAIR_CONFIGS:
        pairs[name] = _solve_pairs(name, sc, args.ttg_limit)
    out["graph_pairs"] = pairs
    return out


def _pair(seed, order=9):
    from gpuboscia_gb300 import instances
    rng = np.random.Generator(np.random.PCG64(seed))
    return instances.graph_matching(order, instances.gnp_graph(rng, order, 0.5),
                                    instances.gnp_graph(rng, order, 0.5), f"pair{order}_{seed}")


def _trained_scorer():
    """The learned scorer: strong-branching labels of four G(9, 1/2) pairs (seeds
    100-103, disjoint from the held-out pairs 200-203), 400 Adam epochs."""
    from gpuboscia_gb300 import scorer
    data = scorer.Dataset.concat([scorer.collect_strong_branching(_pair(100 + k), max_nodes=30, max_candidates=64)
                                  for k in range(4)])
    sc = scorer.Scorer(32, seed=0)
    sc.train(data, epochs=400, lr=3e-3)
    return sc


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


def run_gpu(args, rank, world):
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
    ttg = time_to_gap(args, inst) if rank == 0 and args.ttg_limit > 0 and birkhoff else None
    if rank != 0:
        return
    hbm_peak, bf16_peak, peak_kind = load_peaks()
    grads = node_iters + N  # iterations plus the final certificate gradient of each node
    if birkhoff:
        flops = grads * 8.0 * order ** 3
        achieved_tf = flops / (kernel_ms / 1000.0) / 1e12
        roofline = {"bound": "tensor", "achieved": achieved_tf, "peak": bf16_peak, "unit": "TFLOP/s",
                    "frac": achieved_tf / bf16_peak,
                    "traffic": (TRAFFIC_PER_NODE[(args.workload, args.precision)] * N
                                if (args.workload, args.precision) in TRAFFIC_PER_NODE else None),
                    "peak_kind": peak_kind,
                    "kernel": "relax_kernel<GRAPH_MATCHING,BIRKHOFF>",
                    "work": f"{grads} gradients x 8*{order}^3 flop per launch"}
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
            "plain_fp64": plain, "time_to_gap": ttg,
            "status_counts": {str(s): int((statuses == s).sum()) for s in np.unique(statuses)}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="birkhoff_gnp36", choices=sorted(WORKLOADS))
    ap.add_argument("--nodes", type=int, default=None)
    ap.add_argument("--iters", type=int, default=None)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--plain-steps", type=int, default=2,
                    help="timed steps of the plain FP64 method on the same batch (0 skips it)")
    ap.add_argument("--ttg-limit", type=float, default=30.0,
                    help="time limit of each time-to-gap solve in seconds (0 skips them)")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--ref-budget", type=float, default=8.0)
    ap.add_argument("--launch-shape", default="auto", choices=["auto", "tc", "simt", "tuned"],
                    help="mixed Birkhoff gradient: the default rule, tensor cores, FP32 SIMT "
                         "(over the nonzero lists for sparse graphs above order 64), or the "
                         "autotuner's choice on the batch (gbx_relax_autotune)")
    ap.add_argument("--solve", default=None, choices=sorted(PAIR_CONFIGS),
                    help="only solve the held-out graph pairs with this time-to-gap configuration "
                         "(one JSON line; for profiling the search)")
    args = ap.parse_args()
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
    if w["kind"] != "birkhoff":
        args.precision = "fp64"   # mixed precision covers graph matching over Birkhoff only
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
        run_gpu(args, rank, world)
    if world > 1 and args.impl == "gb300":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
