"""Python mirror of the reference's public API over the C ABI.

Objectives and LMOs keep their data as float64 numpy arrays and produce the C
descriptors of include/gpuboscia_gb300.h either over host arrays (``where="host"``)
or over device copies (``where="cuda"``, torch tensors). ``solve`` runs the whole
branch and bound in the library (gbx_solve); ``relax_batch`` / ``lmo_batch`` /
``node_feasible_batch`` expose the batched GPU kernels over torch tensors.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import Optional, Sequence

import numpy as np

from . import _abi as A


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


class _Keep:
    """Holds the arrays a descriptor points at."""

    def __init__(self):
        self.items = []

    def ptr(self, arr, where: str):
        if arr is None:
            return None
        if where == "host":
            a = np.ascontiguousarray(arr)
            self.items.append(a)
            return a.ctypes.data
        import torch
        if isinstance(arr, torch.Tensor):
            t = arr.contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(arr)).to("cuda")
        self.items.append(t)
        return t.data_ptr()


# ---------------------------------------------------------------- objectives
@dataclasses.dataclass
class DenseQuadraticObjective:
    """f(x) = 0.5*s*x'Qx + s*l*c'x + k (GlobalCachedDenseQuadraticObjective,
    dense_quadratic_objectives.cuh:18-112). ``Q`` is given in the usual
    orientation; it is stored transposed for the kernel (a symmetric Q is
    unchanged)."""
    Q: np.ndarray
    c: Optional[np.ndarray] = None
    scale: float = 1.0
    linear_scale: float = 1.0
    constant: float = 0.0

    @property
    def n(self) -> int:
        return int(np.asarray(self.Q).shape[0])

    def to_c(self, where: str, keep: _Keep) -> A.Objective:
        Q = _f64(self.Q)
        o = A.Objective()
        o.kind = A.OBJ_DENSE_QUADRATIC
        o.n = Q.shape[0]
        o.Q = keep.ptr(_f64(Q.T), where)
        o.c = keep.ptr(_f64(self.c) if self.c is not None else None, where)
        o.scale, o.linear_scale, o.constant = self.scale, self.linear_scale, self.constant
        return o


def ILSObjective(AtA, Atb, btb: float) -> DenseQuadraticObjective:
    """||Ax - b||^2 from A'A, A'b, b'b (ILSGlobalCachedObjective, dense_quadratic_objectives.cuh:114-124)."""
    return DenseQuadraticObjective(AtA, Atb, 2.0, -1.0, btb)


@dataclasses.dataclass
class GraphMatchingObjective:
    """f(X) = scale*||A X - X B||_F^2 over order x order X (row-major)."""
    A: np.ndarray
    B: np.ndarray
    scale: float = 1.0

    @property
    def order(self) -> int:
        return int(np.asarray(self.A).shape[0])

    @property
    def n(self) -> int:
        return self.order ** 2

    def to_c(self, where: str, keep: _Keep) -> A.Objective:
        o = A.Objective()
        o.kind = A.OBJ_GRAPH_MATCHING
        o.order = self.order
        o.n = self.n
        o.A = keep.ptr(_f64(self.A), where)
        o.B = keep.ptr(_f64(self.B), where)
        o.scale = self.scale
        o.linear_scale = 1.0
        return o


# ---------------------------------------------------------------- LMOs
@dataclasses.dataclass
class BoxLMO:
    supports_dicg = True

    def to_c(self, n: int, where: str, keep: _Keep) -> A.LMO:
        return A.LMO(A.LMO_BOX, n, 1.0, None, 0)

    def relaxation_feasible(self, x, lb, ub, tol) -> bool:
        return True


@dataclasses.dataclass
class UnitSimplexLMO:
    right_side: float = 1.0
    int_vars: Sequence[int] = ()
    equality: bool = False
    supports_dicg = True

    def to_c(self, n: int, where: str, keep: _Keep) -> A.LMO:
        flags = np.zeros(n, dtype=np.uint8)
        for j in self.int_vars:
            if 0 <= j < n:
                flags[j] = 1
        kind = A.LMO_EQUALITY_SIMPLEX if self.equality else A.LMO_SIMPLEX
        return A.LMO(kind, n, float(self.right_side), keep.ptr(flags, where), 0)

    def relaxation_feasible(self, x, lb, ub, tol) -> bool:
        x = np.asarray(x, dtype=np.float64)
        if self.equality:
            return bool((x >= -tol).all() and math.isfinite(x.sum()) and abs(x.sum() - self.right_side) <= tol)
        return bool((x >= 0).all() and x.sum() <= self.right_side + tol)


def EqualitySimplexLMO(right_side=1.0, int_vars=()) -> UnitSimplexLMO:
    return UnitSimplexLMO(right_side, int_vars, True)


@dataclasses.dataclass
class BirkhoffLMO:
    order: int
    supports_dicg = True

    def to_c(self, n: int, where: str, keep: _Keep) -> A.LMO:
        return A.LMO(A.LMO_BIRKHOFF, n, 1.0, None, self.order)


@dataclasses.dataclass
class CardinalityLMO:
    """x = (w, z): sum w = 1, 0 <= w <= z, sum z <= cardinality, z in [0, 1]
    (GBX_LMO_CARDINALITY; Frank-Wolfe only)."""
    assets: int
    cardinality: int
    supports_dicg = False

    def to_c(self, n: int, where: str, keep: _Keep) -> A.LMO:
        assert n == 2 * self.assets
        return A.LMO(A.LMO_CARDINALITY, n, float(self.cardinality), None, 0)


@dataclasses.dataclass
class LinkedCardinalityLMO:
    """The sparse-Sharpe set {(v, y): 0 <= v_i <= upper_i y_i, sum y <= cardinality,
    y in [0, 1]} (GBX_LMO_LINKED_CARDINALITY, examples/sparse_sharpe.cu:266-546):
    v_i at i, y_i at n/2 + i for the len(upper) active assets, the rest of each
    half padding. Frank-Wolfe and DICG; branching fixes y."""
    upper: np.ndarray
    cardinality: int
    supports_dicg = True

    def to_c(self, n: int, where: str, keep: _Keep) -> A.LMO:
        U = _f64(self.upper)
        assert n % 2 == 0 and len(U) <= n // 2
        return A.LMO(A.LMO_LINKED_CARDINALITY, n, float(self.cardinality), None, len(U), keep.ptr(U, where))

    def relaxation_feasible(self, x, lb, ub, tol) -> bool:
        x = np.asarray(x, dtype=np.float64)
        h, k = len(x) // 2, len(self.upper)
        v, y = x[:k], x[h:h + k]
        return bool((v >= -tol).all() and (v <= np.asarray(self.upper) * y + tol).all()
                    and (y >= -tol).all() and (y <= 1 + tol).all() and y.sum() <= self.cardinality + tol)


# ---------------------------------------------------------------- problem / settings
@dataclasses.dataclass
class Problem:
    n_vars: int
    lb: np.ndarray
    ub: np.ndarray
    int_vars: Sequence[int] = ()


@dataclasses.dataclass
class Settings:
    """gpuboscia::Settings + DeviceResidentConfig (gpuboscia.cuh:21-32, device_resident_solver.cuh:1004-1025)."""
    gpu_batch_size: int = 1024
    num_streams: int = 8
    gpu_max_iters: int = 20000
    gpu_eps: float = 1e-3
    gpu_eps_decay: float = 0.8
    gpu_eps_min: float = 1e-6
    integer_tol: float = 1e-6
    abs_gap_tol: float = 1e-6
    rel_gap_tol: float = 1e-2
    algorithm: int = A.ALG_DICG
    line_search: int = A.LS_SECANT
    secant_iters: int = 4
    secant_tol: float = 1e-10
    secant_denom_eps: float = 1e-14
    precision: int = A.PRECISION_FP64
    time_limit_seconds: float = math.inf
    natural_lower_bound: float = -math.inf
    root_initial_point: Optional[np.ndarray] = None
    branch_k: int = 3
    use_cuda_graph: int = 1
    scorer: Optional[object] = None   # gpuboscia_gb300.scorer.Scorer: learned branching
    autotune: int = 1
    device_frontier: int = 0        # open nodes stay in HBM; each search round runs on the device
    incumbent_cutoff: int = 0       # stop node relaxations whose FW bound clears the incumbent
    frontier_capacity: int = 0      # pool size in nodes (0: automatic)
    frontier_slots: int = 2         # device frontier: batches in flight (1 or 2)
    node_limit: int = 0             # stop after this many processed nodes (0: none)
    round_trace: int = 0            # device frontier: record the timing of up to this many rounds

    def algorithm_c(self) -> A.Algorithm:
        return A.Algorithm(self.algorithm, self.line_search, self.secant_iters, self.secant_tol,
                           self.secant_denom_eps, self.precision)

    def to_c(self, keep: _Keep) -> A.Settings:
        s = A.Settings()
        for f in ("gpu_batch_size", "num_streams", "gpu_max_iters", "gpu_eps", "gpu_eps_decay", "gpu_eps_min",
                  "integer_tol", "abs_gap_tol", "rel_gap_tol", "time_limit_seconds", "natural_lower_bound",
                  "branch_k", "use_cuda_graph", "autotune", "device_frontier", "incumbent_cutoff",
                  "frontier_capacity", "frontier_slots", "node_limit"):
            setattr(s, f, getattr(self, f))
        s.algorithm = self.algorithm_c()
        s.root_initial_point = keep.ptr(_f64(self.root_initial_point) if self.root_initial_point is not None
                                        else None, "host")
        if self.scorer is not None:
            sc = self.scorer.to_c()
            keep.items.append(sc)
            s.scorer = C.addressof(sc)
        return s


@dataclasses.dataclass
class Result:
    objective: float
    x: np.ndarray
    dual_bound: float
    nodes_processed: int
    elapsed_seconds: float
    reached_tolerance: bool
    reached_time_limit: bool
    reached_node_limit: bool = False
    batches: int = 0                  # relaxation launches of the search
    round_ms: Optional[np.ndarray] = None     # device time of each round (Settings.round_trace)
    round_nodes: Optional[np.ndarray] = None  # nodes each round finished


def problem_to_c(p: Problem, keep: _Keep) -> A.Problem:
    iv = np.ascontiguousarray(np.asarray(list(p.int_vars), dtype=np.int32))
    return A.Problem(p.n_vars, keep.ptr(_f64(p.lb), "host"), keep.ptr(_f64(p.ub), "host"),
                     keep.ptr(iv, "host") if len(iv) else None, len(iv))


def check_problem(problem: Problem, settings: Settings) -> None:
    """The sizes the C ABI cannot see: gbx_solve reads n_vars doubles from lb,
    ub and the root point, and indexes with the integer variables."""
    n = problem.n_vars
    if not isinstance(n, (int, np.integer)) or n <= 0:
        raise ValueError(f"n_vars must be a positive integer, got {n!r}")
    for name, arr in (("lb", problem.lb), ("ub", problem.ub)):
        if np.asarray(arr).shape != (n,):
            raise ValueError(f"problem.{name} must have shape ({n},), got {np.asarray(arr).shape}")
    iv = np.asarray(list(problem.int_vars), dtype=np.int64)
    if iv.size and (iv.min() < 0 or iv.max() >= n):
        raise ValueError(f"integer variable index out of range [0, {n})")
    if settings.root_initial_point is not None and np.asarray(settings.root_initial_point).shape != (n,):
        raise ValueError(f"root_initial_point must have shape ({n},)")


def solve(problem: Problem, objective, lmo, settings: Optional[Settings] = None) -> Result:
    """gpuboscia::solve on the GPU (gbx_solve)."""
    settings = settings or Settings()
    check_problem(problem, settings)
    lib = A.load()
    keep = _Keep()
    n = problem.n_vars
    o = objective.to_c("cuda", keep)
    lm = lmo.to_c(n, "cuda", keep)
    s = settings.to_c(keep)
    pr = problem_to_c(problem, keep)
    x = np.zeros(n, dtype=np.float64)
    r = A.Result()
    r.x = x.ctypes.data
    tr = None
    if settings.round_trace > 0:
        cap = int(settings.round_trace)
        tms, tnodes = np.zeros(cap, np.float32), np.zeros(cap, np.int32)
        tr = A.RoundTrace(cap, 0, tms.ctypes.data, tnodes.ctypes.data)
        s.trace = C.addressof(tr)
    rc = lib.gbx_solve(C.byref(pr), C.byref(o), C.byref(lm), C.byref(s), C.byref(r))
    if rc == A.ERR_INVALID:
        raise ValueError(lib.gbx_last_error().decode())
    A.check(lib, rc, "gbx_solve")
    out = Result(r.objective, x if r.has_incumbent else np.zeros(0), r.dual_bound, r.nodes_processed,
                 r.elapsed_seconds, bool(r.reached_tolerance), bool(r.reached_time_limit),
                 bool(r.reached_node_limit), int(r.batches))
    if tr is not None:
        out.round_ms, out.round_nodes = tms[:tr.count].copy(), tnodes[:tr.count].copy()
    return out


# ---------------------------------------------------------------- batched kernels
class RelaxWorkspace:
    """Caller-owned device scratch for gbx_relax_batch (grows on demand)."""

    def __init__(self):
        self.buf = None

    def get(self, nbytes: int):
        import torch
        if self.buf is None or self.buf.numel() < nbytes:
            self.buf = torch.empty(max(nbytes, 256), dtype=torch.uint8, device="cuda")
        return self.buf


def _stream_ptr(stream) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


def _check_rows(lead, rows, dtype, extra=(), n_vars=None):
    """lead: the [cases, n] tensor that sets the shape; rows: (name, tensor or
    None) pairs that must hold cases*n elements of dtype; extra: (name,
    tensor, dtype, count) checked as given (count None: n elements, one per
    variable); n_vars: the objective's variable
    count, which n must equal (the kernels size vectors from the objective).
    All contiguous on lead's CUDA device. Returns (cases, n)."""
    import torch
    name0, t0 = lead
    if not isinstance(t0, torch.Tensor) or t0.dim() != 2:
        raise ValueError(f"{name0} must be a 2-D tensor [cases, n]")
    cases, n = t0.shape
    if n_vars is not None and n_vars != n:
        raise ValueError(f"the objective has {n_vars} variables, the rows of {name0} {n}")
    spec = [(name0, t0, dtype, cases * n)]
    spec += [(nm, t, dtype, cases * n) for nm, t in rows if t is not None]
    spec += [(nm, t, dt, n if count is None else count) for nm, t, dt, count in extra if t is not None]
    for name, t, dt, count in spec:
        if not isinstance(t, torch.Tensor):
            raise ValueError(f"{name} must be a torch tensor")
        if t.dtype != dt:
            raise ValueError(f"{name} must be {dt}, got {t.dtype}")
        if t.numel() != count:
            raise ValueError(f"{name} must hold {count} elements, got {t.numel()}")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
    for name, t, _, _ in spec:
        if not t.is_cuda or t.device != t0.device:
            raise ValueError(f"{name} must be on {name0}'s CUDA device ({t0.device}), got {t.device}")
    return cases, n


def check_node_tensors(x, lb, ub, eps, iterations, status, integer_flags=None, n_vars=None) -> tuple:
    """The node batch as gbx_relax_batch reads it (gbx_node_batch): x is
    [N, n] float64 and lb / ub hold N*n float64, eps N float64, iterations N
    int32, status N uint8, integer_flags n uint8 -- contiguous, on x's CUDA
    device, n equal to the objective's n_vars when given. A mismatch would
    make the kernel read or write outside a buffer, so it is refused here.
    Returns (N, n)."""
    import torch
    if not isinstance(x, torch.Tensor) or x.dim() != 2:
        raise ValueError("x must be a 2-D tensor [nodes, n_vars]")
    N, n = x.shape
    if n_vars is not None and n_vars != n:
        raise ValueError(f"the objective has {n_vars} variables, the node vectors {n}")
    spec = [("x", x, torch.float64, N * n), ("lb", lb, torch.float64, N * n), ("ub", ub, torch.float64, N * n),
            ("eps", eps, torch.float64, N), ("iterations", iterations, torch.int32, N),
            ("status", status, torch.uint8, N)]
    if integer_flags is not None:
        spec.append(("integer_flags", integer_flags, torch.uint8, n))
    for name, t, dtype, count in spec:
        if not isinstance(t, torch.Tensor):
            raise ValueError(f"{name} must be a torch tensor")
        if t.dtype != dtype:
            raise ValueError(f"{name} must be {dtype}, got {t.dtype}")
        if t.numel() != count:
            raise ValueError(f"{name} must hold {count} elements, got {t.numel()}")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
    for name, t, _, _ in spec:
        if not t.is_cuda or t.device != x.device:
            raise ValueError(f"{name} must be on x's CUDA device ({x.device}), got {t.device}")
    return N, n


def relax_batch(objective, lmo, algorithm: A.Algorithm, x, lb, ub, eps, iterations, status,
                max_iters: int, integer_flags=None, candidate_tol: float = 1e-6,
                workspace: Optional[RelaxWorkspace] = None, stream=None, keep: Optional[_Keep] = None,
                cutoff: Optional[float] = None):
    """Run gbx_relax_batch over device tensors (x, iterations, status updated in place).

    cutoff: incumbent value at which a node may stop iterating (gbx_node_batch.cutoff).
    Returns dict(gap, value, best_vertex, best_vertex_val) of new device tensors.
    """
    import torch
    N, n = check_node_tensors(x, lb, ub, eps, iterations, status, integer_flags, getattr(objective, "n", None))
    lib = A.load()
    keep = keep or _Keep()
    o = objective.to_c("cuda", keep)
    lm = lmo.to_c(n, "cuda", keep)
    dev = x.device
    out = dict(gap=torch.empty(N, dtype=torch.float64, device=dev),
               value=torch.empty(N, dtype=torch.float64, device=dev),
               best_vertex=torch.zeros(N, n, dtype=torch.float64, device=dev),
               best_vertex_val=torch.empty(N, dtype=torch.float64, device=dev))
    b = A.NodeBatch(N, max_iters, candidate_tol, x.data_ptr(), lb.data_ptr(), ub.data_ptr(), eps.data_ptr(),
                    iterations.data_ptr(), status.data_ptr(), out["gap"].data_ptr(), out["value"].data_ptr(),
                    out["best_vertex"].data_ptr(), out["best_vertex_val"].data_ptr(),
                    integer_flags.data_ptr() if integer_flags is not None else None)
    if cutoff is not None:
        cut = torch.full((1,), float(cutoff), dtype=torch.float64, device=dev)
        out["cutoff"] = cut   # returned with the outputs: alive while the launch runs
        b.cutoff = cut.data_ptr()
    need = lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(algorithm), N)
    if need == 0:
        A.check(lib, A.ERR_INVALID, "gbx_relax_workspace_bytes")
    ws = (workspace or RelaxWorkspace()).get(need)
    rc = lib.gbx_relax_batch(C.byref(o), C.byref(lm), C.byref(algorithm), C.byref(b), ws.data_ptr(), need,
                             _stream_ptr(stream))
    A.check(lib, rc, "gbx_relax_batch")
    out["_keep"] = (keep, ws)
    return out


def lmo_batch(lmo, mode: int, direction, lb, ub, x=None, want_step: bool = False, stream=None):
    """Batched forward (mode 0) or in-face (mode 1) oracle over device tensors [cases, n]."""
    import torch
    if mode == 1 and x is None:
        raise ValueError("the in-face oracle (mode 1) needs x")
    cases, n = _check_rows(("direction", direction), [("lb", lb), ("ub", ub), ("x", x)], torch.float64)
    lib = A.load()
    keep = _Keep()
    lm = lmo.to_c(n, "cuda", keep)
    out = torch.zeros(cases, n, dtype=torch.float64, device=direction.device)
    step = torch.zeros(cases, dtype=torch.float64, device=direction.device) if want_step else None
    rc = lib.gbx_lmo_batch(C.byref(lm), cases, mode, direction.data_ptr(), x.data_ptr() if x is not None else None,
                           lb.data_ptr(), ub.data_ptr(), out.data_ptr(), step.data_ptr() if step is not None else None,
                           _stream_ptr(stream))
    A.check(lib, rc, "gbx_lmo_batch")
    torch.cuda.current_stream().synchronize()
    return out, step


def set_launch_shape(objective, lmo, algorithm: A.Algorithm, n: int, tensor_core: int = -1, persistent: int = 0,
                     oracle_warps: int = -1, nodes_per_sm: int = -1):
    """gbx_relax_set_launch_shape: pin this problem shape's launch shape (tensor_core -1 default rule,
    0 FP32 SIMT gradient -- over the nonzero lists for sparse graphs above order 64 --, 1 tensor cores;
    persistent 0 one CTA per node, 1 persistent grid, 2 a cluster of four CTAs per node, 3 a pair of CTAs
    per node for the FP64 dense quadratic objective), then
    gbx_relax_set_oracle_warps (-1 default, 1 or 4 warps per integer oracle at orders 129..512) and
    gbx_relax_set_nodes_per_sm (-1 default, 1 or 2 nodes per SM for the FP64 kernels)."""
    lib = A.load()
    keep = _Keep()
    o = objective.to_c("cuda", keep)
    lm = lmo.to_c(n, "cuda", keep)
    rc = lib.gbx_relax_set_launch_shape(C.byref(o), C.byref(lm), C.byref(algorithm), tensor_core, persistent)
    if rc == A.ERR_INVALID:
        raise ValueError(lib.gbx_last_error().decode())
    A.check(lib, rc, "gbx_relax_set_launch_shape")
    if oracle_warps != -1:
        rc = lib.gbx_relax_set_oracle_warps(C.byref(o), C.byref(lm), C.byref(algorithm), oracle_warps)
        if rc == A.ERR_INVALID:
            raise ValueError(lib.gbx_last_error().decode())
        A.check(lib, rc, "gbx_relax_set_oracle_warps")
    if nodes_per_sm != -1:
        rc = lib.gbx_relax_set_nodes_per_sm(C.byref(o), C.byref(lm), C.byref(algorithm), nodes_per_sm)
        if rc == A.ERR_INVALID:
            raise ValueError(lib.gbx_last_error().decode())
        A.check(lib, rc, "gbx_relax_set_nodes_per_sm")


def objective_gradient_batch(objective, x, precision: int = A.PRECISION_FP64, stream=None):
    """Gradients of the objective at the rows of the device tensor x [cases, n]."""
    import torch
    cases, n = _check_rows(("x", x), [], torch.float64, n_vars=getattr(objective, "n", None))
    lib = A.load()
    keep = _Keep()
    o = objective.to_c("cuda", keep)
    g = torch.empty(cases, n, dtype=torch.float64, device=x.device)
    rc = lib.gbx_objective_gradient_batch(C.byref(o), precision, cases, x.data_ptr(), g.data_ptr(),
                                          _stream_ptr(stream))
    A.check(lib, rc, "gbx_objective_gradient_batch")
    torch.cuda.current_stream().synchronize()
    return g


def objective_gradient_batch_f32(objective, x, stream=None):
    """Pipelined tensor-core gradients of FP32 points x [cases, n] (orders <= 128)."""
    import torch
    if not isinstance(x, torch.Tensor):
        raise ValueError("x must be a 2-D tensor [cases, n]")
    lib = A.load()
    keep = _Keep()
    X = x.to(dtype=torch.float32).contiguous()
    cases, n = _check_rows(("x", X), [], torch.float32, n_vars=getattr(objective, "n", None))
    o = objective.to_c("cuda", keep)
    g = torch.empty(cases, n, dtype=torch.float32, device=X.device)
    rc = lib.gbx_objective_gradient_batch_f32(C.byref(o), cases, X.data_ptr(), g.data_ptr(), _stream_ptr(stream))
    A.check(lib, rc, "gbx_objective_gradient_batch_f32")
    return g


def node_feasible_batch(lmo, lb, ub, integer_flags=None, stream=None):
    import torch
    cases, n = _check_rows(("lb", lb), [("ub", ub)], torch.float64, [("integer_flags", integer_flags, torch.uint8, None)])
    lib = A.load()
    keep = _Keep()
    lm = lmo.to_c(n, "cuda", keep)
    out = torch.zeros(cases, dtype=torch.uint8, device=lb.device)
    rc = lib.gbx_node_feasible_batch(C.byref(lm), cases, lb.data_ptr(), ub.data_ptr(),
                                     integer_flags.data_ptr() if integer_flags is not None else None,
                                     out.data_ptr(), _stream_ptr(stream))
    A.check(lib, rc, "gbx_node_feasible_batch")
    torch.cuda.current_stream().synchronize()
    return out


class BatchRelaxer:
    """A fixed batch shape with descriptors, outputs and workspace built once;
    launch() is a single gbx_relax_batch call on the given stream."""

    def __init__(self, objective, lmo, algorithm: A.Algorithm, x, lb, ub, eps, iterations, status,
                 max_iters: int, integer_flags=None, candidate_tol: float = 1e-6, stream=None):
        import torch
        N, n = check_node_tensors(x, lb, ub, eps, iterations, status, integer_flags,
                                  getattr(objective, "n", None))
        self.lib = A.load()
        self.keep = _Keep()
        self.obj = objective.to_c("cuda", self.keep)
        self.lmo = lmo.to_c(n, "cuda", self.keep)
        self.alg = algorithm
        dev = x.device
        self.gap = torch.empty(N, dtype=torch.float64, device=dev)
        self.value = torch.empty(N, dtype=torch.float64, device=dev)
        self.best_vertex = torch.zeros(N, n, dtype=torch.float64, device=dev)
        self.best_vertex_val = torch.empty(N, dtype=torch.float64, device=dev)
        self.tensors = (x, lb, ub, eps, iterations, status, integer_flags)
        self.batch = A.NodeBatch(N, max_iters, candidate_tol, x.data_ptr(), lb.data_ptr(), ub.data_ptr(),
                                 eps.data_ptr(), iterations.data_ptr(), status.data_ptr(), self.gap.data_ptr(),
                                 self.value.data_ptr(), self.best_vertex.data_ptr(), self.best_vertex_val.data_ptr(),
                                 integer_flags.data_ptr() if integer_flags is not None else None)
        self.ws_bytes = self.lib.gbx_relax_workspace_bytes(C.byref(self.obj), C.byref(self.lmo), C.byref(self.alg), N)
        if self.ws_bytes == 0:
            A.check(self.lib, A.ERR_INVALID, "gbx_relax_workspace_bytes")
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.stream = _stream_ptr(stream)
        self._args = (C.byref(self.obj), C.byref(self.lmo), C.byref(self.alg), C.byref(self.batch),
                      C.c_void_p(self.ws.data_ptr()), C.c_size_t(self.ws_bytes), C.c_void_p(self.stream))

    def launch(self) -> None:
        rc = self.lib.gbx_relax_batch(*self._args)
        if rc != A.OK:
            A.check(self.lib, rc, "gbx_relax_batch")

    def autotune(self, repeats: int = 2):
        """gbx_relax_autotune on this batch (inputs restored): keeps the fastest launch
        shape for the problem shape; returns (tensor-core gradient, persistent grid)."""
        chosen = (C.c_int * 2)()
        rc = self.lib.gbx_relax_autotune(*self._args, repeats, C.cast(chosen, C.c_void_p))
        A.check(self.lib, rc, "gbx_relax_autotune")
        return int(chosen[0]), int(chosen[1])
