"""Learned branching scorer: strong-branching labels from the solver's own
relaxations, training and inference on the GPU by the library's kernels.

The scorer is an MLP of GBX_SCORER_FEATURES features (``gbx_branch_features``)
-> H -> H -> 1. It only decides which fractional variables branch_pow2 splits
on; most-fractional branching stays the fallback and the FW dual bound alone
decides pruning and optimality (``Settings.scorer``).

Labels: for a node with relaxation x (and certified bound L), each candidate
variable j gets the two children x_j <= floor(x_j) and x_j >= ceil(x_j),
relaxed in one ``gbx_relax_batch`` call with the node's own settings; with
child bounds L0, L1 (+inf when infeasible) the strong-branching score is the
product rule max(L0 - L, e) * max(L1 - L, e). Training minimises the listwise
cross-entropy between softmax(scores of the node's candidates) and the
sharpened strong-branching distribution score^(1/tau) / sum (tau = 1/2)
(``gbx_scorer_gradient``), with Adam (``gbx_scorer_adam``).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import math
from typing import List, Optional

import numpy as np

from . import _abi as A
from . import api

F = A.SCORER_FEATURES


def _stream(stream=None):
    import torch
    return (stream or torch.cuda.current_stream()).cuda_stream


class Scorer:
    """Device parameters (FP32 master copy and BF16 inference copy) of the MLP."""

    def __init__(self, hidden: int = 32, seed: int = 0, params: Optional[np.ndarray] = None):
        import torch
        self.hidden = hidden
        lib = A.load()
        self.count = lib.gbx_scorer_param_count(F, hidden)
        if params is None:
            params = self.init_params(hidden, seed)
        assert params.shape == (self.count,)
        self.params = torch.from_numpy(np.asarray(params, np.float32).copy()).cuda()
        self.params_bf16 = self.params.to(torch.bfloat16)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0

    @staticmethod
    def init_params(hidden: int, seed: int) -> np.ndarray:
        """He-uniform weights, zero biases (layout W1, b1, W2, b2, w3, b3)."""
        rng = np.random.Generator(np.random.PCG64(seed))
        H = hidden
        w1 = rng.uniform(-1, 1, (H, F)) * math.sqrt(6.0 / F)
        w2 = rng.uniform(-1, 1, (H, H)) * math.sqrt(6.0 / H)
        w3 = rng.uniform(-1, 1, H) * math.sqrt(6.0 / H)
        return np.concatenate([w1.ravel(), np.zeros(H), w2.ravel(), np.zeros(H), w3, np.zeros(1)]).astype(np.float32)

    def to_c(self) -> A.Scorer:
        return A.Scorer(F, self.hidden, self.params.data_ptr(), self.params_bf16.data_ptr())

    def numpy(self) -> np.ndarray:
        return self.params.cpu().numpy()

    def forward(self, features, bf16: bool = False, stream=None):
        """Scores of device (or numpy) features [rows, F]; returns a device tensor."""
        import torch
        _check_features(features)
        dev = self.params.device
        X = _dev_f32(features, dev)
        out = torch.empty(X.shape[0], dtype=torch.float32, device=dev)
        sc = self.to_c()
        lib = A.load()
        A.check(lib, lib.gbx_scorer_forward(C.byref(sc), X.shape[0], X.data_ptr(), out.data_ptr(), int(bf16),
                                            _stream(stream)), "gbx_scorer_forward")
        return out

    def gradient(self, features, group_ptr, target, stream=None):
        """(dL/dparams, L) of the listwise loss; device tensors."""
        import torch
        gpn = _check_groups(features, group_ptr, target)
        dev = self.params.device
        gp = _on(group_ptr if isinstance(group_ptr, torch.Tensor) else gpn.astype(np.int32), dev, torch.int32,
                 "group_ptr")
        return self._gradient(_dev_f32(features, dev), gp, _dev_f32(target, dev, "target"), stream)

    def _gradient(self, X, gp, t, stream=None):
        """gradient() on checked device tensors: X [rows, F] float32, gp the
        int32 group offsets from 0 to rows, t [rows] float32."""
        import torch
        rows, groups = X.shape[0], gp.numel() - 1
        sc = self.to_c()
        lib = A.load()
        nb = lib.gbx_scorer_workspace_bytes(C.byref(sc), rows)
        dev = self.params.device
        ws = torch.empty(nb, dtype=torch.uint8, device=dev)
        grad = torch.empty(self.count, dtype=torch.float32, device=dev)
        loss = torch.empty(1, dtype=torch.float32, device=dev)
        A.check(lib, lib.gbx_scorer_gradient(C.byref(sc), rows, X.data_ptr(), groups, gp.data_ptr(), t.data_ptr(),
                                             grad.data_ptr(), loss.data_ptr(), ws.data_ptr(), nb, _stream(stream)),
                "gbx_scorer_gradient")
        return grad, loss

    def adam(self, grad, lr: float = 1e-3, stream=None):
        self.step += 1
        sc = self.to_c()
        lib = A.load()
        A.check(lib, lib.gbx_scorer_adam(C.byref(sc), grad.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
                                         self.step, lr, _stream(stream)), "gbx_scorer_adam")

    def train(self, data: "Dataset", epochs: int = 200, lr: float = 3e-3) -> List[float]:
        """Full-batch Adam on the dataset; returns the loss per epoch."""
        import torch
        _check_groups(data.features, data.group_ptr, data.target)
        dev = self.params.device
        X = _dev_f32(data.features, dev)
        gp = _on(data.group_ptr.astype(np.int32), dev, torch.int32, "group_ptr")
        t = _dev_f32(data.target, dev, "target")
        losses = []
        for _ in range(epochs):
            g, l = self._gradient(X, gp, t)
            self.adam(g, lr)
            losses.append(float(l.item()) / max(1, data.groups))
        return losses


def _check_features(features) -> int:
    """Feature rows as the scorer kernels read them: [rows, F]. Returns rows."""
    shape = tuple(features.shape) if hasattr(features, "shape") else np.shape(features)
    if len(shape) != 2 or shape[1] != F:
        raise ValueError(f"features must be [rows, {F}], got {shape}")
    return int(shape[0])


def _check_groups(features, group_ptr, target) -> np.ndarray:
    """Listwise batch as the gradient kernel reads it: features [rows, F],
    group offsets rising from 0 to rows, one target per row. Returns the
    offsets on the host."""
    rows = _check_features(features)
    if hasattr(group_ptr, "detach"):
        group_ptr = group_ptr.detach().cpu().numpy()
    gpn = np.asarray(group_ptr).astype(np.int64).ravel()
    if gpn.size < 1 or gpn[0] != 0 or gpn[-1] != rows or np.any(np.diff(gpn) < 0):
        raise ValueError(f"group_ptr must rise from 0 to the row count {rows}")
    if int(np.prod(np.shape(target))) != rows:
        raise ValueError(f"target must hold one value per row ({rows})")
    return gpn


def _on(a, device, dtype, name):
    """a (tensor or array) as a contiguous tensor of dtype on the scorer's
    device. Host data is copied there; a tensor already on another CUDA
    device is refused (the kernels read every operand on one device)."""
    import torch
    if isinstance(a, torch.Tensor):
        if a.is_cuda and a.device != device:
            raise ValueError(f"{name} is on {a.device}, the scorer's parameters on {device}")
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dtype).contiguous()


def _dev_f32(a, device, name="features"):
    import torch
    return _on(a, device, torch.float32, name)


def features(x, lb, ub, order: int, depth: int, gap: float, value: float, vars_) -> np.ndarray:
    """Host features of candidates vars_ of one node (gbx_branch_features)."""
    lib = A.load()
    x, lb, ub = (np.ascontiguousarray(v, np.float64).ravel() for v in (x, lb, ub))
    vs = np.ascontiguousarray(vars_, np.int32).ravel()
    if lb.size != x.size or ub.size != x.size:
        raise ValueError("x, lb and ub must have the same length")
    if vs.size and (vs.min() < 0 or vs.max() >= x.size):
        raise ValueError(f"candidate variable index out of range [0, {x.size})")
    out = np.zeros((len(vs), F), np.float32)
    lib.gbx_branch_features(len(x), x.ctypes.data, lb.ctypes.data, ub.ctypes.data, order, depth, gap, value,
                            len(vs), vs.ctypes.data, out.ctypes.data)
    return out


@dataclasses.dataclass
class Dataset:
    features: np.ndarray      # [rows, F] float32
    group_ptr: np.ndarray     # [groups + 1] int32
    target: np.ndarray        # [rows] float32, sums to 1 per group
    sb_scores: np.ndarray     # [rows] raw strong-branching scores

    @property
    def groups(self) -> int:
        return len(self.group_ptr) - 1

    @staticmethod
    def concat(parts: List["Dataset"]) -> "Dataset":
        f, g, t, s = [], [0], [], []
        for p in parts:
            f.append(p.features)
            t.append(p.target)
            s.append(p.sb_scores)
            g.extend((p.group_ptr[1:] + g[-1]).tolist())
        return Dataset(np.concatenate(f), np.asarray(g, np.int32), np.concatenate(t), np.concatenate(s))


def collect_strong_branching(inst, max_nodes: int = 40, max_candidates: int = 24, max_iters: int = 400,
                             eps: float = 1e-6, tau: float = 0.5) -> Dataset:
    """Strong-branching labels along a best-first search that branches on the
    strong-branching winner, every relaxation by the library (FP64 path).
    Targets are softmax(log(score) / tau) over the node's candidates."""
    import heapq
    import torch
    obj, lmo, prob = inst.objective, inst.lmo, inst.problem
    n = len(prob.lb)
    order = lmo.order if isinstance(lmo, api.BirkhoffLMO) else 0
    int_vars = np.asarray(list(prob.int_vars), np.int64)
    s = inst.settings
    alg = A.Algorithm(s.algorithm, A.LS_QUADRATIC_EXACT if s.line_search == A.LS_SECANT else s.line_search,
                      s.secant_iters, s.secant_tol, s.secant_denom_eps, A.PRECISION_FP64)
    flags = np.zeros(n, np.uint8)
    flags[int_vars] = 1
    d_flags = torch.from_numpy(flags).cuda()

    def relax(lbs, ubs):
        N = lbs.shape[0]
        T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
        x = T(np.clip(lbs, 0, None).copy())
        it = torch.zeros(N, dtype=torch.int32, device="cuda")
        st = torch.zeros(N, dtype=torch.uint8, device="cuda")
        out = api.relax_batch(obj, lmo, alg, x, T(lbs), T(ubs), T(np.full(N, eps)), it, st, max_iters, d_flags,
                              1e-6)
        torch.cuda.synchronize()
        gap, val, stt = out["gap"].cpu().numpy(), out["value"].cpu().numpy(), st.cpu().numpy()
        bound = np.where(stt == A.NODE_INFEASIBLE, np.inf, np.where(np.isfinite(gap) & (gap >= 0), val - gap, -np.inf))
        return x.cpu().numpy(), gap, val, stt, bound

    lb0, ub0 = np.asarray(prob.lb, np.float64), np.asarray(prob.ub, np.float64)
    x, gap, val, stt, bnd = relax(lb0[None], ub0[None])
    heap = [(float(bnd[0]), 0, lb0, ub0, x[0], float(gap[0]), float(val[0]), 0)]
    tick = 1
    parts_f, parts_t, parts_s, gp = [], [], [], [0]
    done = 0
    while heap and done < max_nodes:
        L, _, lb, ub, xn, g, v, depth = heapq.heappop(heap)
        fr = xn[int_vars] - np.floor(xn[int_vars])
        dist = np.minimum(fr, 1 - fr)
        cand = int_vars[dist > 1e-6]
        if len(cand) == 0:
            continue
        cand = cand[np.argsort(-np.minimum(fr, 1 - fr)[dist > 1e-6], kind="stable")][:max_candidates]
        C_ = len(cand)
        lbs = np.repeat(lb[None], 2 * C_, 0)
        ubs = np.repeat(ub[None], 2 * C_, 0)
        for t, j in enumerate(cand):
            ubs[2 * t, j] = math.floor(xn[j])
            lbs[2 * t + 1, j] = math.ceil(xn[j])
        cx, cg, cv, cs, cb = relax(lbs, ubs)
        base = L if np.isfinite(L) else 0.0
        e = 1e-6 * max(1.0, abs(base))
        d0 = np.maximum(cb[0::2] - base, e)
        d1 = np.maximum(cb[1::2] - base, e)
        d0 = np.where(np.isfinite(d0), d0, 1e3 * (1 + abs(base)))
        d1 = np.where(np.isfinite(d1), d1, 1e3 * (1 + abs(base)))
        score = d0 * d1
        w = np.exp((np.log(score) - np.log(score).max()) / tau)
        tgt = w / w.sum()
        parts_f.append(features(xn, lb, ub, order, depth, g, v, cand))
        parts_t.append(tgt.astype(np.float32))
        parts_s.append(score.astype(np.float32))
        gp.append(gp[-1] + C_)
        done += 1
        best = int(np.argmax(score))
        for side in (0, 1):
            r = 2 * best + side
            if cs[r] == A.NODE_INFEASIBLE:
                continue
            heapq.heappush(heap, (float(cb[r]), tick, lbs[r], ubs[r], cx[r], float(cg[r]), float(cv[r]), depth + 1))
            tick += 1
    return Dataset(np.concatenate(parts_f), np.asarray(gp, np.int32), np.concatenate(parts_t),
                   np.concatenate(parts_s))
