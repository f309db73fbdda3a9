"""Seeded synthetic instances of the benchmark workloads and the reference's example models.

Every draw comes from numpy's PCG64 generator (bit-stable across platforms);
normals use an explicit Box-Muller transform so no library sampler decides
the values. The generators return plain numpy arrays plus the objective /
LMO / problem objects of gpuboscia_gb300.api.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import api
from ._abi import ALG_DICG

SEEDS = {1: 1001, 2: 1002, 3: 1003, 4: 1004, 5: 1005}


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def normal(rng: np.random.Generator, size, mean=0.0, std=1.0) -> np.ndarray:
    """Box-Muller over the generator's uniform doubles."""
    count = int(np.prod(size))
    m = (count + 1) // 2
    u1 = 1.0 - rng.random(m)          # (0, 1]
    u2 = rng.random(m)
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2.0 * np.pi * u2), r * np.sin(2.0 * np.pi * u2)])[:count]
    return (mean + std * z).reshape(size)


def permutation(rng: np.random.Generator, n: int) -> np.ndarray:
    """Fisher-Yates over the generator's integers."""
    p = np.arange(n)
    for i in range(n - 1, 0, -1):
        j = int(rng.integers(0, i + 1))
        p[i], p[j] = p[j], p[i]
    return p


def gnp_graph(rng: np.random.Generator, n: int, p: float) -> np.ndarray:
    u = rng.random((n, n))
    A = (np.triu(u, 1) < p).astype(np.float64)
    A = np.triu(A, 1)
    return A + A.T


def random_regular(rng: np.random.Generator, n: int, d: int, mixing: int = 10) -> np.ndarray:
    """Random simple d-regular graph: the circulant graph (i ~ i +- 1..d/2, plus
    the antipode when d is odd) randomised by mixing*|E| degree-preserving swaps."""
    assert n * d % 2 == 0 and d < n
    A = np.zeros((n, n))
    for i in range(n):
        for k in range(1, d // 2 + 1):
            A[i, (i + k) % n] = A[(i + k) % n, i] = 1.0
        if d % 2:
            A[i, (i + n // 2) % n] = A[(i + n // 2) % n, i] = 1.0
    return double_edge_swaps(rng, A, mixing * (n * d // 2))


def double_edge_swaps(rng: np.random.Generator, A: np.ndarray, swaps: int) -> np.ndarray:
    """Degree-preserving swaps (a-b, c-d) -> (a-d, c-b) keeping the graph simple."""
    A = A.copy()
    edges = np.argwhere(np.triu(A, 1) > 0)
    m = len(edges)
    done = 0
    while done < swaps:
        i = int(rng.integers(0, m))
        j = int(rng.integers(0, m))
        a, b = edges[i]
        c, d = edges[j]
        if rng.random() < 0.5:
            c, d = d, c
        if len({a, b, c, d}) < 4 or A[a, d] or A[c, b]:
            continue
        A[a, b] = A[b, a] = A[c, d] = A[d, c] = 0.0
        A[a, d] = A[d, a] = A[c, b] = A[b, c] = 1.0
        edges[i] = (a, d)
        edges[j] = (c, b)
        done += 1
    return A


def permute(A: np.ndarray, p: np.ndarray) -> np.ndarray:
    """B = P A P' with P[i, p[i]] = 1, i.e. B[i, j] = A[p[i], p[j]]."""
    return A[np.ix_(p, p)]


@dataclasses.dataclass
class Instance:
    name: str
    problem: api.Problem
    objective: object
    lmo: object
    settings: api.Settings
    known_optimum: float | None = None
    solution: np.ndarray | None = None


def box_qp(n: int = 64, seed: int = SEEDS[1]) -> Instance:
    """Box-constrained binary QP: f = x'Qx/2 + c'x, Q = M'M/64 + 0.1 I, x binary in [0,1]^n."""
    rng = _rng(seed)
    M = normal(rng, (n, n))
    Q = M.T @ M / 64.0 + 0.1 * np.eye(n)
    Q = 0.5 * (Q + Q.T)
    c = rng.random(n) * 2.0 - 1.0
    prob = api.Problem(n, np.zeros(n), np.ones(n), list(range(n)))
    s = api.Settings(algorithm=0, line_search=4, rel_gap_tol=1e-6, abs_gap_tol=1e-6)
    return Instance("box_bqp_n64", prob, api.DenseQuadraticObjective(Q, c), api.BoxLMO(), s)


def portfolio(assets: int = 100, months: int = 600, cardinality: int = 10, seed: int = SEEDS[3]) -> Instance:
    """Cardinality-constrained mean-variance portfolio.

    Returns of a 3-factor model: factor returns N(0.5 %, 4 %) per month, betas
    N(1, 0.3), idiosyncratic volatility U[4 %, 10 %]. Sigma and mu are the sample
    covariance and mean. min w'Sigma w - 0.5 mu'w over x = (w, z) with
    sum w = 1, 0 <= w <= z, sum z <= cardinality, z binary: f = x'Qx/2 + c'x with
    Q = diag(2 Sigma, 0) and c = (-0.5 mu, 0)."""
    rng = _rng(seed)
    f = normal(rng, (months, 3), 0.005, 0.04)
    beta = normal(rng, (assets, 3), 1.0, 0.3)
    vol = 0.04 + 0.06 * rng.random(assets)
    eps = normal(rng, (months, assets)) * vol[None, :]
    R = f @ beta.T + eps
    mu = R.mean(0)
    D = R - mu
    Sigma = D.T @ D / (months - 1)
    n = 2 * assets
    Q = np.zeros((n, n))
    Q[:assets, :assets] = 2.0 * Sigma
    c = np.zeros(n)
    c[:assets] = -0.5 * mu
    prob = api.Problem(n, np.zeros(n), np.ones(n), list(range(assets, n)))
    s = api.Settings(algorithm=0, line_search=4, rel_gap_tol=1e-6, abs_gap_tol=1e-6, gpu_batch_size=64)
    return Instance(f"portfolio_n{assets}_k{cardinality}", prob, api.DenseQuadraticObjective(Q, c),
                    api.CardinalityLMO(assets, cardinality), s)


def portfolio_node_batch(assets: int, cardinality: int, nodes: int, seed: int = 7):
    """Open nodes with uneven fixings of z: some forced in (at most cardinality),
    some forced out."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = 2 * assets
    lb = np.zeros((nodes, n))
    ub = np.ones((nodes, n))
    for k in range(nodes):
        ins = rng.choice(assets, int(rng.integers(0, cardinality + 1)), replace=False)
        outs = rng.choice(np.setdiff1d(np.arange(assets), ins), int(rng.integers(0, assets // 3)), replace=False)
        lb[k, assets + ins] = 1.0
        ub[k, assets + outs] = 0.0
    return lb, ub


def graph_matching(order: int, A: np.ndarray, B: np.ndarray, name: str, known=None, solution=None) -> Instance:
    n = order * order
    prob = api.Problem(n, np.zeros(n), np.ones(n), list(range(n)))
    s = api.Settings(algorithm=1, line_search=0, natural_lower_bound=0.0, rel_gap_tol=1e-6, abs_gap_tol=1e-6)
    return Instance(name, prob, api.GraphMatchingObjective(A, B, 1.0), api.BirkhoffLMO(order), s, known, solution)


def birkhoff_gnp(order: int = 36, seed: int = SEEDS[2]) -> Instance:
    """Graph matching on a random graph: A = G(order, 1/2), B = P A P', optimum 0 at X = P'."""
    rng = _rng(seed)
    A = gnp_graph(rng, order, 0.5)
    p = permutation(rng, order)
    B = permute(A, p)
    X = np.zeros((order, order))
    X[p, np.arange(order)] = 1.0   # X = P': AX = XB
    return graph_matching(order, A, B, f"birkhoff_gnp_n{order}", 0.0, X.ravel())


def birkhoff_regular_perturbed(order: int = 120, degree: int = 8, swaps: int = 20,
                               seed: int = SEEDS[4]) -> Instance:
    """Graph matching on d-regular graphs: A d-regular, B = A after `swaps` double-edge swaps, then permuted (optimum > 0)."""
    rng = _rng(seed)
    A = random_regular(rng, order, degree)
    B = permute(double_edge_swaps(rng, A, swaps), permutation(rng, order))
    return graph_matching(order, A, B, f"birkhoff_regular_n{order}_perturbed")


def birkhoff_regular_isomorphic(order: int = 400, degree: int = 10, seed: int = SEEDS[5]) -> Instance:
    """Isomorphic d-regular pair: A d-regular, B = P A P' (optimum 0)."""
    rng = _rng(seed)
    A = random_regular(rng, order, degree)
    p = permutation(rng, order)
    X = np.zeros((order, order))
    X[p, np.arange(order)] = 1.0
    return graph_matching(order, A, permute(A, p), f"birkhoff_regular_n{order}", 0.0, X.ravel())


def birkhoff_node_batch(order: int, nodes: int, seed: int, max_forced: int | None = None,
                        forbid_frac: float = 0.05):
    """Open B&B nodes with uneven fixings over the order x order Birkhoff
    polytope: node i forces a random number of edges of its own random
    permutation and forbids a random subset of the others, so every node is
    feasible but nodes differ in size and active set. Returns (lb, ub) [nodes, n]."""
    rng = _rng(seed)
    n = order * order
    max_forced = order // 3 if max_forced is None else max_forced
    lb = np.zeros((nodes, n))
    ub = np.ones((nodes, n))
    for i in range(nodes):
        p = permutation(rng, order)
        keep = np.zeros((order, order), dtype=bool)
        keep[np.arange(order), p] = True
        forced = int(rng.integers(0, max_forced + 1))
        rows = permutation(rng, order)[:forced]
        L = np.zeros((order, order))
        L[rows, p[rows]] = 1.0
        U = np.where((rng.random((order, order)) < forbid_frac) & ~keep, 0.0, 1.0)
        lb[i] = L.ravel()
        ub[i] = U.ravel()
    return lb, ub


def box_node_batch(n: int, nodes: int, seed: int, max_fixed: int | None = None):
    """Open B&B nodes of a binary box problem with uneven numbers of fixed variables."""
    rng = _rng(seed)
    max_fixed = n // 4 if max_fixed is None else max_fixed
    lb = np.zeros((nodes, n))
    ub = np.ones((nodes, n))
    for i in range(nodes):
        k = int(rng.integers(0, max_fixed + 1))
        idx = permutation(rng, n)[:k]
        val = (rng.random(k) < 0.5).astype(np.float64)
        lb[i, idx] = val
        ub[i, idx] = val
    return lb, ub


# ---------------------------------------------------------------- instance files
def load_mat(path, name: str = "A") -> np.ndarray:
    """The real matrix `name` of a MATLAB v5 file (gbx_read_mat), row-major float64."""
    import ctypes as C
    from . import _abi as A
    lib = A.load()
    r, c = C.c_int(0), C.c_int(0)
    p = str(path).encode()
    rc = lib.gbx_read_mat(p, name.encode(), C.byref(r), C.byref(c), None, 0)
    if rc != A.OK:
        raise (ValueError if rc == A.ERR_INVALID else RuntimeError)(lib.gbx_last_error().decode())
    out = np.zeros((r.value, c.value))
    rc = lib.gbx_read_mat(p, name.encode(), C.byref(r), C.byref(c), out.ctypes.data, out.size)
    A.check(lib, rc, "gbx_read_mat")
    return out


def load_dimacs(path) -> np.ndarray:
    """The symmetric 0/1 adjacency of a DIMACS edge list (gbx_read_dimacs)."""
    import ctypes as C
    from . import _abi as A
    lib = A.load()
    n = C.c_int(0)
    p = str(path).encode()
    rc = lib.gbx_read_dimacs(p, C.byref(n), None, 0)
    if rc != A.OK:
        raise (ValueError if rc == A.ERR_INVALID else RuntimeError)(lib.gbx_last_error().decode())
    out = np.zeros((n.value, n.value))
    rc = lib.gbx_read_dimacs(p, C.byref(n), out.ctypes.data, out.size)
    A.check(lib, rc, "gbx_read_dimacs")
    return out


def graph_matching_from_file(path, seed: int = 0) -> Instance:
    """examples/main.cu:183-226: A from an instance file (.mat variable A, or a
    DIMACS edge list), B = A with rows and columns permuted by a seeded random
    permutation (B[r, c] = A[p[r], p[c]]), so the optimum is 0 at X = P'."""
    import os
    A = load_dimacs(path) if str(path).endswith(".dimacs") else load_mat(path, "A")
    if A.shape[0] != A.shape[1]:
        raise ValueError(f"{path}: adjacency is {A.shape[0]}x{A.shape[1]}, not square")
    m = A.shape[0]
    p = permutation(_rng(seed), m)
    B = A[np.ix_(p, p)]
    X = np.zeros((m, m))
    X[p, np.arange(m)] = 1.0   # A X = X B
    return graph_matching(m, A, B, os.path.basename(str(path)), 0.0, X.ravel())


# ---------------------------------------------------------------- sparse Sharpe
def sparse_sharpe(prices: np.ndarray, assets: int = 125, cardinality: int = 10, observations: int = 60,
                  epsilon: float = 1e-3, padded: int | None = None) -> Instance:
    """examples/sparse_sharpe.cu:550-799: discrete sparse Sharpe-ratio portfolio.

    prices: T x N gross returns (the MAT variable `data`); the first `assets`
    columns over the last `observations` rows. minimize 0.5 v'(Sigma + eps I)v
    - mu'v over 0 <= v_i <= U_i y_i, sum y <= cardinality, y binary; the
    portfolio is w = v / sum v. U_i = max(c_i + sqrt(max((H^-1)_ii r^2, 0)), 0)
    with c = H^-1 mu and r^2 = max(mu'c, 0) bounds every v on the level set
    below f = 0, and -r^2 / 2 (the unconstrained minimum) is the natural lower
    bound. x = (v, y) with y at `padded` (default: assets)."""
    prices = np.asarray(prices, np.float64)
    T, N = prices.shape
    if not 1 <= cardinality <= assets <= N:
        raise ValueError("need 1 <= cardinality <= assets <= available columns")
    half = assets if padded is None else int(padded)
    if half < assets:
        raise ValueError("padded must be >= assets")
    obs = T if observations <= 0 else min(observations, T)
    R = prices[T - obs:, :assets] - 1.0
    mu = R.sum(0) / obs
    D = R - mu
    H = D.T @ D * (1.0 / (obs - 1) if obs > 1 else 1.0) + epsilon * np.eye(assets)
    L = np.linalg.cholesky(H)
    center = np.linalg.solve(L.T, np.linalg.solve(L, mu))
    r2 = max(float(mu @ center), 0.0)
    Hinv_diag = np.diag(np.linalg.solve(L.T, np.linalg.solve(L, np.eye(assets))))
    U = np.maximum(center + np.sqrt(np.maximum(Hinv_diag * r2, 0.0)), 0.0)
    n = 2 * half
    Q = np.zeros((n, n))
    Q[:assets, :assets] = H
    c = np.zeros(n)
    c[:assets] = -mu
    lb = np.zeros(n)
    ub = np.zeros(n)
    ub[:assets] = U
    ub[half:half + assets] = 1.0
    prob = api.Problem(n, lb, ub, list(range(half, half + assets)))
    s = api.Settings(algorithm=1, line_search=3, secant_iters=16, secant_tol=1e-10, secant_denom_eps=1e-14,
                     gpu_max_iters=10000, integer_tol=1e-5, abs_gap_tol=1e-6, rel_gap_tol=1e-2,
                     natural_lower_bound=-0.5 * r2)
    return Instance(f"sparse_sharpe_n{assets}_m{cardinality}", prob, api.DenseQuadraticObjective(Q, c),
                    api.LinkedCardinalityLMO(U, cardinality), s)


def synthetic_gross_returns(months: int, assets: int, seed: int = SEEDS[3]) -> np.ndarray:
    """Monthly gross returns (1 + r) of a 3-factor model, the shape of the
    sparse-Sharpe example's `data` matrix."""
    rng = _rng(seed)
    f = normal(rng, (months, 3), 0.006, 0.04)
    beta = normal(rng, (assets, 3), 1.0, 0.3)
    vol = 0.03 + 0.08 * rng.random(assets)
    alpha = normal(rng, assets, 0.0, 0.004)
    return 1.0 + f @ beta.T + alpha[None, :] + normal(rng, (months, assets)) * vol[None, :]


def weighted_clique(vertices: int = 20, cardinality: int = 5, seed: int = 222222222) -> Instance:
    """examples/weighted_clique.cu:64-150: the maximum-weight induced subgraph
    with exactly `cardinality` vertices, as a convex binary quadratic.

    Edge weights w_ij ~ U[0, 1). f(x) = 2 sum_{i<j} (1 - w_ij) x_i x_j
    + lam sum_i x_i (x_i - 1), lam = vertices - 1: in 0.5 x'Qx + c'x form Q has
    2 lam on the diagonal and 2 (1 - w_ij) off it, c = -lam. The lam term is
    zero at binary points and makes Q diagonally dominant (convex). Over the
    equality simplex sum x = cardinality, x binary; DICG, the example's
    tolerances and its natural bound lam (cardinality^2 / vertices - cardinality)
    (Cauchy-Schwarz on sum x_i^2). The weights come from PCG64, not the
    example's mt19937_64, so the instance has the example's shape, not its
    exact numbers."""
    rng = _rng(seed)
    n = vertices
    W = np.zeros((n, n))
    iu = np.triu_indices(n, 1)
    W[iu] = rng.random(len(iu[0]))
    W = W + W.T
    lam = float(n - 1)
    Q = 2.0 * (1.0 - W)
    np.fill_diagonal(Q, 2.0 * lam)
    c = np.full(n, -lam)
    prob = api.Problem(n, np.zeros(n), np.ones(n), list(range(n)))
    s = api.Settings(algorithm=ALG_DICG, gpu_batch_size=1024, num_streams=2, gpu_max_iters=1000,
                     abs_gap_tol=1e-7, rel_gap_tol=1e-3,
                     natural_lower_bound=lam * (cardinality * cardinality / n - cardinality))
    return Instance(f"weighted_clique_{n}_{cardinality}", prob, api.DenseQuadraticObjective(Q, c),
                    api.EqualitySimplexLMO(float(cardinality), list(range(n))), s)
