"""The C-ABI library loads on a CPU-only machine, exports every entry point the
header declares, and its structures have the layout the ctypes mirror uses.
No compute call is made here."""
import ctypes as C
import pathlib
import re
import subprocess

import numpy as np
import pytest

from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, build

ROOT = pathlib.Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gpuboscia_gb300.h"


@pytest.fixture(scope="module")
def lib():
    build.build()
    return A.load()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbx_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_exported_set():
    assert declared_functions() == sorted(A.EXPORTED_SYMBOLS)


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(A.LIB_PATH)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (gbx_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    for f in declared_functions():
        assert hasattr(lib, f)
    assert lib.gbx_abi_version() == 4


_LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include "gpuboscia_gb300.h"
#define S(T) printf(#T " %zu\n", sizeof(T));
#define O(T, f) printf(#T "." #f " %zu\n", offsetof(T, f));
int main(void) {
  S(gbx_objective) O(gbx_objective, Q) O(gbx_objective, constant) O(gbx_objective, B)
  S(gbx_lmo) O(gbx_lmo, is_int) O(gbx_lmo, order)
  S(gbx_algorithm) O(gbx_algorithm, secant_tol) O(gbx_algorithm, precision)
  S(gbx_node_batch) O(gbx_node_batch, x) O(gbx_node_batch, integer_flags)
  S(gbx_problem) O(gbx_problem, n_int)
  S(gbx_settings) O(gbx_settings, algorithm) O(gbx_settings, time_limit_seconds) O(gbx_settings, use_cuda_graph)
  O(gbx_settings, scorer) O(gbx_settings, autotune) O(gbx_settings, device_frontier)
  O(gbx_settings, frontier_capacity) O(gbx_settings, incumbent_cutoff) O(gbx_node_batch, cutoff)
  O(gbx_settings, frontier_slots) O(gbx_settings, node_limit) O(gbx_result, reached_node_limit)
  O(gbx_result, batches) O(gbx_settings, trace) S(gbx_round_trace) O(gbx_round_trace, nodes)
  S(gbx_scorer) O(gbx_scorer, params) O(gbx_scorer, params_bf16)
  S(gbx_result) O(gbx_result, x)
  return 0;
}
"""


def test_struct_layouts_match_ctypes(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(_LAYOUT_C)
    exe = tmp_path / "layout"
    # the header is plain C: it compiles warning-free under strict C99
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", str(ROOT / "include"),
                    str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    M = {"gbx_objective": A.Objective, "gbx_lmo": A.LMO, "gbx_algorithm": A.Algorithm,
         "gbx_node_batch": A.NodeBatch, "gbx_problem": A.Problem, "gbx_settings": A.Settings,
         "gbx_result": A.Result, "gbx_scorer": A.Scorer, "gbx_round_trace": A.RoundTrace}
    for key, val in got.items():
        if "." in key:
            t, f = key.split(".")
            assert getattr(M[t], f).offset == int(val), key
        else:
            assert C.sizeof(M[key]) == int(val), key


def test_default_settings_match_reference_defaults(lib):
    s = A.Settings()
    lib.gbx_default_settings(C.byref(s))
    d = A.default_settings()
    for f, _ in A.Settings._fields_:
        if f == "algorithm":
            for g, _ in A.Algorithm._fields_:
                assert getattr(s.algorithm, g) == getattr(d.algorithm, g), g
        elif f not in ("root_initial_point", "trace"):
            assert getattr(s, f) == getattr(d, f), f


def test_workspace_sizing_is_host_only(lib):
    """gbx_relax_workspace_bytes runs without a GPU; invalid descriptors give 0."""
    keep = api._Keep()
    inst_A = np.zeros((36, 36))
    obj = api.GraphMatchingObjective(inst_A, inst_A).to_c("host", keep)
    lmo = api.BirkhoffLMO(36).to_c(36 * 36, "host", keep)
    alg = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    assert lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(alg), 256) > 0
    big = api.GraphMatchingObjective(np.zeros((120, 120)), np.zeros((120, 120))).to_c("host", keep)
    blmo = api.BirkhoffLMO(120).to_c(120 * 120, "host", keep)
    # order 120 node vectors spill to the global workspace: it scales with the batch
    w1 = lib.gbx_relax_workspace_bytes(C.byref(big), C.byref(blmo), C.byref(alg), 1)
    w8 = lib.gbx_relax_workspace_bytes(C.byref(big), C.byref(blmo), C.byref(alg), 8)
    assert w8 > w1 > 120 * 120 * 8
    bad = A.LMO(A.LMO_BIRKHOFF, 36 * 36, 1.0, None, 35)
    assert lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(bad), C.byref(alg), 4) == 0
    assert b"order" in lib.gbx_last_error()
    assert lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(alg), -1) == 0
    assert b"n_nodes" in lib.gbx_last_error()


def test_static_entry_rejects_negative_sizes_with_a_message(lib):
    """The allocation-free entry checks the batch's sizes itself, before it
    sizes the scratch or touches a device, and says why it refused."""
    keep = api._Keep()
    obj = api.DenseQuadraticObjective(np.eye(4)).to_c("host", keep)
    lmo = api.BoxLMO().to_c(4, "host", keep)
    alg = A.Algorithm(A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    for n_nodes, iters in ((-1, 5), (3, -2)):
        lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(A.LMO(A.LMO_BIRKHOFF, 16, 1.0, None, 3)),
                                      C.byref(alg), 1)   # leaves an unrelated message behind
        b = A.NodeBatch()
        b.n_nodes, b.max_iters = n_nodes, iters
        assert lib.gbx_relax_batch_static(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b), None) \
            == A.ERR_INVALID
        assert b"non-negative" in lib.gbx_last_error()


def test_relax_rejects_bad_arguments_without_launching(lib):
    keep = api._Keep()
    obj = api.DenseQuadraticObjective(np.eye(4)).to_c("host", keep)
    lmo = api.BoxLMO().to_c(4, "host", keep)
    alg = A.Algorithm(A.ALG_FRANK_WOLFE, 9, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    b = A.NodeBatch()
    assert lib.gbx_relax_batch(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b), None, 0, None) == A.ERR_INVALID
    alg.line_search = A.LS_OPEN_LOOP
    b.n_nodes = 2
    assert lib.gbx_relax_batch(C.byref(obj), C.byref(lmo), C.byref(alg), C.byref(b), None, 0, None) == A.ERR_INVALID
    assert b"null" in lib.gbx_last_error()


def test_device_frontier_rejects_bad_settings_without_launching(lib):
    """gbx_solve with device_frontier checks its arguments on the host before any
    CUDA call (frontier.cu, solve_device_frontier), so every rejection below is
    reachable without a GPU and names the offending setting."""
    keep = api._Keep()
    n = 4
    obj = api.DenseQuadraticObjective(np.eye(n)).to_c("host", keep)
    lmo = api.BoxLMO().to_c(n, "host", keep)
    lb, ub = np.zeros(n), np.ones(n)
    iv = np.arange(n, dtype=np.int32)
    prob = A.Problem(n, lb.ctypes.data, ub.ctypes.data, iv.ctypes.data, n)
    res = A.Result()

    def solve(**kw):
        s = A.default_settings()
        s.device_frontier = 1
        for k, v in kw.items():
            setattr(s, k, v)
        rc = lib.gbx_solve(C.byref(prob), C.byref(obj), C.byref(lmo), C.byref(s), C.byref(res))
        return rc, lib.gbx_last_error().decode()

    for kw, word in [(dict(gpu_batch_size=0), "gpu_batch_size"),
                     (dict(gpu_batch_size=1025), "gpu_batch_size"),
                     (dict(branch_k=9), "branch_k"),
                     (dict(branch_k=0), "branch_k"),
                     (dict(frontier_slots=3), "frontier_slots"),
                     (dict(gpu_max_iters=0), "positive"),
                     (dict(gpu_eps_decay=1.5), "tolerance"),
                     (dict(abs_gap_tol=-1.0), "tolerance"),
                     (dict(time_limit_seconds=0.0), "time limit"),
                     (dict(natural_lower_bound=float("nan")), "natural lower bound")]:
        rc, msg = solve(**kw)
        assert rc == A.ERR_INVALID, (kw, rc, msg)
        assert word in msg, (kw, msg)

    sc = A.Scorer(A.SCORER_FEATURES, 7, C.c_void_p(16), None)   # hidden must be 16, 32 or 64
    rc, msg = solve(scorer=C.cast(C.pointer(sc), C.c_void_p))
    assert rc == A.ERR_INVALID and "scorer" in msg

    bad_iv = np.array([n + 3], dtype=np.int32)
    prob_bad = A.Problem(n, lb.ctypes.data, ub.ctypes.data, bad_iv.ctypes.data, 1)
    s = A.default_settings()
    s.device_frontier = 1
    rc = lib.gbx_solve(C.byref(prob_bad), C.byref(obj), C.byref(lmo), C.byref(s), C.byref(res))
    assert rc == A.ERR_INVALID and b"out of range" in lib.gbx_last_error()

    # an LMO the relaxation kernel cannot size (Birkhoff order not matching n)
    blmo = A.LMO(A.LMO_BIRKHOFF, n, 1.0, None, 3)
    rc = lib.gbx_solve(C.byref(prob), C.byref(obj), C.byref(blmo), C.byref(s), C.byref(res))
    assert rc == A.ERR_INVALID


def test_python_solve_checks_sizes_before_the_gpu():
    """api.solve rejects arrays whose sizes disagree with n_vars (the C side
    would read past them) before any device work: these raise on a CPU-only
    machine as ValueError, not as a CUDA error."""
    obj = api.DenseQuadraticObjective(np.eye(3))
    good = api.Problem(3, np.zeros(3), np.ones(3), [0, 1, 2])
    cases = [
        (api.Problem(3, np.zeros(2), np.ones(3), [0]), api.Settings(), "lb"),
        (api.Problem(3, np.zeros(3), np.ones(4), [0]), api.Settings(), "ub"),
        (api.Problem(3, np.zeros(3), np.ones(3), [0, 3]), api.Settings(), "out of range"),
        (api.Problem(3, np.zeros(3), np.ones(3), [-1]), api.Settings(), "out of range"),
        (api.Problem(0, np.zeros(0), np.ones(0), []), api.Settings(), "n_vars"),
        (good, api.Settings(root_initial_point=np.zeros(2)), "root_initial_point"),
    ]
    for prob, s, word in cases:
        with pytest.raises(ValueError, match=word):
            api.solve(prob, obj, api.BoxLMO(), s)
    api.check_problem(good, api.Settings(root_initial_point=np.zeros(3)))


def test_node_batch_tensors_are_checked_before_the_gpu():
    """relax_batch / BatchRelaxer refuse node tensors whose dtype, size,
    layout or device differ from what gbx_node_batch describes (the kernel
    would read or write outside a buffer): ValueError, before any device work."""
    torch = pytest.importorskip("torch")
    N, n = 3, 4
    good = dict(x=torch.zeros(N, n, dtype=torch.float64), lb=torch.zeros(N, n, dtype=torch.float64),
                ub=torch.ones(N, n, dtype=torch.float64), eps=torch.full((N,), 1e-6, dtype=torch.float64),
                iterations=torch.zeros(N, dtype=torch.int32), status=torch.zeros(N, dtype=torch.uint8),
                integer_flags=torch.ones(n, dtype=torch.uint8))
    bad = [
        ("x", torch.zeros(N * n, dtype=torch.float64), "2-D"),
        ("lb", torch.zeros(N, n, dtype=torch.float32), "float64"),
        ("ub", torch.ones(N, n - 1, dtype=torch.float64), "elements"),
        ("eps", torch.full((N + 1,), 1e-6, dtype=torch.float64), "elements"),
        ("iterations", torch.zeros(N, dtype=torch.int64), "int32"),
        ("status", torch.zeros(N, dtype=torch.int32), "uint8"),
        ("integer_flags", torch.ones(n + 1, dtype=torch.uint8), "elements"),
        ("lb", torch.zeros(n, N, dtype=torch.float64).t(), "contiguous"),
        ("eps", [1e-6] * N, "tensor"),
    ]
    obj = api.DenseQuadraticObjective(np.eye(n))
    alg = A.Algorithm(A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    for name, value, word in bad:
        args = dict(good, **{name: value})
        with pytest.raises(ValueError, match=word):
            api.check_node_tensors(**args)
        with pytest.raises(ValueError, match=word):
            api.relax_batch(obj, api.BoxLMO(), alg, args["x"], args["lb"], args["ub"], args["eps"],
                            args["iterations"], args["status"], 10, args["integer_flags"])
    # a (1, n) batch may carry its bounds as flat n-vectors: same memory, accepted
    one = dict(good, x=torch.zeros(1, n, dtype=torch.float64), lb=torch.zeros(n, dtype=torch.float64),
               ub=torch.ones(n, dtype=torch.float64), eps=torch.full((1,), 1e-6, dtype=torch.float64),
               iterations=torch.zeros(1, dtype=torch.int32), status=torch.zeros(1, dtype=torch.uint8))
    # everything right but the device: host tensors are refused last
    for args in (good, one):
        with pytest.raises(ValueError, match="CUDA device"):
            api.check_node_tensors(**args)
        with pytest.raises(ValueError, match="CUDA device"):
            api.BatchRelaxer(obj, api.BoxLMO(), alg, args["x"], args["lb"], args["ub"], args["eps"],
                             args["iterations"], args["status"], 10, args["integer_flags"])


def test_lmo_feasibility_gradient_tensors_are_checked():
    """lmo_batch, node_feasible_batch and the gradient entry points refuse
    tensors that disagree with each other or with the objective's variable
    count (the C side sizes its reads from them): ValueError before any
    device work, the device checked last."""
    torch = pytest.importorskip("torch")
    c, n = 4, 9
    f64 = lambda *s: torch.zeros(*s, dtype=torch.float64)
    lmo = api.BirkhoffLMO(3)
    with pytest.raises(ValueError, match="elements"):
        api.lmo_batch(lmo, 0, f64(c, n), f64(c, n - 1), f64(c, n))
    with pytest.raises(ValueError, match="float64"):
        api.lmo_batch(lmo, 1, f64(c, n), f64(c, n), f64(c, n), x=torch.zeros(c, n, dtype=torch.float32))
    with pytest.raises(ValueError, match="needs x"):
        api.lmo_batch(lmo, 1, f64(c, n), f64(c, n), f64(c, n))
    with pytest.raises(ValueError, match="CUDA device"):
        api.lmo_batch(lmo, 0, f64(c, n), f64(c, n), f64(c, n))
    with pytest.raises(ValueError, match="integer_flags"):
        api.node_feasible_batch(lmo, f64(c, n), f64(c, n), torch.ones(n - 1, dtype=torch.uint8))
    with pytest.raises(ValueError, match="2-D"):
        api.node_feasible_batch(lmo, f64(c * n), f64(c * n))
    with pytest.raises(ValueError, match="CUDA device"):
        api.node_feasible_batch(lmo, f64(c, n), f64(c, n), torch.ones(n, dtype=torch.uint8))
    gm = api.GraphMatchingObjective(np.eye(3), np.eye(3))
    with pytest.raises(ValueError, match="CUDA device"):
        api.objective_gradient_batch(gm, f64(c, n))
    with pytest.raises(ValueError, match="variables"):
        api.objective_gradient_batch(gm, f64(c, 16))
    with pytest.raises(ValueError, match="float64"):
        api.objective_gradient_batch(gm, torch.zeros(c, n, dtype=torch.float32))
    with pytest.raises(ValueError, match="variables"):
        api.objective_gradient_batch_f32(gm, torch.zeros(c, 16))
    # relax_batch: node vectors must match the objective's size
    N = 2
    with pytest.raises(ValueError, match="variables"):
        api.relax_batch(api.DenseQuadraticObjective(np.eye(5)), api.BoxLMO(),
                        A.Algorithm(A.ALG_FRANK_WOLFE, A.LS_OPEN_LOOP, 4, 1e-10, 1e-14, A.PRECISION_FP64),
                        f64(N, 4), f64(N, 4), f64(N, 4), f64(N), torch.zeros(N, dtype=torch.int32),
                        torch.zeros(N, dtype=torch.uint8), 10)


def test_cluster_launch_shape_only_where_it_applies(lib):
    """Persistent 2 (a cluster of four CTAs per node) pins only for mixed
    precision graph matching over the Birkhoff polytope at orders 129..404;
    elsewhere it is refused on the host, without a GPU."""
    keep = api._Keep()
    mixed = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_MIXED)
    fp64 = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    for order, alg, ok in ((400, mixed, True), (300, mixed, True), (36, mixed, False), (400, fp64, False),
                           (500, mixed, False)):
        o = api.GraphMatchingObjective(np.zeros((order, order)), np.zeros((order, order))).to_c("host", keep)
        lm = api.BirkhoffLMO(order).to_c(order * order, "host", keep)
        rc = lib.gbx_relax_set_launch_shape(C.byref(o), C.byref(lm), C.byref(alg), -1, 2)
        assert (rc == A.OK) == ok, (order, lib.gbx_last_error())
        if ok:
            # the cluster shape needs no workspace beyond the one-CTA shape's
            assert lib.gbx_relax_workspace_bytes(C.byref(o), C.byref(lm), C.byref(alg), 4) > 0
        assert lib.gbx_relax_set_launch_shape(C.byref(o), C.byref(lm), C.byref(alg), -1, 0) == A.OK
    o = api.GraphMatchingObjective(np.zeros((400, 400)), np.zeros((400, 400))).to_c("host", keep)
    lm = api.BirkhoffLMO(400).to_c(400 * 400, "host", keep)
    assert lib.gbx_relax_set_launch_shape(C.byref(o), C.byref(lm), C.byref(mixed), -1, 4) == A.ERR_INVALID
    # persistent 3, a pair of CTAs per node, is the FP64 dense quadratic objective's
    assert lib.gbx_relax_set_launch_shape(C.byref(o), C.byref(lm), C.byref(mixed), -1, 3) == A.ERR_UNSUPPORTED
    fp64 = A.Algorithm(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    q = api.DenseQuadraticObjective(np.eye(200)).to_c("host", keep)
    box = api.BoxLMO().to_c(200, "host", keep)
    assert lib.gbx_relax_set_launch_shape(C.byref(q), C.byref(box), C.byref(fp64), -1, 3) == A.OK
    assert lib.gbx_relax_set_launch_shape(C.byref(q), C.byref(box), C.byref(fp64), -1, 0) == A.OK


def test_oracle_warps_only_where_they_apply(lib):
    """Four warps per integer oracle pin only for the large-order mixed
    Birkhoff kernel (orders 129..512); one warp and the default pin anywhere;
    other counts are argument errors. All checked on the host."""
    keep = api._Keep()
    mixed = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_MIXED)
    fp64 = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    for order, alg, ok in ((400, mixed, True), (200, mixed, True), (500, mixed, True), (120, mixed, False),
                           (36, mixed, False), (400, fp64, False)):
        o = api.GraphMatchingObjective(np.zeros((order, order)), np.zeros((order, order))).to_c("host", keep)
        lm = api.BirkhoffLMO(order).to_c(order * order, "host", keep)
        rc = lib.gbx_relax_set_oracle_warps(C.byref(o), C.byref(lm), C.byref(alg), 4)
        assert (rc == A.OK) == ok, (order, lib.gbx_last_error())
        if not ok:
            assert rc == A.ERR_UNSUPPORTED
        assert lib.gbx_relax_set_oracle_warps(C.byref(o), C.byref(lm), C.byref(alg), 1) == A.OK
        assert lib.gbx_relax_set_oracle_warps(C.byref(o), C.byref(lm), C.byref(alg), -1) == A.OK
        for bad in (0, 2, 8):
            assert lib.gbx_relax_set_oracle_warps(C.byref(o), C.byref(lm), C.byref(alg), bad) == A.ERR_INVALID
            assert "oracle warps" in lib.gbx_last_error().decode()


def test_nodes_per_sm_only_for_fp64(lib):
    """Two nodes per SM pin for the FP64 kernels; mixed precision refuses 2 (its
    kernels fix their own occupancy); other counts are argument errors."""
    keep = api._Keep()
    fp64 = A.Algorithm(A.ALG_FRANK_WOLFE, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_FP64)
    mixed = A.Algorithm(A.ALG_DICG, A.LS_QUADRATIC_EXACT, 4, 1e-10, 1e-14, A.PRECISION_MIXED)
    q = api.DenseQuadraticObjective(np.eye(64)).to_c("host", keep)
    box = api.BoxLMO().to_c(64, "host", keep)
    for v in (2, 1, -1):
        assert lib.gbx_relax_set_nodes_per_sm(C.byref(q), C.byref(box), C.byref(fp64), v) == A.OK
    for bad in (0, 3, 4):
        assert lib.gbx_relax_set_nodes_per_sm(C.byref(q), C.byref(box), C.byref(fp64), bad) == A.ERR_INVALID
        assert "nodes per SM" in lib.gbx_last_error().decode()
    o = api.GraphMatchingObjective(np.zeros((36, 36)), np.zeros((36, 36))).to_c("host", keep)
    lm = api.BirkhoffLMO(36).to_c(36 * 36, "host", keep)
    assert lib.gbx_relax_set_nodes_per_sm(C.byref(o), C.byref(lm), C.byref(mixed), 2) == A.ERR_UNSUPPORTED
    assert lib.gbx_relax_set_nodes_per_sm(C.byref(o), C.byref(lm), C.byref(mixed), -1) == A.OK
