"""ctypes mirror of include/gpuboscia_gb300.h and the loader of the CUDA library.

The structures here are byte-for-byte the C structs of the header; keep the two
in step. The library is built in-tree (gpuboscia_gb300/_build) by
``gpuboscia_gb300.build.build()``; importing the compute entry points without it
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
import pathlib

PKG_DIR = pathlib.Path(__file__).resolve().parent
BUILD_DIR = PKG_DIR / "_build"
LIB_PATH = BUILD_DIR / "libgpuboscia_gb300.so"

# status codes
OK = 0
ERR_INVALID = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_WORKSPACE = -4
ERR_TIMEOUT = -5

# node status byte
NODE_FRACTIONAL_UNCONVERGED = 0
NODE_FRACTIONAL_CONVERGED = 1
NODE_INFEASIBLE = 2
NODE_INTEGRAL_UNCONVERGED = 3
NODE_INTEGRAL_CONVERGED = 4
NODE_INITIAL_POINT_SUPPLIED = 0x80

OBJ_DENSE_QUADRATIC = 1
OBJ_GRAPH_MATCHING = 2

LMO_BOX = 1
LMO_SIMPLEX = 2
LMO_EQUALITY_SIMPLEX = 3
LMO_BIRKHOFF = 4
LMO_CARDINALITY = 5
LMO_LINKED_CARDINALITY = 6

ALG_FRANK_WOLFE = 0
ALG_DICG = 1

LS_OPEN_LOOP = 0
LS_SCALED_OPEN_LOOP = 1
LS_SAFEGUARDED_SCALED_OPEN_LOOP = 2
LS_SECANT = 3
LS_QUADRATIC_EXACT = 4

PRECISION_FP64 = 0
PRECISION_MIXED = 1

_dp = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_ip = C.POINTER(C.c_int)


class Objective(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("n", C.c_int),
        ("Q", C.c_void_p), ("c", C.c_void_p),
        ("scale", C.c_double), ("linear_scale", C.c_double), ("constant", C.c_double),
        ("order", C.c_int), ("A", C.c_void_p), ("B", C.c_void_p),
    ]


class LMO(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("n", C.c_int), ("right_side", C.c_double),
        ("is_int", C.c_void_p), ("order", C.c_int), ("upper", C.c_void_p),
    ]


class Algorithm(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("line_search", C.c_int), ("secant_iters", C.c_int),
        ("secant_tol", C.c_double), ("secant_denom_eps", C.c_double),
        ("precision", C.c_int),
    ]


class NodeBatch(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int), ("max_iters", C.c_int), ("candidate_tol", C.c_double),
        ("x", C.c_void_p), ("lb", C.c_void_p), ("ub", C.c_void_p), ("eps", C.c_void_p),
        ("iterations", C.c_void_p), ("status", C.c_void_p), ("gap", C.c_void_p),
        ("value", C.c_void_p), ("best_vertex", C.c_void_p), ("best_vertex_val", C.c_void_p),
        ("integer_flags", C.c_void_p), ("cutoff", C.c_void_p),
    ]


class Problem(C.Structure):
    _fields_ = [
        ("n_vars", C.c_int), ("lb", C.c_void_p), ("ub", C.c_void_p),
        ("int_vars", C.c_void_p), ("n_int", C.c_int),
    ]


SCORER_FEATURES = 16


class Scorer(C.Structure):
    _fields_ = [
        ("n_features", C.c_int), ("hidden", C.c_int),
        ("params", C.c_void_p), ("params_bf16", C.c_void_p),
    ]


class RoundTrace(C.Structure):
    _fields_ = [
        ("capacity", C.c_int), ("count", C.c_int), ("ms", C.c_void_p), ("nodes", C.c_void_p),
    ]


class Settings(C.Structure):
    _fields_ = [
        ("gpu_batch_size", C.c_int), ("num_streams", C.c_int), ("gpu_max_iters", C.c_int),
        ("gpu_eps", C.c_double), ("gpu_eps_decay", C.c_double), ("gpu_eps_min", C.c_double),
        ("integer_tol", C.c_double), ("abs_gap_tol", C.c_double), ("rel_gap_tol", C.c_double),
        ("algorithm", Algorithm),
        ("time_limit_seconds", C.c_double), ("natural_lower_bound", C.c_double),
        ("root_initial_point", C.c_void_p),
        ("branch_k", C.c_int), ("use_cuda_graph", C.c_int),
        ("scorer", C.c_void_p), ("autotune", C.c_int),
        ("device_frontier", C.c_int), ("incumbent_cutoff", C.c_int), ("frontier_capacity", C.c_int),
        ("frontier_slots", C.c_int), ("node_limit", C.c_int),
        ("trace", C.c_void_p),
    ]


class Result(C.Structure):
    _fields_ = [
        ("objective", C.c_double), ("dual_bound", C.c_double),
        ("nodes_processed", C.c_int), ("elapsed_seconds", C.c_double),
        ("reached_tolerance", C.c_int), ("reached_time_limit", C.c_int),
        ("has_incumbent", C.c_int), ("x", C.c_void_p), ("reached_node_limit", C.c_int),
        ("batches", C.c_int),
    ]


def default_settings() -> Settings:
    """create_default_settings() (gpuboscia.cuh:44-47, device_resident_solver.cuh:1004-1025)."""
    inf = float("inf")
    s = Settings()
    s.gpu_batch_size = 1024
    s.num_streams = 8
    s.gpu_max_iters = 20000
    s.gpu_eps = 1e-3
    s.gpu_eps_decay = 0.8
    s.gpu_eps_min = 1e-6
    s.integer_tol = 1e-6
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-2
    s.algorithm = Algorithm(ALG_DICG, LS_SECANT, 4, 1e-10, 1e-14, PRECISION_FP64)
    s.time_limit_seconds = inf
    s.natural_lower_bound = -inf
    s.root_initial_point = None
    s.branch_k = 3
    s.use_cuda_graph = 1
    s.scorer = None
    s.autotune = 1
    s.device_frontier = 0
    s.incumbent_cutoff = 0
    s.frontier_capacity = 0
    s.frontier_slots = 2
    s.node_limit = 0
    s.trace = None
    return s


# bytes of the library-owned scratch of gbx_relax_batch_static (GBX_STATIC_SCRATCH_BYTES)
STATIC_SCRATCH_BYTES = 32 << 20

# exported symbols of the CUDA library, as declared in include/gpuboscia_gb300.h
EXPORTED_SYMBOLS = (
    "gbx_abi_version", "gbx_last_error", "gbx_relax_workspace_bytes",
    "gbx_relax_batch", "gbx_relax_batch_static", "gbx_relax_autotune", "gbx_relax_set_launch_shape",
    "gbx_relax_set_oracle_warps", "gbx_relax_set_nodes_per_sm",
    "gbx_lmo_batch",
    "gbx_objective_gradient_batch", "gbx_objective_gradient_batch_f32",
    "gbx_node_feasible_batch",
    "gbx_default_settings", "gbx_solve",
    "gbx_read_mat", "gbx_read_dimacs",
    "gbx_scorer_param_count", "gbx_branch_features", "gbx_scorer_forward", "gbx_scorer_workspace_bytes",
    "gbx_scorer_gradient", "gbx_scorer_adam",
)

_lib = None


def load(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load the in-tree CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with gpuboscia_gb300.build.build() "
            "(the relaxation has no CPU fallback)")
    lib = C.CDLL(str(p))
    P = C.POINTER
    lib.gbx_abi_version.restype = C.c_int
    lib.gbx_last_error.restype = C.c_char_p
    lib.gbx_relax_workspace_bytes.restype = C.c_size_t
    lib.gbx_relax_workspace_bytes.argtypes = [P(Objective), P(LMO), P(Algorithm), C.c_int]
    lib.gbx_relax_batch.restype = C.c_int
    lib.gbx_relax_batch.argtypes = [P(Objective), P(LMO), P(Algorithm), P(NodeBatch),
                                    C.c_void_p, C.c_size_t, C.c_void_p]
    lib.gbx_relax_batch_static.restype = C.c_int
    lib.gbx_relax_batch_static.argtypes = [P(Objective), P(LMO), P(Algorithm), P(NodeBatch), C.c_void_p]
    lib.gbx_relax_autotune.restype = C.c_int
    lib.gbx_relax_autotune.argtypes = [P(Objective), P(LMO), P(Algorithm), P(NodeBatch), C.c_void_p, C.c_size_t,
                                       C.c_void_p, C.c_int, C.c_void_p]
    lib.gbx_relax_set_launch_shape.restype = C.c_int
    lib.gbx_relax_set_launch_shape.argtypes = [P(Objective), P(LMO), P(Algorithm), C.c_int, C.c_int]
    lib.gbx_relax_set_oracle_warps.restype = C.c_int
    lib.gbx_relax_set_oracle_warps.argtypes = [P(Objective), P(LMO), P(Algorithm), C.c_int]
    lib.gbx_relax_set_nodes_per_sm.restype = C.c_int
    lib.gbx_relax_set_nodes_per_sm.argtypes = [P(Objective), P(LMO), P(Algorithm), C.c_int]
    lib.gbx_lmo_batch.restype = C.c_int
    lib.gbx_lmo_batch.argtypes = [P(LMO), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gbx_objective_gradient_batch.restype = C.c_int
    lib.gbx_objective_gradient_batch.argtypes = [P(Objective), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                 C.c_void_p]
    lib.gbx_objective_gradient_batch_f32.restype = C.c_int
    lib.gbx_objective_gradient_batch_f32.argtypes = [P(Objective), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gbx_node_feasible_batch.restype = C.c_int
    lib.gbx_node_feasible_batch.argtypes = [P(LMO), C.c_int, C.c_void_p, C.c_void_p,
                                            C.c_void_p, C.c_void_p, C.c_void_p]
    lib.gbx_scorer_param_count.restype = C.c_int
    lib.gbx_scorer_param_count.argtypes = [C.c_int, C.c_int]
    lib.gbx_branch_features.restype = None
    lib.gbx_branch_features.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int,
                                        C.c_double, C.c_double, C.c_int, C.c_void_p, C.c_void_p]
    lib.gbx_read_mat.restype = C.c_int
    lib.gbx_read_mat.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p,
                                 C.c_size_t]
    lib.gbx_read_dimacs.restype = C.c_int
    lib.gbx_read_dimacs.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.c_void_p, C.c_size_t]
    lib.gbx_scorer_forward.restype = C.c_int
    lib.gbx_scorer_forward.argtypes = [P(Scorer), C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    lib.gbx_scorer_workspace_bytes.restype = C.c_size_t
    lib.gbx_scorer_workspace_bytes.argtypes = [P(Scorer), C.c_int]
    lib.gbx_scorer_gradient.restype = C.c_int
    lib.gbx_scorer_gradient.argtypes = [P(Scorer), C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p]
    lib.gbx_scorer_adam.restype = C.c_int
    lib.gbx_scorer_adam.argtypes = [P(Scorer), C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float,
                                    C.c_void_p]
    lib.gbx_default_settings.restype = None
    lib.gbx_default_settings.argtypes = [P(Settings)]
    lib.gbx_solve.restype = C.c_int
    lib.gbx_solve.argtypes = [P(Problem), P(Objective), P(LMO), P(Settings), P(Result)]
    if path is None:
        _lib = lib
    return lib


def check(lib: C.CDLL, rc: int, what: str) -> None:
    if rc != OK:
        msg = lib.gbx_last_error()
        raise RuntimeError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")
