"""Instance files (gbx_read_mat / gbx_read_dimacs, examples/main.cu:41-129):
MATLAB v5 matrices written by scipy and by hand (zlib streams with stored,
fixed-Huffman and dynamic-Huffman blocks), the reference's own instance files
when the reference tree is present, DIMACS edge lists, and the error paths."""
import os
import pathlib
import struct
import zlib

import numpy as np
import pytest

from gpuboscia_gb300 import instances
from _refdata import reference_path

REF = reference_path("test_instances")


def _element(t, payload):
    pad = (-len(payload)) % 8
    return struct.pack("<II", t, len(payload)) + payload + b"\0" * pad


def _mat_file(name, M, dtype_code, fmt, compress_level=None):
    """A MAT v5 file with one real matrix, written by hand (column-major)."""
    r, c = M.shape
    flags = _element(6, struct.pack("<II", 6, 0))            # mxDOUBLE_CLASS
    dims = _element(5, struct.pack("<ii", r, c))
    nm = _element(1, name.encode())
    data = _element(dtype_code, struct.pack("<" + fmt * (r * c), *M.T.ravel().tolist()))
    matrix = _element(14, flags + dims + nm + data)
    header = b"MATLAB 5.0 MAT-file written by a test".ljust(116, b" ") + b"\0" * 8 + struct.pack("<H", 0x0100) + b"IM"
    if compress_level is None:
        return header + matrix
    z = zlib.compress(matrix, compress_level)
    return header + struct.pack("<II", 15, len(z)) + z


@pytest.mark.parametrize("level", [None, 0, 1, 9])
@pytest.mark.parametrize("code,fmt,dtype", [(9, "d", float), (2, "B", np.uint8), (3, "h", np.int16),
                                            (7, "f", np.float32)])
def test_handwritten_mat(tmp_path, level, code, fmt, dtype):
    rng = np.random.default_rng(7)
    M = rng.integers(0, 200, size=(37, 23)).astype(dtype)
    f = tmp_path / "m.mat"
    f.write_bytes(_mat_file("A", M, code, fmt, level))
    assert np.array_equal(instances.load_mat(f), M.astype(float))


def test_large_dynamic_block(tmp_path):
    """A long stream with back-references far into the window."""
    rng = np.random.default_rng(1)
    M = (rng.random((300, 300)) < 0.05).astype(float)
    f = tmp_path / "big.mat"
    f.write_bytes(_mat_file("A", M, 9, "d", 6))
    assert np.array_equal(instances.load_mat(f), M)


def test_scipy_written(tmp_path):
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(3)
    A = (rng.random((30, 30)) < 0.3).astype(float)
    B = rng.normal(size=(4, 9))
    for comp in (False, True):
        f = tmp_path / f"s{int(comp)}.mat"
        sio.savemat(f, {"B": B, "A": A, "note": "text"}, do_compression=comp)
        assert np.array_equal(instances.load_mat(f, "A"), A)
        assert np.array_equal(instances.load_mat(f, "B"), B)
        with pytest.raises(ValueError, match="no real matrix named 'C'"):
            instances.load_mat(f, "C")


def test_errors(tmp_path):
    with pytest.raises(ValueError, match="cannot open"):
        instances.load_mat(tmp_path / "missing.mat")
    bad = tmp_path / "bad.mat"
    bad.write_bytes(b"x" * 200)
    with pytest.raises(RuntimeError, match="MAT v5"):
        instances.load_mat(bad)
    M = np.eye(4)
    raw = bytearray(_mat_file("A", M, 9, "d", 9))
    raw[-6] ^= 0xFF           # corrupt the compressed stream
    (tmp_path / "corrupt.mat").write_bytes(bytes(raw))
    with pytest.raises(RuntimeError):
        instances.load_mat(tmp_path / "corrupt.mat")
    d = tmp_path / "bad.dimacs"
    d.write_text("p edge 3 2\ne 1 2\n")
    with pytest.raises(RuntimeError, match="edge count"):
        instances.load_dimacs(d)
    d.write_text("p edge 3 1\ne 1 4\n")
    with pytest.raises(RuntimeError, match="invalid DIMACS edge"):
        instances.load_dimacs(d)


def test_dimacs(tmp_path):
    f = tmp_path / "g.dimacs"
    f.write_text("c a comment\np edge 5 4\ne 1 2\ne 2 3\ne 3 4\ne 4 5\n")
    A = instances.load_dimacs(f)
    want = np.zeros((5, 5))
    for u in range(4):
        want[u, u + 1] = want[u + 1, u] = 1
    assert np.array_equal(A, want)


def test_instance_from_file_has_its_solution(tmp_path):
    rng = np.random.default_rng(5)
    A = np.triu((rng.random((12, 12)) < 0.4).astype(float), 1)
    A = A + A.T
    f = tmp_path / "g.mat"
    f.write_bytes(_mat_file("A", A.astype(np.uint8), 2, "B", 9))
    inst = instances.graph_matching_from_file(f, seed=11)
    Aa, Bb = inst.objective.A, inst.objective.B
    X = inst.solution.reshape(12, 12)
    assert np.array_equal(Aa @ X, X @ Bb)
    assert inst.lmo.order == 12 and inst.problem.n_vars == 144


@pytest.mark.skipif(not REF.is_dir(), reason="reference instance files not present")
def test_reference_instance_files():
    """Every MAT instance the reference ships (examples/main.cu reads them)
    decodes to the same matrix as scipy's reader; every DIMACS file parses to a
    symmetric 0/1 adjacency with the edge count of its problem line."""
    sio = pytest.importorskip("scipy.io")
    mats = sorted(REF.glob("*.mat"))
    assert mats
    for f in mats:
        A = instances.load_mat(f)
        S = sio.loadmat(f)["A"]
        S = S.toarray() if hasattr(S, "toarray") else np.asarray(S, float)
        assert np.array_equal(A, S), f.name
        assert A.shape[0] == A.shape[1] and np.array_equal(A, A.T), f.name
    for f in sorted(REF.glob("*.dimacs")):
        A = instances.load_dimacs(f)
        m = int(next(line for line in f.read_text().splitlines() if line.startswith("p")).split()[3])
        assert np.array_equal(A, A.T) and int(A.sum()) == 2 * m, f.name


DATASETS = REF.parent / "DataSets"


@pytest.mark.skipif(not DATASETS.is_dir(), reason="reference data sets not present")
def test_reference_datasets():
    """The return matrices the sparse-Sharpe example reads (examples/sparse_sharpe.cu
    load_mat, variable `data`) decode to the same values as scipy's reader."""
    sio = pytest.importorskip("scipy.io")
    mats = sorted(DATASETS.glob("*.mat"))
    assert mats
    for f in mats:
        D = instances.load_mat(f, "data")
        S = np.asarray(sio.loadmat(f)["data"], float)
        assert D.shape == S.shape and np.array_equal(D, S), f.name


@pytest.mark.skipif(not REF.is_dir(), reason="reference instance files not present")
@pytest.mark.parametrize("name", ["latin_3_9.mat", "paley_power_9.mat", "paley_prime_13.mat"])
def test_reference_instance_is_solved(name):
    """examples/main.cu's flow on the reference's own graphs (B = A under a
    seeded permutation): the oracle B&B and the device frontier's restated
    search find an isomorphism (objective 0) with a closed certified gap."""
    import sys
    sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent))
    import _frontier_oracle as F
    import _oracle as O
    from gpuboscia_gb300 import _abi as A
    inst = instances.graph_matching_from_file(REF / name, seed=3)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 16
    s.num_streams = 1
    s.gpu_max_iters = 500
    s.abs_gap_tol = 1e-6
    s.rel_gap_tol = 1e-6
    s.time_limit_seconds = 60
    o = O.solve(inst.problem, inst.objective, inst.lmo, s)
    assert o.objective <= 1e-9 and o.reached_tolerance and not o.reached_time_limit
    f = F.solve(inst.problem, inst.objective, inst.lmo, s, 2)
    assert f["objective"] <= 1e-9
    m = inst.lmo.order
    for x in (o.x, f["x"]):
        X = np.asarray(x).reshape(m, m)
        assert np.array_equal(X.sum(0), np.ones(m)) and np.array_equal(X.sum(1), np.ones(m))
        assert np.array_equal(inst.objective.A @ X, X @ inst.objective.B)
