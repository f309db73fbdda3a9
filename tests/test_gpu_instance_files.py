"""A graph-matching instance read from a MAT file (examples/main.cu's flow:
A from the file, B = A under a seeded permutation, optimum 0) solved on the
GPU with the host and the device frontier."""
import numpy as np
import pytest

from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, instances
from test_instance_files import _mat_file

pytestmark = pytest.mark.gpu


def _grid(rows, cols):
    m = rows * cols
    G = np.zeros((m, m), np.uint8)
    for r in range(rows):
        for c in range(cols):
            v = r * cols + c
            if c + 1 < cols:
                G[v, v + 1] = G[v + 1, v] = 1
            if r + 1 < rows:
                G[v, v + cols] = G[v + cols, v] = 1
    return G


@pytest.mark.parametrize("device_frontier,precision", [(0, A.PRECISION_FP64), (1, A.PRECISION_MIXED)])
def test_lattice_file_instance_is_solved(cuda_lib, tmp_path, device_frontier, precision):
    f = tmp_path / "lattice_4x5.mat"
    f.write_bytes(_mat_file("A", _grid(4, 5), 2, "B", 9))
    inst = instances.graph_matching_from_file(f, seed=3)
    s = inst.settings
    s.algorithm = A.ALG_DICG
    s.line_search = A.LS_QUADRATIC_EXACT
    s.gpu_batch_size = 64
    s.gpu_max_iters = 1000
    s.precision = precision
    s.device_frontier = device_frontier
    s.time_limit_seconds = 120
    r = api.solve(inst.problem, inst.objective, inst.lmo, s)
    assert r.objective <= 1e-9
    m = inst.lmo.order
    X = r.x.reshape(m, m)
    assert np.array_equal(inst.objective.A @ X, X @ inst.objective.B)
