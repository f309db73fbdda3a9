"""Failure surfacing without a GPU fault: on a machine where every CUDA call
fails (this CPU-only container), the C ABI returns GBX_ERR_CUDA with CUDA's
message from both frontiers and stays usable afterwards, host-only calls keep
working, and the C++ drop-in turns the failure into std::runtime_error while a
bad setting is still std::invalid_argument. Skipped where a GPU is usable."""
import ctypes as C
import pathlib
import subprocess

import numpy as np
import pytest

from gpuboscia_gb300 import _abi as A
from gpuboscia_gb300 import api, build

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _gpu_usable():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


pytestmark = pytest.mark.skipif(_gpu_usable(), reason="needs a machine where CUDA calls fail")


def test_c_abi_reports_cuda_errors_and_stays_usable():
    build.build()
    lib = A.load()
    keep = api._Keep()
    n = 4
    obj = api.DenseQuadraticObjective(np.eye(n)).to_c("host", keep)
    lmo = api.BoxLMO().to_c(n, "host", keep)
    lb, ub = np.zeros(n), np.ones(n)
    iv = np.arange(n, dtype=np.int32)
    prob = A.Problem(n, lb.ctypes.data, ub.ctypes.data, iv.ctypes.data, n)
    for _ in range(2):   # a second round: the first failure left nothing broken
        for dev in (0, 1):
            s = A.default_settings()
            s.device_frontier = dev
            res = A.Result()
            rc = lib.gbx_solve(C.byref(prob), C.byref(obj), C.byref(lmo), C.byref(s), C.byref(res))
            assert rc == A.ERR_CUDA, (dev, rc)
            assert b"CUDA" in lib.gbx_last_error() or b"driver" in lib.gbx_last_error()
            with pytest.raises(RuntimeError):
                A.check(lib, rc, "gbx_solve")
        # host-only entry points are unaffected
        assert lib.gbx_relax_workspace_bytes(C.byref(obj), C.byref(lmo), C.byref(s.algorithm), 8) > 0
        assert lib.gbx_abi_version() == 4


def test_cpp_dropin_throws_runtime_error(tmp_path):
    lib = build.build()
    cuda = build._cuda_home()
    exe = tmp_path / "no_gpu_errors"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I",
                    str(cuda / "include"), str(ROOT / "tests" / "cpp" / "no_gpu_errors.cpp"), "-o", str(exe),
                    "-L", str(lib.parent), "-lgpuboscia_gb300", "-Wl,-rpath," + str(lib.parent),
                    "-L", str(cuda / "lib64"), "-lcudart", "-Wl,-rpath," + str(cuda / "lib64"), "-lpthread"],
                   check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    assert lines[0].startswith("frontier=0 runtime_error") and lines[1].startswith("frontier=1 runtime_error")
    assert lines[2] == "bad settings invalid_argument"
