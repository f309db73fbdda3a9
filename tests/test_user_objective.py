"""User-written device objectives -- the reference's extension point, a device
struct with n_vars, block_threads, shared_bytes, prepare_block, grad,
value_local and optionally quadratic_curvature_local -- run through a template
relaxation kernel compiled in the caller's nvcc translation unit
(include/gpuboscia/user_relax.cuh, brought in by gpuboscia.cuh).

CPU: the test program and the reference's own graph-isomorphism example
(examples/main.cu, with its GraphIsoObjective functor; skipped without the
reference tree) compile and link unchanged against the drop-in headers.
GPU: the test program's user objectives reach the same certified optima as the
built-in kinds (tests/cpp/user_objective_gpu.cu)."""
import pathlib
import subprocess

import pytest

from _refdata import reference_path

ROOT = pathlib.Path(__file__).resolve().parent.parent
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _nvcc(build, srcs, out, extra=()):
    lib = build.build()
    cuda = build._cuda_home()
    cmd = [str(cuda / "bin" / "nvcc"), "-std=c++17", "-O2", ARCH, "-I", str(ROOT / "include"), *extra, *map(str, srcs),
           "-o", str(out), "-L", str(lib.parent), "-lgpuboscia_gb300", "-Xlinker", "-rpath=" + str(lib.parent),
           "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    from gpuboscia_gb300 import build
    return _nvcc(build, [ROOT / "tests" / "cpp" / "user_objective_gpu.cu"],
                 tmp_path_factory.mktemp("userobj") / "user_objective_gpu")


def test_user_objective_program_compiles(exe):
    assert exe.exists()


EXAMPLE = reference_path("examples", "main.cu")


@pytest.mark.skipif(not EXAMPLE.is_file(), reason="reference tree not present")
def test_reference_graph_isomorphism_example_compiles_unchanged(tmp_path):
    from gpuboscia_gb300 import build
    root = EXAMPLE.parent.parent
    _nvcc(build, [EXAMPLE], tmp_path / "graph_iso",
          ["-I", str(EXAMPLE.parent), f'-DGPUBOSCIA_SOURCE_DIR="{root}"', "-lz"])


@pytest.mark.gpu
def test_user_objectives_reach_the_built_in_optima(cuda_lib, exe):
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout
