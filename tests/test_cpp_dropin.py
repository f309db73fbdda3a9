"""The C++ drop-in headers (gpuboscia::solve over the built-in objective / LMO
types, as a reference program would call them) compiled with the host
compiler and linked against the in-tree library: the reference's
examples/minimal.cu answer and a graph pair, on the host and the device
frontier (tests/cpp/minimal_gpu.cpp); and the host engine's scheduling order
(tests/cpp/scheduling_gpu.cpp)."""
import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _compile_all(cmds):
    """Runs the compile commands side by side (each nvcc front end is single
    threaded) and fails on the first that does not succeed."""
    import concurrent.futures as cf
    with cf.ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for r in ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), cmds):
            assert r.returncode == 0, r.stderr[-3000:]


def _program(tmp_path_factory, name):
    from gpuboscia_gb300 import build
    lib = build.build()
    cuda = build._cuda_home()
    out = tmp_path_factory.mktemp("cppgpu") / name
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I", str(cuda / "include"),
           str(ROOT / "tests" / "cpp" / f"{name}.cpp"), "-o", str(out),
           "-L", str(lib.parent), "-lgpuboscia_gb300", "-Wl,-rpath," + str(lib.parent),
           "-L", str(cuda / "lib64"), "-lcudart", "-Wl,-rpath," + str(cuda / "lib64"), "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    return _program(tmp_path_factory, "minimal_gpu")


@pytest.fixture(scope="module")
def scheduling_exe(tmp_path_factory):
    return _program(tmp_path_factory, "scheduling_gpu")


def test_dropin_program_compiles_and_links(exe):
    assert exe.exists()


@pytest.mark.gpu
def test_dropin_program_runs(cuda_lib, exe):
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout


def test_scheduling_program_compiles_and_links(scheduling_exe):
    assert scheduling_exe.exists()


@pytest.mark.gpu
def test_scheduling_order_as_the_reference_asserts(cuda_lib, scheduling_exe):
    """tests/test_pipeline.cu:723-836: a completed slot is refilled before its
    batch is post-processed, and with an empty frontier the children are
    dispatched before the root's post-processing (root branched once, optimum
    and bound kept)."""
    r = subprocess.run([str(scheduling_exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 failed" in r.stdout


@pytest.mark.parametrize("where,name", [("examples", "minimal.cu"), ("tests", "test_root_initial_point.cu")])
def test_reference_example_compiles_and_links_unchanged(tmp_path, where, name):
    """The reference's own examples/minimal.cu and tests/test_root_initial_point.cu
    (a device objective with the optional grad_multiblock member, the
    reference's DRS_CUDA_CHECK and DRS_HAS_MULTIBLOCK_ATOMICS), unchanged,
    compile with nvcc against the drop-in headers and link against the
    library (minimal.cu's model runs on the GPU in tests/cpp/minimal_gpu.cpp).
    examples/main.cu is compiled and run in test_user_objective.py;
    examples/sparse_sharpe.cu defines its own device LMO, which the
    precompiled kernels do not take."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from _refdata import reference_path
    from gpuboscia_gb300 import build
    src = reference_path(where, name)
    example = name.split(".")[0]
    if not src.is_file():
        pytest.skip("reference tree not available")
    lib = build.build()
    cuda = build._cuda_home()
    out = tmp_path / example
    subprocess.run([str(cuda / "bin" / "nvcc"), "-std=c++17", "-O1", build.ARCH, "-I", str(ROOT / "include"),
                    str(src), "-o", str(out), "-L", str(lib.parent), "-lgpuboscia_gb300"],
                   check=True, capture_output=True, text=True)
    assert out.exists()


def test_reference_consumer_programs_build_unchanged(tmp_path):
    """The reference's package-consumer tests (tests/consumer and
    tests/consumer_cuda of the reference), unchanged, against the drop-in
    headers: the two host translation units build with g++ -Wall -Werror and
    the program exits 0 (branch_pow2, quadratic_exact_step and gap_absolute
    from both units); examples/minimal.cu and consumer_cuda/second.cu build
    together with nvcc in separable compilation and link against the library
    (no duplicate definitions across the units)."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from _refdata import reference_path
    from gpuboscia_gb300 import build
    host = [reference_path("tests", "consumer", f) for f in ("main.cpp", "second.cpp")]
    cuda_units = [reference_path("examples", "minimal.cu"), reference_path("tests", "consumer_cuda", "second.cu")]
    if not all(p.is_file() for p in host + cuda_units):
        pytest.skip("reference tree not available")
    out = tmp_path / "consumer"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-I", str(ROOT / "include")] + [str(p) for p in host]
                   + ["-o", str(out)], check=True)
    assert subprocess.run([str(out)]).returncode == 0
    lib = build.build()
    cuda = build._cuda_home()
    out2 = tmp_path / "consumer_cuda"
    subprocess.run([str(cuda / "bin" / "nvcc"), "-std=c++17", "-O1", "-rdc=true", build.ARCH, "-I", str(ROOT / "include")]
                   + [str(p) for p in cuda_units] + ["-o", str(out2), "-L", str(lib.parent), "-lgpuboscia_gb300"],
                   check=True, capture_output=True, text=True)
    assert out2.exists()


@pytest.fixture(scope="module")
def differential_programs(tmp_path_factory):
    """The differential drivers of tests/cpp, each built against the
    reference's headers (nvcc) and against the drop-in headers and library,
    all six compiles side by side. Skips without the reference tree."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from _refdata import reference_path
    from gpuboscia_gb300 import build
    ref_include = reference_path("include")
    if not (ref_include / "gpuboscia" / "device_resident_solver.cuh").is_file():
        pytest.skip("reference tree not available")
    lib = build.build()
    cuda = build._cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    out = tmp_path_factory.mktemp("differential")
    link = ["-L", str(lib.parent), "-lgpuboscia_gb300", "-L", str(cuda / "lib64"), "-lcudart", "-lpthread"]
    rpath = ["-Wl,-rpath," + str(lib.parent), "-Wl,-rpath," + str(cuda / "lib64")]
    cmds, exes = [], {}
    for name, ours_with_nvcc in (("solver_api", False), ("config_checks", False), ("solve_checks", True)):
        src = ROOT / "tests" / "cpp" / f"{name}.cpp"
        cu = out / f"{name}.cu"
        cu.write_text(src.read_text())
        exes[name] = (out / f"{name}_ours", out / f"{name}_ref")
        if ours_with_nvcc:   # a device objective of its own: nvcc on both sides
            cmds.append([nvcc, "-std=c++17", "-O1", build.ARCH, "-I", str(ROOT / "include"), str(cu), "-o",
                         str(exes[name][0]), "-L", str(lib.parent), "-lgpuboscia_gb300", "-Xlinker", "-rpath",
                         "-Xlinker", str(lib.parent)])
        else:
            cmds.append(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I",
                         str(cuda / "include"), str(src), "-o", str(exes[name][0])] + link + rpath)
        cmds.append([nvcc, "-std=c++17", "-O1", build.ARCH, "-I", str(ref_include), str(cu), "-o",
                     str(exes[name][1])])
    _compile_all(cmds)
    return exes


def _both_outputs(exes):
    return [subprocess.run([str(e)], capture_output=True, text=True, check=True).stdout for e in exes]


def test_solver_api_surface_matches_the_reference(differential_programs):
    """tests/cpp/solver_api.cpp uses every public member of the reference's
    DeviceResidentHybridSolver (both constructor forms, push, the progress and
    scheduling callbacks, solve, every accessor) and both solve entry points
    with the reference's own types. It compiles and links against the
    reference's headers (nvcc) and against the drop-in headers and library
    (g++ -Wall -Werror)."""
    ours, ref = differential_programs["solver_api"]
    assert ours.exists() and ref.exists()


def test_configuration_checks_match_the_reference(differential_programs):
    """The solver constructor's checks on its configuration (counts,
    integer indices, tolerances, time limit, objective size), which run
    before any CUDA call: tests/cpp/config_checks.cpp builds the solver with
    20 bad configurations against the reference's headers (nvcc) and against
    the drop-in (g++), and the exception type, message and the order in which
    two failing checks are reported are the same."""
    a, b = _both_outputs(differential_programs["config_checks"])
    assert a.count("\n") == 20 and "accepted" not in a
    assert a == b


def test_solve_argument_checks_match_the_reference(differential_programs):
    """gpuboscia::solve's checks (algorithm and line-search combinations,
    quadratic-exact without curvature support, the root point, the solver's
    configuration) and the order in which they are reported:
    tests/cpp/solve_checks.cpp, compiled with nvcc against the reference's
    headers and against the drop-in, prints the same 14 lines."""
    a, b = _both_outputs(differential_programs["solve_checks"])
    assert a.count("\n") == 14 and "returned" not in a
    assert a == b
