"""The C++ drop-in headers on the CPU: the reference's test_cpu.cpp assertions
(tests/cpp/test_host.cpp), the host rules against the reference fixtures, and,
where the reference tree is present, live and differential checks against the
reference's own CPU functions and headers (random cases and operation scripts
through the same drivers compiled against each)."""
import json
import math
import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = json.loads((ROOT / "tests" / "golden" / "reference_cpu.json").read_text())


def _cuda_include():
    from gpuboscia_gb300 import build
    return str(build._cuda_home() / "include")


CUDA_INCLUDE = _cuda_include()


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp") / "test_host"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "test_host.cpp"), "-o", str(out)], check=True)
    return out


def test_header_unit_tests(exe):
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    assert "0 failed" in r.stdout


def _table(exe, lines):
    r = subprocess.run([str(exe), "table"], input="\n".join(lines) + "\n", capture_output=True, text=True,
                       check=True)
    return r.stdout.split("\n")


def _eq(a, b):
    return (math.isnan(a) and math.isnan(b)) or a == b


def test_host_rules_match_reference_fixture(exe):
    rows = GOLDEN["gaps"]
    out = _table(exe, [f"gap {b!r} {i!r} 0.01 0.01" for b, i, *_ in rows]
                 + [f"gap {b!r} {i!r} 0.0 0.105" for b, i, *_ in rows])
    for k, (b, i, ga, gr, t1, t2) in enumerate(rows):
        a, r, w = out[k].split()
        assert _eq(float(a), ga) and _eq(float(r), gr) and int(w) == t1, (b, i)
        assert int(out[len(rows) + k].split()[2]) == t2
    out = _table(exe, [f"cert {a!r} {b!r} {c!r}" for a, b, c, _ in GOLDEN["certified"]])
    for k, (*_, e) in enumerate(GOLDEN["certified"]):
        assert float(out[k]) == e
    out = _table(exe, [f"depth {d}" for d, _ in GOLDEN["depth_tol"]])
    for k, (_, e) in enumerate(GOLDEN["depth_tol"]):
        assert float(out[k]) == e
    out = _table(exe, [f"quad {g!r} {c!r} {m!r}" for g, c, m, _ in GOLDEN["quad_step"]])
    for k, (*_, e) in enumerate(GOLDEN["quad_step"]):
        assert float(out[k]) == e


def test_host_rules_live_against_the_reference(exe):
    """gap_utils.h (absolute and relative gap, the tolerance test, the
    certified Frank-Wolfe bound, the depth schedule) and the closed-form
    quadratic-exact step against the reference's own functions (oracle/_ref)
    on random values mixed with zeros, signed infinities and NaN."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np
    import _oracle as O
    R = O.ref()
    if R is None:
        pytest.skip("reference tree not available at build time")
    rng = np.random.default_rng(31)
    special = [0.0, -0.0, 1.0, -1.0, 1e-300, -1e-300, 1e300, math.inf, -math.inf, math.nan]

    def value():
        return float(rng.choice(special)) if rng.random() < 0.3 else float(rng.normal() * 10.0 ** rng.integers(-8, 9))

    pairs = [(value(), value()) for _ in range(400)]
    tols = [(float(rng.choice([0.0, 1e-6, 0.01])), float(rng.choice([0.0, 1e-6, 0.105]))) for _ in pairs]
    out = _table(exe, [f"gap {b!r} {i!r} {ta!r} {tr!r}" for (b, i), (ta, tr) in zip(pairs, tols)])
    for k, ((b, i), (ta, tr)) in enumerate(zip(pairs, tols)):
        a, r, w = out[k].split()
        assert _eq(float(a), R.ref_gap_absolute(b, i)), (b, i)
        assert _eq(float(r), R.ref_gap_relative(b, i)), (b, i)
        assert int(w) == R.ref_gap_within_tolerance(b, i, ta, tr), (b, i, ta, tr)
    triples = [(value(), value(), value()) for _ in range(300)]
    out = _table(exe, [f"cert {a!r} {b!r} {c!r}" for a, b, c in triples])
    for k, (a, b, c) in enumerate(triples):
        assert _eq(float(out[k]), R.ref_certified_fw_lower_bound(a, b, c)), (a, b, c)
    depths = [int(d) for d in rng.integers(-2, 2000, 100)]
    out = _table(exe, [f"depth {d}" for d in depths])
    for k, d in enumerate(depths):
        assert float(out[k]) == R.ref_depth_dependent_tolerance(1e-3, 0.8, 1e-6, d), d
    out = _table(exe, [f"quad {g!r} {c!r} {m!r}" for g, c, m in triples])
    for k, (g, c, m) in enumerate(triples):
        assert _eq(float(out[k]), R.ref_quadratic_exact_step(g, c, m)), (g, c, m)


def test_branch_pow2_live_against_the_reference(exe):
    """branching.h's branch_pow2 (the reference's branching.h:80-118) against
    the reference's own function on random nodes: k from 0 to 4, iterates
    with ties in fractionality, near-integral values around the tolerance,
    bounds already narrowed, and more than 16 candidates (where std::sort's
    order among equal fractionalities is no longer the index order); the
    children (count, order, bounds) are equal."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np
    import _oracle as O
    R = O.ref()
    if R is None:
        pytest.skip("reference tree not available at build time")
    rng = np.random.default_rng(37)
    lines, want = [], []
    for _ in range(300):
        n = int(rng.integers(1, 40))
        k = int(rng.integers(0, 5))
        tol = float(rng.choice([1e-6, 1e-3]))
        ints = sorted(rng.choice(n, int(rng.integers(0, n + 1)), replace=False).tolist())
        lb = rng.integers(-2, 2, n).astype(float)
        ub = lb + rng.integers(0, 4, n)
        x = lb + (ub - lb) * rng.integers(0, 9, n) / 8.0
        near = rng.random(n) < 0.2
        x[near] = np.round(x[near]) + rng.choice([-1, 1], near.sum()) * tol * rng.choice([0.5, 2.0], near.sum())
        iv = np.array(ints, dtype=np.int32)
        olb, oub = np.zeros(16 * n), np.zeros(16 * n)
        cnt = R.ref_branch_pow2(n, lb.ctypes.data, ub.ctypes.data, x.ctypes.data, iv.ctypes.data if ints else None,
                                len(ints), k, tol, olb.ctypes.data, oub.ctypes.data)
        kids = [v for c in range(cnt) for v in list(olb[c * n:(c + 1) * n]) + list(oub[c * n:(c + 1) * n])]
        lines.append(f"branch {n} {k} {tol!r} {len(ints)} {' '.join(map(str, ints))} {_fmt(lb)} {_fmt(ub)} {_fmt(x)}")
        want.append([float(cnt)] + kids)
    out = _table(exe, lines)
    for i, w in enumerate(want):
        got = [float(t) for t in out[i].split()]
        assert got == w, (lines[i], got, w)


def test_queue_and_bound_set_match_the_reference_implementation(tmp_path):
    """concurrent_queue.h here against the reference's own header: one script
    of random operations (pushes with few distinct bounds, so ties are the
    rule; pop_batch and pop_full_batch with cutoffs that drop part of the
    frontier and return short batches; discard_children; best bounds and the
    bound set's inserts and erasures) run through the same driver compiled
    against each. The outputs (which nodes leave in which order) are equal."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    import random
    from _refdata import reference_path
    ref_include = reference_path("include")
    if not (ref_include / "gpuboscia" / "concurrent_queue.h").is_file():
        pytest.skip("reference tree not available")
    src = ROOT / "tests" / "cpp" / "queue_ops.cpp"
    exes = []
    for name, inc in (("ours", ROOT / "include"), ("ref", ref_include)):
        out = tmp_path / name
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(inc), str(src), "-o", str(out)], check=True)
        exes.append(out)
    rng = random.Random(43)
    ops, next_id, bounds_held = [], 0, []
    for _ in range(6000):
        r = rng.random()
        if r < 0.45:
            ops.append(f"push {next_id} {rng.randrange(0, 40)} {rng.choice([-3.0, -2.5, -2.0, -1.0, 0.0, 0.5])!r}")
            next_id += 1
        elif r < 0.6:
            ops.append(f"pop {rng.randrange(0, 9)} {rng.choice([-2.0, 0.0, 0.5, 1e300])!r}")
        elif r < 0.72:
            ops.append(f"full {rng.randrange(1, 9)} {rng.choice([-2.0, 0.0, 0.5, 1e300])!r}")
        elif r < 0.76:
            ops.append(f"discard {rng.randrange(0, 40)}")
        elif r < 0.82:
            ops.append(f"best {rng.choice([-2.0, 0.5, 1e300])!r}")
        elif r < 0.92:
            b = rng.choice([-3.0, -2.0, 0.0, 1.5])
            bounds_held.append(b)
            ops.append(f"bins {b!r}")
        elif r < 0.97:
            ops.append(f"berase {rng.choice(bounds_held or [0.0])!r}")
        else:
            ops.append(f"bbest {rng.choice([-2.5, 0.0, 1e300])!r}")
    script = "\n".join(ops) + "\n"
    ours, ref = (subprocess.run([str(e)], input=script, capture_output=True, text=True, check=True).stdout
                 for e in exes)
    assert ours.count("\n") > 1500
    assert ours == ref


def test_incumbent_and_root_point_checks_match_the_reference_implementation(tmp_path):
    """atomic_incumbent.h, tree.h's validate_root_initial_point and bnb.h's
    feasibility predicates here against the reference's headers: one random
    script (incumbent updates with ties, NaN and infinities; root points for
    box, bounded and equality simplices, a caller's validator and an LMO
    without a point check, with wrong lengths, bad tolerances, non-finite
    entries and bound violations; integer and node feasibility with indices
    out of range, NaN and values at the tolerance) run through the same driver compiled against each (the reference's
    lmo.cuh through nvcc). The outputs, messages included, are equal."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    import random
    from _refdata import reference_path
    from gpuboscia_gb300 import build
    ref_include = reference_path("include")
    if not (ref_include / "gpuboscia" / "tree.h").is_file():
        pytest.skip("reference tree not available")
    src = ROOT / "tests" / "cpp" / "root_point_ops.cpp"
    ours, ref = tmp_path / "ours", tmp_path / "ref"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(src), "-o", str(ours)], check=True)
    cu = tmp_path / "root_point_ops.cu"
    cu.write_text(src.read_text())
    subprocess.run([str(build._cuda_home() / "bin" / "nvcc"), "-std=c++17", "-O1", "-I", str(ref_include), str(cu),
                    "-o", str(ref)], check=True)
    rng = random.Random(47)
    vals = [0.0, 0.25, 0.5, 1.0, 2.0, -1.0, float("nan"), float("inf"), -float("inf"), 1e-10, -1e-10]
    lines = []
    for _ in range(3000):
        if rng.random() < 0.3:
            lines.append(f"inc {rng.choice(vals + [3.0, 3.0, 1.5])!r}")
            continue
        kind = rng.choice(["box", "simplex", "eqsimplex", "accept", "reject", "none"])
        n = rng.randrange(1, 6)
        m = n if rng.random() < 0.85 else rng.choice([0, n + 1, max(0, n - 1)])
        tol = rng.choice([1e-9, 0.0, 1e-3, -1.0, float("nan"), float("inf")])
        lb = [rng.choice([0.0, 0.0, -1.0, float("nan")]) for _ in range(n)]
        ub = [rng.choice([1.0, 1.0, 2.0, -2.0, float("nan")]) for _ in range(n)]
        x = [rng.choice(vals) for _ in range(m)]
        head = f"root {kind}" + (f" {rng.choice([1.0, 1.5, 2.0])!r}" if "simplex" in kind else "")
        lines.append(f"{head} {n} {m} {tol!r} " + " ".join(repr(v) for v in lb + ub + x))
    for _ in range(2000):
        n = rng.randrange(1, 7)
        ints = [rng.randrange(-1, n + 1) for _ in range(rng.randrange(0, n + 1))]
        tol = rng.choice([1e-9, 1e-6, 0.0, 0.3])
        a = [rng.choice([0.0, 0.5, 1.0, 1e-7, 1.0 - 1e-7, 2.9999999999, float("nan"), -0.25]) for _ in range(n)]
        tail = " ".join(map(str, ints))
        if rng.random() < 0.5:
            lines.append(f"intfeas {n} {len(ints)} {tol!r} " + " ".join(repr(v) for v in a) + " " + tail)
        else:
            b = [v + rng.choice([0.0, 1.0, -1e-10, 0.5, -0.5]) for v in a]
            lines.append(f"nodefeas {n} {len(ints)} {tol!r} " + " ".join(repr(v) for v in a + b) + " " + tail)
    script = "\n".join(lines) + "\n"
    a, b = (subprocess.run([str(e)], input=script, capture_output=True, text=True, check=True).stdout
            for e in (ours, ref))
    assert a.count("\n") == len(lines)
    assert "ok" in a and "violates the LMO" in a and "dimensions or tolerance" in a and "requires LMO" in a
    assert a == b


def test_reference_root_point_test_compiles_and_passes_unchanged(tmp_path):
    """The reference's own CPU test of the root-point checks
    (tests/test_root_initial_point.cpp of the reference), compiled unchanged
    against the drop-in headers with g++: it accepts and rejects the same
    points and prints its success line."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from _refdata import reference_path
    src = reference_path("tests", "test_root_initial_point.cpp")
    if not src.is_file():
        pytest.skip("reference tree not available")
    exe = tmp_path / "root_point"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Root initial-point validation passed" in r.stdout


def test_interface_defaults_match_the_reference(tmp_path):
    """Settings, Result, DeviceResidentConfig and LineSearchOptions defaults,
    the enums' values and name strings, and the scheduling event types: one
    driver (tests/cpp/defaults_dump.cpp) naming only the reference's fields,
    compiled against the drop-in headers with g++ and against the reference's
    gpuboscia.cuh with nvcc, prints the same lines."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    from _refdata import reference_path
    from gpuboscia_gb300 import build
    ref_include = reference_path("include")
    if not (ref_include / "gpuboscia" / "gpuboscia.cuh").is_file():
        pytest.skip("reference tree not available")
    src = ROOT / "tests" / "cpp" / "defaults_dump.cpp"
    ours, ref = tmp_path / "ours", tmp_path / "ref"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I", CUDA_INCLUDE,
                    str(src), "-o", str(ours)], check=True)
    cu = tmp_path / "defaults_dump.cu"
    cu.write_text(src.read_text())
    subprocess.run([str(build._cuda_home() / "bin" / "nvcc"), "-std=c++17", "-O1", "-I", str(ref_include), str(cu),
                    "-o", str(ref)], check=True)
    a, b = (subprocess.run([str(e)], capture_output=True, text=True, check=True).stdout for e in (ours, ref))
    assert a.count("\n") >= 40
    assert a == b


def test_dicg_helpers_match_the_reference_implementation(tmp_path):
    """lmo_dicg.h's free helpers here against the reference's lmo_dicg.h:
    the tolerance test, the simplex linear and in-face feasibility checks,
    the box and bounded-simplex in-face oracles and DICG maximum steps (with
    and without full mass), on 3,000 random cases with values at the
    tolerances and signed zeros, through tests/cpp/dicg_helpers.cpp compiled
    against each. The outputs are equal."""
    import sys
    import random
    sys.path.insert(0, str(ROOT / "tests"))
    from _refdata import reference_path
    ref_include = reference_path("include")
    if not (ref_include / "gpuboscia" / "lmo_dicg.h").is_file():
        pytest.skip("reference tree not available")
    src = ROOT / "tests" / "cpp" / "dicg_helpers.cpp"
    exes = []
    for name, inc in (("ours", ROOT / "include"), ("ref", ref_include)):
        out = tmp_path / name
        subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(inc), str(src), "-o", str(out)], check=True)
        exes.append(out)
    rng = random.Random(53)
    vals = [0.0, 0.5, 1.0, 2.0, 1e-7, 1 - 1e-7, 0.9999, -1e-4, 3.0]
    lines = []
    for _ in range(3000):
        r = rng.random()
        if r < 0.1:
            lines.append(f"approx {rng.choice(vals + [1.0 + 1e-5, 1.0 + 2e-4])!r} {rng.choice(vals)!r}")
        elif r < 0.25:
            n = rng.randrange(1, 6)
            v = [rng.choice(vals) for _ in range(n)]
            lines.append(f"feas {rng.choice([1.0, 2.0, 2.5])!r} {n} " + " ".join(map(repr, v)))
        elif r < 0.4:
            n = rng.randrange(1, 6)
            ax = [rng.choice(vals) for _ in range(2 * n)]
            lines.append(f"infeas {rng.choice([1.0, 2.0])!r} {n} " + " ".join(map(repr, ax)))
        elif r < 0.7:
            n = rng.randrange(1, 8)
            lb = [rng.choice([0.0, -1.0, 1.0]) for _ in range(n)]
            ub = [lo + rng.choice([0.0, 1.0, 2.0]) for lo in lb]
            x = [rng.choice([lo, hi, (lo + hi) / 2, lo + 1e-7, hi - 5e-7]) for lo, hi in zip(lb, ub)]
            g = [rng.choice([-1.0, 0.0, -0.0, 0.5, 2.0, 1e-7, -3e-7]) for _ in range(n)]
            lines.append(f"box {n} " + " ".join(map(repr, g + x + lb + ub)))
        else:
            n = rng.randrange(1, 8)
            rhs = rng.choice([1.0, 2.0, 3.5])
            full = rng.randrange(2)
            ints = [rng.randrange(2) for _ in range(n)]
            lb = [float(rng.randrange(2)) if i else 0.0 for i in ints]
            ub = [lo + rng.choice([1.0, 2.0]) if i else rhs for lo, i in zip(lb, ints)]
            x = [rng.choice([lo, hi, (lo + hi) / 2, lo + 1e-7]) for lo, hi in zip(lb, ub)]
            g = [rng.choice([-1.0, 0.0, 0.5, 2.0, -0.25, 1e-7]) for _ in range(n)]
            lines.append(f"simplex {full} {rhs!r} {n} " + " ".join(map(str, ints)) + " "
                         + " ".join(map(repr, g + x + lb + ub)))
    script = "\n".join(lines) + "\n"
    a, b = (subprocess.run([str(e)], input=script, capture_output=True, text=True, check=True).stdout
            for e in exes)
    assert a.count("\n") == len(lines)
    assert a == b


def test_logger_header_drives_like_the_examples(tmp_path):
    """include/gpuboscia/logger.h: the examples' Logger / LoggerParams /
    SolutionStats calls compile warning-free; rows are throttled by the node
    interval except for new incumbents; a disabled logger prints nothing."""
    out = tmp_path / "logger_demo"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "logger_demo.cpp"), "-o", str(out)], check=True)
    text = subprocess.run([str(out)], capture_output=True, text=True, check=True).stdout
    rows = [line.split() for line in text.splitlines() if line.startswith("  ") and line.split()[-1][0].isdigit()]
    nodes = [int(r[1]) if r[0] == "*" else int(r[0]) for r in rows]
    # rows at 0, every >= 100 nodes, and the new incumbent at 120 (marked)
    assert nodes == [0, 120, 240, 360]
    assert [r[0] == "*" for r in rows] == [False, True, False, False]
    assert "Decomposition-Invariant Frank-Wolfe" in text and "secant" in text
    assert "Reached tolerance" in text and "2 of 20 entries nonzero" in text
    assert text.count("variables 20") == 1    # the disabled logger printed nothing


def _fmt(v):
    return " ".join(repr(float(e)) for e in v)


def test_host_lmo_oracles_match_the_reference_outputs(tmp_path):
    """BoxLMO / UnitSimplexLMO / EqualitySimplexLMO / BirkhoffLMO compute_v_cpu,
    compute_inface_v_cpu and dicg_maximum_step_cpu (include/gpuboscia/lmo.h over
    lmo_dicg.h) reproduce, exactly, the reference's own CPU oracles on the
    golden cases (tests/golden/reference_cpu.json: forward vertex, in-face
    vertex, and for box and simplex the maximum step along inface(g) -
    forward(-g); Birkhoff orders 3-36 with forced, forbidden and face edges)."""
    exe = tmp_path / "lmo_cpu"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "lmo_cpu.cpp"), "-o", str(exe)], check=True)
    lines, want = [], []
    for c in GOLDEN["box"]:
        n = len(c["g"])
        lines.append(f"box {n} {_fmt(c['g'])} {_fmt(c['lb'])} {_fmt(c['ub'])} {_fmt(c['x'])}")
        want.append(c["forward"] + c["inface"] + [c["step"]])
    for c in GOLDEN["simplex"]:
        n = len(c["g"])
        lines.append(f"simplex {c['equality']} {c['rhs']!r} {n} {len(c['ints'])} {' '.join(map(str, c['ints']))} "
                     f"{_fmt(c['g'])} {_fmt(c['lb'])} {_fmt(c['ub'])} {_fmt(c['x'])}")
        want.append(c["forward"] + c["inface"] + [c["step"]])
    for c in GOLDEN["birkhoff"]:
        lines.append(f"birkhoff {c['order']} {_fmt(c['cost'])} {_fmt(c['lb'])} {_fmt(c['ub'])} {_fmt(c['x'])}")
        want.append(c["forward"] + c["inface"])
    r = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = [[float(t) for t in line.split()] for line in r.stdout.splitlines()]
    assert len(got) == len(want) == len(GOLDEN["box"]) + len(GOLDEN["simplex"]) + len(GOLDEN["birkhoff"])
    for i, (g, w) in enumerate(zip(got, want)):
        assert len(g) == len(w), i
        assert all(_eq(a, b) for a, b in zip(g, w)), (i, g, w)


def test_host_lmo_oracles_live_against_the_reference(tmp_path):
    """The drop-in headers' CPU oracles against the reference's own CPU
    functions (oracle/_ref, built where the reference tree was present) on
    fresh random cases: bounded and equality simplices with integral and
    fractional right-hand sides, tie-heavy gradients and forced integer
    coordinates (forward vertex, in-face vertex, DICG maximum step), and
    Birkhoff orders 3-16 with forbidden entries and forced pairs."""
    import sys
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np
    import _oracle as O
    R = O.ref()
    if R is None:
        pytest.skip("reference tree not available at build time")
    exe = tmp_path / "lmo_cpu"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "lmo_cpu.cpp"), "-o", str(exe)], check=True)
    rng = np.random.default_rng(23)
    lines, want = [], []
    for c in range(400):
        n = int(rng.integers(2, 30))
        eq = int(rng.integers(0, 2))
        ints = sorted(rng.choice(n, int(rng.integers(0, n + 1)), replace=False).tolist())
        rhs = float(rng.integers(1, 10)) + (0.5 if c % 2 else 0.0)
        g = rng.integers(-2, 3, n) / 8.0
        lb = np.zeros(n)
        ub = np.where(np.isin(np.arange(n), ints), rng.integers(1, 4, n), rhs).astype(float)
        for j in ints[:2]:
            lb[j] = 1.0 if lb.sum() + 1 <= rhs else 0.0
        x = lb.copy()
        rest = rhs - lb.sum() if eq else (rhs - lb.sum()) * rng.random()
        for j in rng.permutation(n):
            add = min(ub[j] - x[j], rest)
            x[j] += add
            rest -= add
        iv = np.array(ints, dtype=np.int32)
        fwd, face, step = np.zeros(n), np.zeros(n), np.zeros(1)
        ip = iv.ctypes.data if ints else None
        R.ref_simplex_lmo(eq, 0, n, rhs, ip, len(ints), g.ctypes.data, None, lb.ctypes.data, ub.ctypes.data,
                          fwd.ctypes.data, None)
        R.ref_simplex_lmo(eq, 1, n, rhs, ip, len(ints), g.ctypes.data, x.ctypes.data, lb.ctypes.data,
                          ub.ctypes.data, face.ctypes.data, step.ctypes.data)
        lines.append(f"simplex {eq} {rhs!r} {n} {len(ints)} {' '.join(map(str, ints))} "
                     f"{_fmt(g)} {_fmt(lb)} {_fmt(ub)} {_fmt(x)}")
        want.append(list(fwd) + list(face) + [float(step[0])])
    for _ in range(100):
        order = int(rng.choice([3, 4, 5, 6, 7, 8, 12, 16]))
        n = order * order
        cost = rng.integers(-3, 4, n) / 4.0
        lb, ub = np.zeros(n), np.ones(n)
        p = rng.permutation(order)
        forbid = rng.random(n) < 0.25
        forbid[np.arange(order) * order + p] = False
        ub[forbid] = 0.0
        lb[np.arange(order) * order + p] = (rng.random(order) < 0.15).astype(float)
        x = np.zeros(n)
        x[np.arange(order) * order + p] = 1.0
        fwd, face = np.zeros(n), np.zeros(n)
        R.ref_birkhoff_lmo(order, 0, cost.ctypes.data, None, lb.ctypes.data, ub.ctypes.data, fwd.ctypes.data)
        zl, on = np.zeros(n), np.ones(n)
        R.ref_birkhoff_lmo(order, 1, cost.ctypes.data, x.ctypes.data, zl.ctypes.data, on.ctypes.data,
                           face.ctypes.data)
        lines.append(f"birkhoff {order} {_fmt(cost)} {_fmt(lb)} {_fmt(ub)} {_fmt(x)}")
        want.append(list(fwd) + list(face))
    r = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    got = [[float(t) for t in line.split()] for line in r.stdout.splitlines()]
    assert len(got) == len(want) == 500
    for i, (gv, w) in enumerate(zip(got, want)):
        assert len(gv) == len(w), i
        assert all(_eq(a, b) for a, b in zip(gv, w)), (i, lines[i], gv, w)


# the reference's public header names (include/gpuboscia/ of the reference)
REFERENCE_HEADERS = [
    "algorithms.cuh", "atomic_incumbent.h", "bnb.h", "branching.h", "concurrent_queue.h",
    "dense_quadratic_objectives.cuh", "device_resident_solver.cuh", "gap_utils.h", "gpuboscia.cuh",
    "heuristics.h", "line_search_options.h", "lmo.cuh", "lmo_dicg.h", "logger.h", "multiblock.cuh", "node.h",
    "node_select.h", "problem.h", "tree.h",
]


@pytest.mark.parametrize("name", REFERENCE_HEADERS)
def test_every_reference_header_name_compiles_alone(tmp_path, name):
    """A program that includes any of the reference's headers by its own name
    compiles against the drop-in set with g++ (no nvcc), warning-free."""
    src = tmp_path / "one.cpp"
    src.write_text(f"#include <gpuboscia/{name}>\nint main() {{ return 0; }}\n")
    subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    "-I", CUDA_INCLUDE, str(src)], check=True)


def test_every_reference_header_name_compiles_alone_under_nvcc(tmp_path):
    """The same one-include programs as CUDA translation units (the way the
    reference's users compile them): each compiles with nvcc for sm_103a,
    which also brings in the device-side names (MultiBlockContext, the
    template relaxation of user objectives)."""
    import concurrent.futures as cf
    from gpuboscia_gb300 import build
    nvcc = str(build._cuda_home() / "bin" / "nvcc")

    def one(name):
        src = tmp_path / f"{name.replace('.', '_')}.cu"
        src.write_text(f"#include <gpuboscia/{name}>\nint main() {{ return 0; }}\n")
        r = subprocess.run([nvcc, "-std=c++17", build.ARCH, "-I", str(ROOT / "include"), "-c", str(src), "-o",
                            str(src.with_suffix(".o"))], capture_output=True, text=True)
        return name, r.returncode, r.stderr[-2000:]

    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        for name, rc, err in ex.map(one, REFERENCE_HEADERS):
            assert rc == 0, (name, err)


def test_node_selection_policies(tmp_path):
    src = tmp_path / "sel.cpp"
    src.write_text(r'''
#include <cstdio>
#include <gpuboscia/node_select.h>
int main() {
    std::vector<Node> nodes;
    const double bound[5] = {3.0, -1.0, 2.0, 0.5, 7.0};
    const int depth[5] = {1, 4, 2, 9, 0};
    for (int i = 0; i < 5; ++i) {
        nodes.emplace_back(i, -1, depth[i], std::vector<double>{0.0}, std::vector<double>{1.0});
        nodes.back().dual_bound = bound[i];
    }
    NodeSelector sel = best_first;
    for (int i : sel(nodes, 3)) std::printf("%d ", i);
    std::printf("| ");
    for (int i : depth_first(nodes, 2)) std::printf("%d ", i);
    std::printf("| %zu %zu\n", best_first(nodes, 10).size(), best_first({}, 4).size());
    return 0;
}
''')
    exe = tmp_path / "sel"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    "-I", CUDA_INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["1", "3", "2", "|", "3", "1", "|", "5", "0"]


def test_node_state_names_have_the_reference_values(tmp_path):
    """DRSNodeState / DRSInitialPointSupplied (device_resident_solver.cuh:192-202)
    under the drop-in header: the reference's values, usable as status bytes."""
    src = tmp_path / "ns.cpp"
    src.write_text(r'''
#include <gpuboscia/device_resident_solver.cuh>
static_assert(DRSFractionalUnconverged == 0 && DRSFractionalConverged == 1 && DRSInfeasible == 2 &&
              DRSIntegralUnconverged == 3 && DRSIntegralConverged == 4 && DRSInitialPointSupplied == 0x80, "");
int main() { const uint8_t s = DRSIntegralUnconverged | DRSInitialPointSupplied; return s == 0x83 ? 0 : 1; }
''')
    exe = tmp_path / "ns"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
                    "-I", CUDA_INCLUDE, str(src), "-o", str(exe)], check=True)
    subprocess.run([str(exe)], check=True)


@pytest.mark.parametrize("defines", [[], ["-DGBX_NO_NVTX"]])
def test_nvtx_ranges_nest_and_compile_out(tmp_path, defines):
    """The solver's NVTX ranges (dispatch, upload, relaxation, download,
    completion, frontier replays) come from a header-only helper: ranges
    nest and close on scope exit, cost nothing without a profiler attached,
    and compile out under GBX_NO_NVTX."""
    src = tmp_path / "nv.cpp"
    src.write_text(r'''
#include <gpuboscia/nvtx.h>
#include <stdexcept>
static int work(int k) {
    gpuboscia::detail::NvtxRange r("gbx.test.outer");
    { gpuboscia::detail::NvtxRange q("gbx.test.inner"); k += 1; }
    if (k > 2) throw std::runtime_error("early exit closes the range");
    return k;
}
int main() {
    int s = work(0) + work(1);
    try { work(5); } catch (const std::exception&) { s += 10; }
    return s == 13 ? 0 : 1;
}
''')
    exe = tmp_path / "nv"
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", *defines, "-I", str(ROOT / "include"),
                    "-I", CUDA_INCLUDE, str(src), "-o", str(exe)], check=True)
    subprocess.run([str(exe)], check=True)
