"""The C++ drop-in headers on the CPU: the reference's test_cpu.cpp assertions
(tests/cpp/test_host.cpp) and the host rules against the reference fixtures."""
import json
import math
import pathlib
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = json.loads((ROOT / "tests" / "golden" / "reference_cpu.json").read_text())


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
