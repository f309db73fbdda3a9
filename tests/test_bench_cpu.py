"""bench.py's reference arm (--impl reference) needs no GPU: its one JSON line
carries the contract's keys with the GPU arm's metric, unit and config, and
under torchrun only rank 0 prints."""
import json
import os
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parent.parent
ARGS = ["--impl", "reference", "--steps", "2", "--warmup", "1", "--nodes", "16", "--iters", "5",
        "--ref-budget", "0.2", "--workload", "birkhoff_gnp36"]


def _run(env_extra=None, args=ARGS):
    env = dict(os.environ, **(env_extra or {}))
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                          env=env, cwd=ROOT, timeout=600)


def test_reference_arm_line():
    r = _run()
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    sys.path.insert(0, str(ROOT))
    import bench
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "nodes/s"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["n_gpus"] == 1
    assert d["steps"] == 2 and d["warmup"] == 1 and d["ms_per_step"] > 0
    assert d["scaling"] == "weak" and d["vs_baseline"] is None and d["data"] == "synthetic"
    assert d["config"]["workload"] == "birkhoff_gnp36" and d["config"]["nodes_per_batch"] == 16
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr
    assert not [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_default_workload_is_the_order_400_search():
    """Without --workload the bench measures the order-400 isomorphic 10-regular
    pair with 1024-node batches; the reference arm times the oracle on a
    bounded sample of that workload's open nodes."""
    r = _run(args=["--impl", "reference", "--steps", "1", "--warmup", "1", "--iters", "1", "--ref-budget", "0"])
    assert r.returncode == 0, r.stderr
    d = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][0])
    cfg = d["config"]
    assert cfg["workload"] == "birkhoff_regular400" and cfg["order"] == 400 and cfg["nodes_per_batch"] == 1024
    assert d["value"] > 0 and d["cpu_baseline"]["sample"]
