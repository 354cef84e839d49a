"""CPU tests of bench.py's reference arm (`--impl reference`): the CPU
implementation of the path -- the reference compiled from its sources where
oracle/_ref exists, else the oracle port -- timed on the host cores, printed
as one JSON line with the GPU arm's metric, unit and workload.  Under
torchrun only rank 0 runs it; the other ranks exit 0 without work."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(args, env=None, timeout=600):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT,
                          env=e, capture_output=True, text=True, timeout=timeout)


def test_reference_arm_prints_one_contract_line():
    out = run_bench(["--impl", "reference", "--steps", "1", "--warmup", "3"])
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    line = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["steps"] == 1 and line["warmup"] >= 3
    assert line["config"]["workload"] == bench.WORKLOAD["name"]
    assert line["value"] > 0
    cpu = line["cpu_baseline"]
    assert cpu["kind"] in ("reference", "port") and cpu["cores"] >= 1
    assert cpu["value"] == line["value"] and cpu["one_core"]["value"] > 0
    assert "N * (n+1) force calls" in cpu["counting"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_without_work():
    out = run_bench(["--impl", "reference", "--steps", "1", "--warmup", "3", "--gpus", "2"],
                    env={"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2",
                         "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": "29531"}, timeout=120)
    assert out.returncode == 0, out.stderr[-2000:]
    assert not [l for l in out.stdout.splitlines() if l.startswith("{")], out.stdout
