"""bench.py's reference arm on the CPU (it needs no GPU): one JSON line with
the metric, "impl": "reference", a cpu_baseline describing the run and an
e2e object with zero copy bytes; ranks other than 0 exit 0 without output."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config",
           "small", "--steps", "1", "--warmup", "1", "--cpu-sample", "3000"]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, cwd=ROOT, timeout=600)


def test_reference_arm_line():
    r = _run({})
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "Mvis/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["metric"].startswith("Mvis/s grid+degrid")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "3000" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "Mvis/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0 and r.stdout.strip() == ""
