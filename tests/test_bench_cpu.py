"""bench.py on CPU: the reference arm runs the oracle alone (no product
module is imported) at the workload's own size, and `--gpus N` without a
launcher runs N local ranks (rank 0 reports n_gpus = N)."""
import json
import os
import pathlib
import subprocess
import sys

ROOT = pathlib.Path(__file__).resolve().parent.parent


def _bench(*args, timeout=600):
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env["HP_ORACLE_THREADS"] = "2"
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                       timeout=timeout, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_runs_the_oracle_only():
    out = _bench("--impl", "reference", "--num-vars", "6", "--steps", "2", "--warmup", "1")
    assert out["impl"] == "reference" and out["n_gpus"] == 1
    assert out["config"]["num_vars"] == 6 and "full size" in out["config"]["workload"]
    assert out["product_code_loaded"] == []
    assert out["steps"] == 2 and out["value"] > 0
    assert out["e2e"]["h2d_bytes_per_step"] == 0


def test_gpus_flag_without_launcher_runs_n_ranks():
    out = _bench("--impl", "reference", "--gpus", "2", "--workload", "commit", "--num-vars", "8", "--steps", "1",
                 "--warmup", "0")
    assert out["n_gpus"] == 2
    assert out["metric"] == "MSM pts/s"
