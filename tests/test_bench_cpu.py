"""bench.py's reference arm on the host (no GPU): the JSON line it prints and
its behaviour on ranks other than 0.  The arm times the reference's CPU
implementation of the batched L2 solve (the compiled MEX kernels where they
built, else their C restatement) inside the FP64 solver restatement."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
        "cpu_baseline", "e2e"}


def _bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           *args], cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=300)


def test_reference_arm_prints_one_contract_line():
    r = _bench({"RANK": "0", "WORLD_SIZE": "1"}, "--steps", "1", "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert KEYS <= set(out)
    assert out["impl"] == "reference" and out["unit"] == "recons/s"
    assert out["higher_is_better"] is True and out["steps"] == 1 and out["warmup"] == 0
    assert out["value"] > 0 and out["ms_per_step"] > 0
    cb = out["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert cb["value"] == out["value"] and cb["sample"]
    assert out["e2e"] == {"value": out["value"], "unit": "recons/s",
                          "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same workload the GPU arm reports
    assert out["config"]["grid"] == [128, 128] and out["config"]["n_det"] == 256
    assert out["config"]["n_t"] == 2030 and out["config"]["iterations"] == 50


def test_reference_arm_is_silent_on_other_ranks():
    r = _bench({"RANK": "1", "WORLD_SIZE": "2"}, "--steps", "1", "--warmup", "0")
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
