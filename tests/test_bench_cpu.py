"""bench.py on the host (no GPU): the reference arm's JSON line and its
behaviour on ranks other than 0, and the GPU arm's CPU-baseline helper.  The
reference arm times the reference's CPU implementation of the batched L2
solve (the compiled MEX kernels where they built, else their C restatement)
inside the FP64 solver restatement."""
import json
import os
import subprocess
import sys

import numpy as np

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


def test_cpu_baseline_leg_runs_a_bounded_sample():
    """The GPU arm's CPU-baseline helper on a stand-in for the model's
    attributes (no device needed): the full solve and the short
    single-thread sample both run the FP64 oracle on the same geometry."""
    from types import SimpleNamespace

    import bench
    from oracle import model as M
    disc = SimpleNamespace(nx=24, nz=24, fov=(-0.003, 0.003, -0.003, 0.003))
    probe = SimpleNamespace(n_det=32, radius=0.02, angular_coverage=135.0, fs=4e7,
                            n_samples=900, delay=0.0, eir=None, eir_length=65)
    model = SimpleNamespace(Discretization=disc, Probe=probe, c=1500.0, fmin=1e5, fmax=12e6,
                            norm=1.0)
    om = M.Model(M.ArcProbe(n_det=32, radius=0.02, coverage_deg=135.0, n_samples=900,
                            eir_length=65), M.Grid(24, 24, disc.fov), c=1500.0, norm=1.0)
    rng = np.random.default_rng(3)
    b = om.forward(rng.random((1, 24, 24)))[0]
    rec, t_full = bench.oracle_solve(model, b, 2, 6)
    assert rec.shape == (24, 24) and rec.min() >= 0 and t_full > 0
    _, t_one = bench.oracle_solve(model, b, 1, bench.ONE_THREAD_ITERS)
    assert t_one > 0
    # the TV and L1 modes' oracle legs on the same stand-in
    rec_tv, t_tv = bench.oracle_tv_solve(model, b, 2, 5e-3, 2)
    assert rec_tv.shape == (24, 24) and rec_tv.min() >= 0 and t_tv > 0
    rec_l1, t_l1 = bench.oracle_l1_solve(model, b, 3, 1e-3, 2)
    assert rec_l1.shape == (24, 24) and np.isfinite(rec_l1).all() and t_l1 > 0


def test_clock_summary_parses_the_nvidia_smi_samples(tmp_path):
    """The clocks object bench.py attaches to its JSON line: median SM clock
    under load, the maximum clock, and every throttle reason seen Active."""
    import bench
    path = tmp_path / "clocks.csv"
    path.write_text(
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
        "0, 1980, 2070, 1390.5, 0x4, Not Active, Not Active, Not Active, Active\n"
        "0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active\n"
        "garbage line\n")
    c = bench.Clocks(0, str(path))
    c.proc = object()  # samples already written; no nvidia-smi here
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    assert path.exists()  # a file the caller named is kept


def test_roofline_bytes_per_launch():
    """Algorithmic bytes behind roofline.achieved at the bench's batch of 64:
    FP32 travel table 4PD + image 4PW + sinogram 4TDW for an interpolation
    launch (about 154 MB), read + write of the sinogram for the IR
    convolution, of the image for the prefilter."""
    import bench
    P, D, T, W = 128 * 128, 256, 2030, 64
    fwd = bench.algorithmic_bytes("interp_forward", W)
    assert fwd == 4 * P * D + 4 * P * W + 4 * T * D * W
    assert abs(fwd / 1e6 - 154.0) < 1.0
    assert bench.algorithmic_bytes("interp_adjoint", W) == fwd
    assert bench.algorithmic_bytes("ir_conv", W) == 8 * T * D * W
    assert bench.algorithmic_bytes("prefilter", W) == 8 * P * W
    assert bench.algorithmic_bytes("something_else", W) is None
