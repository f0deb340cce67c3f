"""Benchmark: batched non-negative L2-regularised reconstruction
(rec_nn_with_L2_reg) on one GB300, checked against the FP64 oracle solve.

Workload (one "step" = one batched solve of --batch independent sinograms):
  128 x 128 px at 0.2 mm pitch (25.4 mm FOV); 256-element arc, R = 40 mm,
  135 deg; 2030 samples at 40 MHz; c = 1500 m/s; Gaussian-modulated 5 MHz EIR
  (60 % bandwidth, 256 taps zero-padded to 257); Butterworth [0.1, 12] MHz;
  no SIR; disk + vessel phantoms, 1 % Gaussian noise; lambdaL2 = 1e-2
  (identity), 50 outer iterations; the model is normalised by its largest
  singular value (power iteration on the GPU).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl ours|reference]

Prints ONE JSON line (rank 0).  ``value`` is recons/s with the sinograms
already in HBM; ``e2e`` is the same metric through the public Python API
with pinned host buffers (H2D of the sinograms and D2H of the images inside
the timed region).  ``--impl reference`` times the CPU implementation of the
same path (the reference's compiled MEX when it was built on this host,
otherwise the project's C restatement of it, inside the FP64 wrappers and
solver) on a bounded sample of the workload.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "mb-rec-msot_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "NNLS recons/s at <=1e-3 rel. error vs FP64: learned+batched vs plain, 1 GB300"
N_GRID, N_DET, N_T, N_ITER, LAMBDA = 128, 256, 2030, 50, 1e-2
ONE_THREAD_ITERS = 2  # outer iterations of the single-thread CPU sample
HBM_FALLBACK_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-oracle", action="store_true", help="skip the FP64 oracle solve")
    ap.add_argument("--clocks-csv", default=None,
                    help="keep the nvidia-smi clock samples of the timed region in this file")
    ap.add_argument("--op", action="store_true",
                    help="time the operator alone: one step = A then A^T on the batch")
    ap.add_argument("--tv", action="store_true",
                    help="batched multispectral TV-NNLS on mixed grid sizes (28 wavelengths x "
                         "16 frames): one JSON line")
    ap.add_argument("--tv-grids", default="128,200,256,400",
                    help="grid sizes the --tv instances are drawn from")
    ap.add_argument("--tv-batch", type=int, default=64,
                    help="--tv: most instances per solve call")
    ap.add_argument("--tv-concurrent", action="store_true",
                    help="also time the grid sizes solved concurrently (one host thread and "
                         "private stream per grid size)")
    ap.add_argument("--sweep", action="store_true",
                    help="SIR operator sweep (128^2, 256^2, 400^2; generated 8x8-sub-element "
                         "SPMR tables): one JSON line per grid")
    ap.add_argument("--warmstart", action="store_true",
                    help="learned warm start: train the U-Net on plain-solver pairs, then "
                         "iterations and recons/s to the 200-iteration plain accuracy on 256 "
                         "frames, dmas_cf timed on the same frames: one JSON line")
    ap.add_argument("--ws-grid", type=int, default=128)
    ap.add_argument("--ws-pairs", type=int, default=2048)
    ap.add_argument("--ws-train-steps", type=int, default=3000)
    ap.add_argument("--ws-frames", type=int, default=256)
    ap.add_argument("--ws-input-iters", type=int, default=10)
    ap.add_argument("--ws-backprojection", default="transpose", choices=["transpose", "waveeq"],
                    help="network input when --ws-input-iters is 0")
    ap.add_argument("--no-fp16", action="store_true",
                    help="skip the FP16-storage line of the headline")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-start arm of the headline line")
    ap.add_argument("--learned-pairs", type=int, default=4096)
    ap.add_argument("--learned-steps", type=int, default=6000)
    ap.add_argument("--learned-input-iters", type=int, default=5,
                    help="plain iterations of the learned arm's network input")
    ap.add_argument("--learned-trajectory", type=int, default=0,
                    help="learned arm: also feed the last m steps x_k - x_(k-m) (0: off)")
    ap.add_argument("--learned-target-iters", type=int, default=0,
                    help="plain iterations of the training targets (0: the headline's)")
    ap.add_argument("--unet", action="store_true",
                    help="warm-start U-Net alone (4 levels, 32 base channels, batch 16): "
                         "training steps and forward passes: one JSON line")
    ap.add_argument("--unet-side", type=int, default=128)
    ap.add_argument("--bp", action="store_true",
                    help="analytic reconstructors: backproject_waveeq and dmas_cf on 256 "
                         "frames of 256 det x 2030 samples, 128 x 128 px")
    ap.add_argument("--prep", action="store_true",
                    help="raw-sinogram pre-processing (crop 3, Butterworth window, zero-phase "
                         "filter) of 64 x 256 x 2033 samples: one JSON line")
    ap.add_argument("--l1", action="store_true",
                    help="batched L1-NNLS (rec_nn_with_L1_eye_reg) at 400x400 px, 512-element "
                         "arc over 270 deg, 4096 samples, 64 instances: one JSON line")
    ap.add_argument("--l1-grid", type=int, default=400)
    ap.add_argument("--l1-fp16", action="store_true",
                    help="--l1: FP16 storage (scaled per instance) of the forward's interpolation "
                         "input")
    ap.add_argument("--l1-bf16", action="store_true",
                    help="--l1: BF16 storage of the forward's interpolation input")
    ap.add_argument("--l1-refine", type=int, default=0,
                    help="--l1 with --l1-bf16: every k-th outer iteration in FP32")
    ap.add_argument("--l1-iters", type=int, default=50)
    ap.add_argument("--l1-check-iters", type=int, default=0,
                    help="iterations of the instance-0 solve compared with the FP64 oracle "
                         "(0: the same as --l1-iters)")
    return ap.parse_args()


def workload_config(batch, n_gpus):
    return {
        "workload": "rec_nn_with_L2_reg, 128x128 px @0.2 mm, 256-el arc R=40 mm 135 deg, "
                    "2030 samples @40 MHz, EIR 257 taps, lambdaL2=1e-2, 50 outer iterations",
        "grid": [N_GRID, N_GRID], "n_det": N_DET, "n_t": N_T, "iterations": N_ITER,
        "lambdaL2": LAMBDA, "batch_per_gpu": batch, "global_batch": batch * n_gpus,
        "parallelism": f"replicas x{n_gpus}",
        "l2": "flushed (512 MB write) between timed steps",
    }


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


# ----------------------------------------------------------------------------
# clocks during the timed region
# ----------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, path=None):
        """Samples every 200 ms into ``path`` (kept), or into a temporary file."""
        import tempfile
        self.proc = None
        self.keep = path is not None
        self.path = path or os.path.join(tempfile.gettempdir(), f"clocks_bench_{os.getpid()}.csv")
        self.idx = gpu_index

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.idx), "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        if not self.keep:
            try:
                os.remove(self.path)
            except OSError:
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------------------------
# our implementation
# ----------------------------------------------------------------------------
def build_model(batch, norm=None):
    from msot_gb300 import Discretization, MSOTmodel, Probe
    from msot_gb300.synthetic import gauss_pulse_eir
    h = 0.2e-3 * 127 / 2
    probe = Probe(n_det=N_DET, radius=0.040, angular_coverage=135.0, fs=4e7, n_samples=N_T,
                  delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
    disc = Discretization([-h, h], N_GRID)
    return MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, norm, max_batch=batch)


def make_data(model, batch, seed):
    """Seeded disk + vessel phantoms -> sinograms on the GPU (+1 % noise)."""
    import torch
    from msot_gb300.synthetic import phantom
    rng = np.random.default_rng(seed)
    imgs = np.stack([phantom(model.Discretization, rng) for _ in range(batch)]).astype(np.float32)
    x = torch.tensor(imgs, device="cuda")
    y = model.forward(x)
    amp = y.abs().amax(dim=(1, 2), keepdim=True)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    y = y + 0.01 * amp * torch.randn(y.shape, device="cuda", generator=gen)
    return x, y.contiguous()


def oracle_solve(model, b_np, threads, n_iter=None):
    """CPU-baseline leg: FP64 oracle solve of one instance with the same model
    parameters as the GPU plan (n_iter outer iterations, default the
    workload's); the full solve is also the accuracy reference."""
    from oracle import model as M
    from oracle import native
    from oracle import solvers as S
    native.port().set_threads(threads)
    g = model.Discretization
    p = model.Probe
    op = M.ArcProbe(n_det=p.n_det, radius=p.radius, coverage_deg=p.angular_coverage, fs=p.fs,
                    n_samples=p.n_samples, delay=p.delay, eir=p.eir, eir_length=p.eir_length)
    om = M.Model(op, M.Grid(g.nx, g.nz, g.fov), c=model.c, fmin=model.fmin, fmax=model.fmax,
                 norm=model.norm)
    P = g.nx * g.nz
    fwd = lambda v: om.forward(v.reshape(1, g.nx, g.nz)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, p.n_det, -1)).ravel()
    t0 = time.perf_counter()
    rec, _, _ = S.rec_nn_with_L2_reg(fwd, adj, b_np.astype(np.float64).ravel(), P,
                                     N_ITER if n_iter is None else int(n_iter), LAMBDA)
    return rec.reshape(g.nx, g.nz), time.perf_counter() - t0


# DRAM bytes (read + write) per launch of each family's kernel at batch 64,
# from one ncu --set full capture per kernel of `bench.py --op --batch 64`
# (profiles/das_kernels_128px_b64.md, profiles/eir_conv_fft_128px_b64.md)
NCU_TRAFFIC_B64 = {"interp_forward": 84.3648e6 + 97.833984e6,
                   "interp_adjoint": 77.760256e6 + 3.016448e6,
                   "ir_conv": 133.13664e6 + 83.677184e6,
                   "prefilter": 4.246784e6}


def algorithmic_bytes(kid_name, batch):
    P, D, T = N_GRID * N_GRID, N_DET, N_T
    if kid_name in ("interp_forward", "interp_adjoint"):
        return 4 * P * D + 4 * P * batch + 4 * T * D * batch
    if kid_name == "ir_conv":
        return 2 * 4 * T * D * batch
    if kid_name == "prefilter":
        return 2 * 4 * P * batch
    if kid_name == "permute":
        return 2 * 4 * P * batch + 4 * P
    return None


def run_operator(args):
    """Operator-only step (A then A^T on --batch images); prints a JSON line
    with applies/s.  Used for profiling the operator kernels."""
    import torch
    from msot_gb300 import _lib
    L = _lib.load()
    B = args.batch
    model = build_model(B, norm=2.0243e-05)  # fixed sigma_max: no estimation launches
    tuning = model.autotune(B)  # the kernel variants the solve uses on this geometry
    x, b = make_data(model, B, seed=7)
    for _ in range(args.warmup):
        model.transpose(model.forward(x))
    torch.cuda.synchronize()
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(args.steps):
        model.transpose(model.forward(x))
    z.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(z) / args.steps
    return {"metric": "A + A^T pairs/s (instances)", "value": B / (ms / 1e3), "unit": "pairs/s",
            "ms_per_step": ms, "batch": B, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "impl": "ours-operator", "autotune": tuning}


# ----------------------------------------------------------------------------
# replicas over ranks: each rank solves its own batch (no data-path
# collective); the step time is the slowest rank's
# ----------------------------------------------------------------------------
def rank_seed(rank: int) -> int:
    """Seed of a rank's synthetic batch (distinct phantoms per replica)."""
    return 1000 + int(rank)


def max_over_ranks(x: float, dist=None) -> float:
    """MAX of x over the ranks of the default process group (NCCL: on the
    device; gloo: on the host); x itself without a group."""
    if dist is None:
        return float(x)
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(batch_per_rank: int, world: int, ms_per_step: float) -> float:
    """Whole-job recons/s: every rank's batch per the slowest rank's step."""
    return batch_per_rank * world / (ms_per_step / 1e3)


def run_ours(args, rank, world):
    import torch
    from msot_gb300 import _lib, rec_nn_with_L2_reg
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    L = _lib.load()
    B = args.batch
    model = build_model(B)
    tuning = model.autotune(B)  # kernel variants timed on this geometry and batch
    x_true, b = make_data(model, B, seed=rank_seed(rank))
    flush = torch.empty(512 * 1024 * 1024 // 4, device="cuda")
    dist = None
    if world > 1:
        import torch.distributed as dist
    for _ in range(args.warmup):
        rec = rec_nn_with_L2_reg(model, b, N_ITER, LAMBDA)[0]
    torch.cuda.synchronize()
    # --- timed region: K batched solves, device time by CUDA events ----------------
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    n0 = L.msot_launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(torch.cuda.current_device(), args.clocks_csv) as clk:
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record()
            rec = rec_nn_with_L2_reg(model, b, N_ITER, LAMBDA)[0]
            ev[k][1].record()
        torch.cuda.synchronize()
    launches = L.msot_launch_count() - n0
    ms = max_over_ranks(float(sum(a.elapsed_time(z) for a, z in ev)), dist)
    ms_per_step = ms / args.steps
    value = job_throughput(B, world, ms_per_step)
    # --- end to end through the public API with host buffers --------------------------
    b_host = b.cpu().pin_memory()
    rec_host = torch.empty((B, N_GRID, N_GRID), dtype=torch.float32).pin_memory()
    e2e_ms = 0.0
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = rec_nn_with_L2_reg(model, b_host, N_ITER, LAMBDA)[0]
        rec_host.copy_(r)
        torch.cuda.synchronize()
        e2e_ms += (time.perf_counter() - t0) * 1e3
    e2e_ms = max_over_ranks(e2e_ms / args.steps, dist)
    e2e = {"value": job_throughput(B, world, e2e_ms), "unit": "recons/s",
           "h2d_bytes_per_step": int(b_host.numel() * 4),
           "d2h_bytes_per_step": int(rec_host.numel() * 4)}
    # --- live per-kernel event timing (one instrumented solve) ------------------------
    L.msot_profile_enable(1)
    rec_nn_with_L2_reg(model, b, N_ITER, LAMBDA)
    torch.cuda.synchronize()
    fam = {}
    import ctypes as C
    for kid in range(16):
        name = L.msot_profile_kernel_name(kid)
        if not name:
            break
        n, t = C.c_int(), C.c_double()
        L.msot_profile_read(kid, C.byref(n), C.byref(t))
        if n.value:
            fam[name.decode()] = {"launches": n.value, "ms": t.value}
    L.msot_profile_enable(0)
    if rank != 0:
        return None
    peak, peak_kind = peaks()
    dom = max(fam.items(), key=lambda kv: kv[1]["ms"]) if fam else None
    roof = None
    if dom:
        name, d = dom
        avg_s = d["ms"] / d["launches"] / 1e3
        alg = algorithmic_bytes(name, B)
        ach = alg / avg_s / 1e9 if alg else None
        roof = {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peak, "unit": "GB/s",
                "frac": ach / peak if ach else None,
                "traffic": NCU_TRAFFIC_B64.get(name) if B == 64 else None,
                "peak_source": f"{peak_kind} hbm_gbs (copy)",
                "avg_launch_us": avg_s * 1e6, "bytes_per_launch": alg,
                "families_ms_per_solve": {k: round(v["ms"], 3) for k, v in fam.items()}}
        if name == "interp_forward":
            # the forward's real bound: every (pixel, detector) pair gathers the
            # W values of its pixel from L2 (P D W 4 bytes per launch), against
            # the measured random 32-byte-sector gather rate of an L2-resident
            # buffer (msot_l2_gather_probe, 64 MiB)
            g = C.c_double()
            L.msot_l2_gather_probe(64 << 20, C.byref(g))
            gather = 4.0 * N_GRID * N_GRID * N_DET * B
            roof["l2_gather"] = {"achieved": gather / avg_s / 1e9, "peak": g.value,
                                 "unit": "GB/s", "frac": gather / avg_s / 1e9 / g.value,
                                 "bytes_per_launch": gather,
                                 "peak_source": "measured: msot_l2_gather_probe, 64 MiB"}
    # --- FP64 oracle: accuracy of instance 0 + the CPU baseline sample ----------------
    acc = None
    cpu = None
    if not args.no_oracle and world == 1:  # rank 0 at N = 1 only
        threads = os.cpu_count() or 1
        ref, t_cpu = oracle_solve(model, b[0].cpu().numpy(), threads)
        got = rec[0].cpu().numpy().astype(np.float64)
        acc = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        cpu = {"value": 1.0 / t_cpu, "unit": "recons/s", "cores": threads, "kind": "port",
               "sample": "one full 50-iteration FP64 solve of instance 0 (C restatement of the "
                         "MEX kernels + numpy FFT wrappers/LSQR)"}
        _, t_one = oracle_solve(model, b[0].cpu().numpy(), 1, ONE_THREAD_ITERS)
        cpu["single_thread"] = {
            "value": (ONE_THREAD_ITERS / N_ITER) / t_one, "unit": "recons/s", "cores": 1,
            "sample": f"{ONE_THREAD_ITERS} of the {N_ITER} outer iterations of instance 0 with "
                      f"the C kernels on one thread; recons/s = ({ONE_THREAD_ITERS}/{N_ITER}) / "
                      "time"}
    fp16 = None
    if not args.no_fp16 and world == 1:
        fp16 = fp16_arm(model, b, rec, ref if acc is not None else None, args, flush)
    learned = None
    if not args.no_learned and world == 1:
        learned = learned_arm(model, args)
    return {
        "metric": METRIC, "value": value, "unit": "recons/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded disk+vessel phantoms, 1% noise)",
        "config": workload_config(B, world), "clocks": clk.summary(), "e2e": e2e,
        "gpu_launches": int(launches), "roofline": roof, "cpu_baseline": cpu,
        "autotune": tuning, "learned": learned, "storage_fp16": fp16,
        "rel_error_vs_fp64": acc, "host": platform.machine(),
    }


def fp16_arm(model, b, rec32, ref0, args, flush):
    """The headline solve with the DAS forward's interpolation input stored
    in FP16 (power-of-two scale per instance, FP32 accumulation;
    msot_plan_set_storage): recons/s timed like the headline (same batch,
    steps, L2 flush), the forward's live per-launch time, and its accuracy --
    instance 0 against the FP64 oracle solve (when the oracle ran) and every
    instance against the FP32 GPU solve (itself 3e-7 from FP64).  A secondary
    line: the headline value stays the FP32-storage solve."""
    import ctypes as C
    import torch
    from msot_gb300 import _lib, rec_nn_with_L2_reg
    L = _lib.load()
    B = b.shape[0]
    model.set_storage("fp16")
    try:
        tuning = model.autotune(B)  # the kernel variants for the 16-bit input
        for _ in range(2):
            rec_nn_with_L2_reg(model, b, N_ITER, LAMBDA)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record()
            r = rec_nn_with_L2_reg(model, b, N_ITER, LAMBDA)[0]
            ev[k][1].record()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(z) for a, z in ev) / args.steps
        L.msot_profile_enable(1)
        rec_nn_with_L2_reg(model, b, N_ITER, LAMBDA)
        torch.cuda.synchronize()
        n, t = C.c_int(), C.c_double()
        L.msot_profile_read(1, C.byref(n), C.byref(t))
        L.msot_profile_enable(0)
    finally:
        model.set_storage("fp32")
        model.autotune(B)
    d = ((r - rec32).flatten(1).norm(dim=1) / rec32.flatten(1).norm(dim=1)).double()
    e0 = None
    if ref0 is not None:
        got = r[0].cpu().numpy().astype(np.float64)
        e0 = float(np.linalg.norm(got - ref0) / np.linalg.norm(ref0))
    return {"value": job_throughput(B, 1, ms), "unit": "recons/s", "ms_per_step": ms,
            "interp_forward_us": t.value / max(1, n.value) * 1e3,
            "rel_error_vs_fp64_instance0": e0,
            "max_rel_diff_vs_fp32_solve": float(d.max()), "autotune": tuning,
            "storage": "interpolation input FP16 (power-of-two scale per instance), "
                       "FP32 accumulation"}


def learned_arm(model, args, frames=64):
    """The metric's learned arm on the headline geometry: a U-Net (4 levels,
    32 base channels; the project's kernels) trained on `learned_pairs` pairs
    the plain GPU solver generates (input: the plain iterate after
    learned_input_iters iterations; target: the solution after
    learned_target_iters iterations, default the headline's), then on
    `frames` held-out frames: the accuracy to reach is the headline plain
    solve's (N_ITER iterations) relative distance to a 1000-iteration solve;
    the learned solve is the input iterations + network + the fewest warm
    iterations that reach it (residual-rise fallback included).  Times are
    CUDA events of the batched calls."""
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.synthetic import phantom_batch
    from msot_gb300.warmstart import LearnedWarmStart
    P = args.learned_pairs
    target_iters = args.learned_target_iters or N_ITER
    ii = args.learned_input_iters
    ws = LearnedWarmStart(model, LAMBDA, levels=4, base_channels=32, max_batch=16,
                          input_iters=ii, trajectory=args.learned_trajectory)
    imgs = phantom_batch(model.Discretization, P + frames, seed=11)
    (f, t, b), pair_ms = _event_ms(lambda: ws.make_pairs(imgs, target_iters, seed=12))
    losses, train_ms = _event_ms(lambda: ws.fit(f[:P], t[:P], args.learned_steps, batch=16,
                                                lr=2e-3))
    bt = b[P:P + frames].contiguous()
    del f, t, b
    xs = rec_nn_with_L2_reg(model, bt, 1000, LAMBDA)[0]
    err = lambda x: float((x - xs).norm() / xs.norm())
    rec_nn_with_L2_reg(model, bt, N_ITER, LAMBDA)  # warm-up
    xp, plain_ms = _event_ms(lambda: rec_nn_with_L2_reg(model, bt, N_ITER, LAMBDA)[0])
    target = err(xp)
    ws.solve(bt, 5)  # warm-up (graph capture of the input and warm iterations)
    scan, found = [], None
    for k in (0, 2, 4, 6, 8, 10, 12, 14, 16, 18, 20, 22, 24, 26, 28, 30, 32, 34, 36, 38, 40,
              45, 50, 60, 80, 100, 150):
        if k == 0:  # the network's start itself (input iterations + network)
            (w0, _, fell), ms = _event_ms(lambda: ws.start(bt))
            r = w0
        else:
            (r, fell), ms = _event_ms(lambda: ws.solve(bt, k, restart_iters=N_ITER))
        e = err(r)
        scan.append({"warm_iterations": k, "rel_err": e, "ms": ms,
                     "fallback_instances": int(fell.sum())})
        if e <= target:
            found = (k, ms)
            break
    out = {"plain": {"iterations": N_ITER, "recons_per_s": frames / (plain_ms / 1e3),
                     "rel_err_vs_1000_it": target},
           "accuracy_target": "the plain solve's distance to a 1000-iteration solve",
           "frames": frames, "warm_scan": scan,
           "training": {"pairs": P, "pair_generation_s": pair_ms / 1e3,
                        "steps": len(losses), "batch": 16,
                        "ms_per_step": train_ms / max(1, len(losses)),
                        "loss_first": float(np.mean(losses[:20])),
                        "loss_last": float(np.mean(losses[-100:])),
                        "input": f"plain iterate after {ii} iterations" + (
                            f", and its last {args.learned_trajectory} steps"
                            if args.learned_trajectory else ""),
                        "target": f"plain solution after {target_iters} iterations",
                        "grid": list(model.image_shape),
                        "note": "a subset of the 20k-pair, 256 px training set, sized for "
                                "the default bench run"}}
    if found:
        k, ms = found
        out.update({"recons_per_s": frames / (ms / 1e3), "ratio_to_plain": plain_ms / ms,
                    "iterations": {"plain": N_ITER, "learned": ii + k,
                                   "saved": N_ITER - ii - k}})
    else:
        out.update({"recons_per_s": None, "ratio_to_plain": None,
                    "iterations": {"plain": N_ITER, "learned": None, "saved": None}})
    return out


# ----------------------------------------------------------------------------
# reference arm: the CPU implementation of the same path
# ----------------------------------------------------------------------------
SAMPLE_ITERS = 5


def run_reference(args, rank):
    if rank != 0:
        return None
    from oracle import model as M
    from oracle import native
    from oracle import solvers as S
    threads = os.cpu_count() or 1
    if native.ref_available() and platform.machine() in ("x86_64", "AMD64"):
        lib, kind = native.ref(), "reference"
    else:
        lib, kind = native.port(), "port"
    lib.set_threads(threads)
    probe = M.config1_probe()
    grid = M.config_grid(N_GRID)
    om = M.Model(probe, grid, c=1500.0, lib=lib)
    om.norm = 2.0243e-05  # sigma_max of this geometry (power iteration); scales time not work
    rng = np.random.default_rng(1000)
    img = M.phantom(grid, rng)
    b = M.noisy_sinogram(om, img, rng).ravel()
    fwd = lambda v: om.forward(v.reshape(1, N_GRID, N_GRID)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, N_DET, -1)).ravel()
    times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        S.rec_nn_with_L2_reg(fwd, adj, b, N_GRID * N_GRID, SAMPLE_ITERS, LAMBDA)
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(dt)
    t_step = float(np.mean(times))
    value = (SAMPLE_ITERS / N_ITER) / t_step  # recons/s, extrapolated from the sample
    sample = (f"{SAMPLE_ITERS} of the {N_ITER} outer iterations of one instance per step, "
              f"{'reference MEX' if kind == 'reference' else 'C restatement of the MEX'} "
              f"kernels in FP64 numpy wrappers; recons/s = ({SAMPLE_ITERS}/{N_ITER}) / step time")
    return {
        "metric": METRIC, "value": value, "unit": "recons/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(1, 1), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "recons/s", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": value, "unit": "recons/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "host": platform.machine(),
    }


def fp32_nominal_tflops() -> float:
    """FP32 FMA-pipe rate of the current device at the measured maximum SM
    clock: SMs x 128 lanes x 2 flops x clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f)["sm_max_mhz"])
    except Exception:
        mhz = 2070.0
    return sms * 128 * 2 * float(mhz) * 1e6 / 1e12


def run_sweep(args):
    """Operator throughput sweep of the SIR model: A and A^T, FP32, on random
    non-negative images U[0, 1], grids 128^2 / 256^2 / 400^2 over the fixed
    25.4 mm FOV, 256 elements x 2030 samples, SPMR tables from 8 x 8
    point sources on a 0.25 mm x 10 mm flat element.  Times the interpolation
    kernels (the forwardMex / transposeMex equivalents) and the full operator
    with CUDA events, a 512 MB L2 flush between timed launches; reports the
    adjoint test, GB/s against the HBM peak and the FP32 rate."""
    import ctypes as C
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, _lib
    from msot_gb300.sir import spmr_tables
    from msot_gb300.synthetic import gauss_pulse_eir
    L = _lib.load()
    W = args.batch if args.batch != 64 else 8
    peak, peak_kind = peaks()
    flush = torch.empty(512 * 1024 * 1024 // 4, device="cuda")
    out = []
    for n in (128, 256, 400):
        probe = Probe(n_det=N_DET, radius=0.040, angular_coverage=135.0, fs=4e7, n_samples=N_T,
                      delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
        disc = Discretization([-0.0127, 0.0127], n)
        t0 = time.perf_counter()
        sir, se, idx, meta = spmr_tables(probe, disc, 1500.0, element=(0.25e-3, 10e-3, 0.0),
                                         sub=(8, 8))
        t_tab = time.perf_counter() - t0
        model = MSOTmodel(probe, disc, 1500.0, True, True, 0, 1e5, 12e6, 1.0,
                          sir_tables=(sir, se, idx), max_batch=W)
        gen = torch.Generator(device="cuda").manual_seed(n)
        x = torch.rand((W, n, n), device="cuda", generator=gen)
        ys = torch.randn((W, N_DET, N_T), device="cuda", generator=gen)
        raw = torch.empty((W, N_DET, N_T), device="cuda")
        xr = torch.empty((W, n, n), device="cuda")

        def interp_f():
            _lib.check(L.msot_interp_forward(model.plan, C.c_void_p(x.data_ptr()),
                                             C.c_void_p(raw.data_ptr()), W, None))

        def interp_t():
            _lib.check(L.msot_interp_transpose(model.plan, C.c_void_p(ys.data_ptr()),
                                               C.c_void_p(xr.data_ptr()), W, None))

        res = {}
        for name, fn in (("interp_forward", interp_f), ("interp_transpose", interp_t),
                         ("A", lambda: model.forward(x)), ("AT", lambda: model.transpose(ys))):
            for _ in range(args.warmup):
                fn()
            ms = []
            for _ in range(args.steps):
                flush.zero_()
                a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record()
                fn()
                z.record()
                torch.cuda.synchronize()
                ms.append(a.elapsed_time(z))
            res[name] = float(np.median(ms))
        y = model.forward(x)
        xa = model.transpose(ys)
        yd, sd = y.double(), ys.double()
        adj = abs(float((yd * sd).sum()) - float((x.double() * xa.double()).sum())) / (
            float(yd.norm()) * float(sd.norm()))
        P, NS, S = n * n, sir.shape[0], sir.shape[1]
        s_mean = float(np.mean((se[:, 1] - se[:, 0] + 1)[idx.ravel() - 1]))
        n_taps = 2.0 * model.radius
        alg_bytes = 4 * P * N_DET * 2 + 4 * S * NS + 4 * P * W + 4 * N_T * N_DET * W
        flops = 2.0 * P * N_DET * W * s_mean * n_taps
        line = {"sweep": "sir_operator", "grid": [n, n], "n_det": N_DET, "n_t": N_T,
                "batch": W, "spmr": {"n_sir": NS, "sir_len": S, "mean_support": s_mean,
                                      "build_s": t_tab},
                "ms": res, "adjoint_test": adj}
        for k in ("interp_forward", "interp_transpose"):
            sec = res[k] / 1e3
            line[k] = {"gbs": alg_bytes / sec / 1e9, "hbm_frac": alg_bytes / sec / 1e9 / peak,
                       "tflops": flops / sec / 1e12,
                       "fp32_frac_nominal": flops / sec / 1e12 / fp32_nominal_tflops()}
        line["peak_source"] = (f"{peak_kind} hbm_gbs (copy); "
                               f"FP32 nominal {fp32_nominal_tflops():.1f} TF/s")
        out.append(line)
        print(json.dumps(line), flush=True)
        del model
    return None


def oracle_tv_solve(model, b_np, n_iter, reg, threads):
    """FP64 oracle TV solve of one instance with the same model parameters."""
    from oracle import model as M
    from oracle import native
    from oracle import solvers as S
    native.port().set_threads(threads)
    g = model.Discretization
    p = model.Probe
    op = M.ArcProbe(n_det=p.n_det, radius=p.radius, coverage_deg=p.angular_coverage, fs=p.fs,
                    n_samples=p.n_samples, delay=p.delay, eir=p.eir, eir_length=p.eir_length)
    om = M.Model(op, M.Grid(g.nx, g.nz, g.fov), c=model.c, fmin=model.fmin, fmax=model.fmax,
                 norm=model.norm)
    fwd = lambda v: om.forward(v.reshape(1, g.nx, g.nz)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, p.n_det, -1)).ravel()
    t0 = time.perf_counter()
    rec = S.rec_nn_with_TV_reg(fwd, adj, b_np.astype(np.float64).ravel(), g.nx, g.nz, 1, n_iter,
                               reg)[0]
    return rec.reshape(g.nx, g.nz), time.perf_counter() - t0


def oracle_l1_solve(model, b_np, n_iter, reg, threads):
    """FP64 oracle L1 solve of one instance with the same model parameters."""
    from oracle import model as M
    from oracle import native
    from oracle import solvers as S
    native.port().set_threads(threads)
    g = model.Discretization
    p = model.Probe
    op = M.ArcProbe(n_det=p.n_det, radius=p.radius, coverage_deg=p.angular_coverage, fs=p.fs,
                    n_samples=p.n_samples, delay=p.delay, eir=p.eir, eir_length=p.eir_length)
    om = M.Model(op, M.Grid(g.nx, g.nz, g.fov), c=model.c, fmin=model.fmin, fmax=model.fmax,
                 norm=model.norm)
    fwd = lambda v: om.forward(v.reshape(1, g.nx, g.nz)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, p.n_det, -1)).ravel()
    t0 = time.perf_counter()
    rec = S.rec_nn_with_L1_eye_reg(fwd, adj, b_np.astype(np.float64).ravel(), n_iter, reg)[0]
    return rec.reshape(g.nx, g.nz), time.perf_counter() - t0


def run_l1(args):
    """Batched L1-regularised NNLS (rec_nn_with_L1_eye_reg): 64 instances of
    400 x 400 px (25.4 mm FOV), 512-element arc of radius 40 mm over 270 deg,
    4096 samples at 40 MHz, seeded disk + vessel phantoms with 1 % noise,
    regParam 1e-3, l1_iters outer iterations.  FP32 storage and arithmetic
    with FP64 inner products, norms and stopping tests.  Accuracy: instance 0
    solved with l1_check_iters (default l1_iters) iterations on the GPU and by
    the FP64 oracle on all host cores, which is also the CPU baseline."""
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, rec_nn_with_L1_eye_reg
    from msot_gb300 import _lib
    from msot_gb300.synthetic import gauss_pulse_eir, phantom_batch
    n, B, D, T, reg = args.l1_grid, 64, 512, 4096, 1e-3
    probe = Probe(n_det=D, radius=0.040, angular_coverage=270.0, fs=4e7, n_samples=T,
                  delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
    disc = Discretization([-0.0127, 0.0127], n)
    model = MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, None, max_batch=B)
    x = phantom_batch(disc, B, seed=404)
    y = model.forward(x)
    amp = y.abs().amax(dim=(1, 2), keepdim=True)
    gen = torch.Generator(device="cuda").manual_seed(405)
    b = (y + 0.01 * amp * torch.randn(y.shape, device="cuda", generator=gen)).contiguous()
    fmt = "fp16" if args.l1_fp16 else ("bf16" if args.l1_bf16 else "fp32")
    if fmt != "fp32":  # after the data: the sinograms come from the FP32 operator
        model.set_storage(fmt, args.l1_refine)
    L = _lib.load()
    for _ in range(max(1, args.warmup)):
        rec_nn_with_L1_eye_reg(model, b, args.l1_iters, reg)
    n0 = L.msot_launch_count()
    ms = []
    for _ in range(args.steps):
        ms.append(_event_ms(lambda: rec_nn_with_L1_eye_reg(model, b, args.l1_iters, reg))[1])
    launches = (L.msot_launch_count() - n0) // max(1, args.steps)
    ms_step = float(np.mean(ms))
    acc = None
    if not args.no_oracle:
        k = args.l1_check_iters or args.l1_iters
        g0 = rec_nn_with_L1_eye_reg(model, b[:1], k, reg)[0][0].cpu().numpy().astype(np.float64)
        ref, t_cpu = oracle_l1_solve(model, b[0].cpu().numpy(), k, reg, os.cpu_count() or 1)
        acc = {"instance": 0, "iterations": k,
               "rel_error_vs_fp64": float(np.linalg.norm(g0 - ref) / np.linalg.norm(ref)),
               "cpu_fp64_s": t_cpu, "cores": os.cpu_count()}
    cpu = None
    if acc and acc["iterations"] == args.l1_iters:
        cpu = {"value": 1.0 / acc["cpu_fp64_s"], "unit": "recons/s", "cores": os.cpu_count(),
               "kind": "port", "sample": "instance 0, FP64 oracle solve"}
    return {"mode": "l1_nnls", "metric": "L1-NNLS recons/s", "value": B / (ms_step / 1e3),
            "storage": ({"interp_input": fmt, "fp32_every": args.l1_refine}
                        if fmt != "fp32" else {"interp_input": "fp32"}),
            "cpu_baseline": cpu,
            "unit": "recons/s", "ms_per_step": ms_step, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "gpu_launches_per_step": launches,
            "accuracy": acc, "dtype": "f32 (FP64 inner products / norms / stopping tests)",
            "data": "synthetic seeded disk+vessel phantoms, 1% noise",
            "config": {"workload": f"rec_nn_with_L1_eye_reg, {n}x{n} px @25.4 mm FOV, 512-el "
                                   f"arc R=40 mm 270 deg, 4096 samples @40 MHz, EIR 257 taps, "
                                   f"regParam={reg}, {args.l1_iters} outer iterations",
                       "batch": B, "grid": [n, n], "n_det": D, "n_t": T}}


def run_bp(args):
    """backproject_waveeq (backproject_waveeq.m:1-50; the K(t, t') product on
    the tensor-core GEMM) and dmas_cf (dmas_cf.m:19-107) on 256 frames of
    256 detectors x 2030 samples, 128 x 128 px over the 25.4 mm FOV, psf 1,
    K = bp_kernel of the acquisition times; CUDA events around the calls."""
    import torch
    from msot_gb300.analytic import backproject_waveeq, bp_kernel_device, dmas_cf
    F, D, T, n = 256, N_DET, N_T, N_GRID
    g = torch.Generator(device="cuda").manual_seed(9)
    sig = torch.randn((F, D, T), device="cuda", generator=g)
    h = 0.2e-3 * 127 / 2
    x = np.linspace(-h, h, n)
    K = bp_kernel_device(np.arange(1, T + 1) / 4e7)
    bp = lambda: backproject_waveeq(sig, x, x, 1500.0, 4e7, 0.0, 135.0, 0.040,
                                    np.array([[1.0]]), K)
    dm = lambda: dmas_cf(sig, x, x, 1500.0, 4e7, 0.0, 135.0, 0.040)
    for _ in range(max(1, args.warmup)):
        bp(); dm()
    bp_ms = np.mean([_event_ms(bp)[1] for _ in range(args.steps)])
    dm_ms = np.mean([_event_ms(dm)[1] for _ in range(args.steps)])
    flops = 2.0 * T * T * D * F
    return {"mode": "analytic", "metric": "frames / s", "frames": F,
            "backproject_waveeq": {"ms_per_256_frames": bp_ms, "frames_per_s": F / (bp_ms / 1e3),
                                   "gemm_flops": flops,
                                   "gemm_tflops_fp32_equiv_upper_bound": flops / (bp_ms * 1e9)},
            "dmas_cf": {"ms_per_256_frames": dm_ms, "frames_per_s": F / (dm_ms / 1e3)},
            "steps": args.steps, "warmup": args.warmup, "dtype": "f32 (FP64 indices / sums)",
            "data": "synthetic Gaussian noise sinograms",
            "config": {"workload": f"{F} frames, {D} det x {T} samples, {n} x {n} px"}}


def run_prep(args):
    """Pre-processing of a batch of raw sinograms (64 instances x 256
    detectors x 2033 samples, crop 3 -> 2030): window (order-2 band-pass
    [300, T - 200]) and zero-phase filter (0.1-12 MHz at 40 MHz), CUDA
    events; the filter is the T x T circulant GEMM (2 T^2 flops per column)."""
    import torch
    from msot_gb300 import _lib
    from msot_gb300.preprocess import Preprocessor
    W, D, T_raw, n_crop = 64, N_DET, N_T + 3, 3
    T = T_raw - n_crop
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn((W, D, T_raw), device="cuda", generator=g)
    out = torch.empty((W, D, T), device="cuda")
    prep = Preprocessor(T_raw, n_crop, (2, 300.0, T - 200.0), 4e7, 1e5, 12e6, max_cols=W * D)
    for _ in range(args.warmup):
        prep(x, out)
    L = _lib.load()
    n0 = L.msot_launch_count()
    ms = _event_ms(lambda: [prep(x, out) for _ in range(args.steps)])[1] / args.steps
    flops = 2.0 * T * T * W * D
    return {"mode": "preprocess", "metric": "sinograms pre-processed / s",
            "value": W / (ms / 1e3), "unit": "sinograms/s", "ms_per_step": ms,
            "gemm_tflops": flops / (ms * 1e9), "steps": args.steps, "warmup": args.warmup,
            "gpu_launches_per_step": (L.msot_launch_count() - n0) // args.steps,
            "dtype": "f32", "data": "synthetic Gaussian noise",
            "config": {"workload": f"crop {n_crop}, window, zero-phase filter; "
                                   f"{W} x {D} x {T_raw}"}}


def run_tv(args):
    """Batched multispectral TV-regularised NNLS (rec_nn_with_TV_reg): 28
    wavelengths x 16 frames = 448 sinograms of 256 x 2030; each instance's
    grid is drawn uniformly from --tv-grids (25.4 mm FOV); each frame has
    2-3 chromophores (disk + vessel phantoms) with random positive spectra;
    1 % noise; lambda_TV = 5e-3, 100 outer iterations.  Instances of one grid
    size are solved in batches of up to --tv-batch; the value is instances / total
    device time of the solves (sinograms resident)."""
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, rec_nn_with_TV_reg
    from msot_gb300.synthetic import gauss_pulse_eir, phantom
    n_wl, n_fr, n_iter, reg, B = 28, 16, 100, 5e-3, args.tv_batch
    grids = [int(v) for v in args.tv_grids.split(",")]
    rng = np.random.default_rng(2024)
    grid_of = rng.choice(grids, size=(n_fr, n_wl))
    n_chrom = rng.integers(2, 4, size=n_fr)
    spectra = [rng.uniform(0.1, 1.0, size=(int(k), n_wl)) for k in n_chrom]
    probe = Probe(n_det=N_DET, radius=0.040, angular_coverage=135.0, fs=4e7, n_samples=N_T,
                  delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
    per_grid, total_ms, acc = {}, 0.0, None
    jobs = []  # (model, [sinogram batches]) per grid, kept for the concurrent run
    for n in grids:
        inst = [(f, l) for f in range(n_fr) for l in range(n_wl) if grid_of[f, l] == n]
        if not inst:
            continue
        disc = Discretization([-0.0127, 0.0127], n)
        model = MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, None, max_batch=B)
        tuning = model.autotune(B)
        maps = {}
        imgs = np.empty((len(inst), n, n), dtype=np.float32)
        for i, (f, l) in enumerate(inst):
            if f not in maps:
                maps[f] = [phantom(disc, np.random.default_rng(1000 * f + c))
                           for c in range(int(n_chrom[f]))]
            imgs[i] = sum(spectra[f][c, l] * maps[f][c] for c in range(int(n_chrom[f])))
        ms_grid = 0.0
        first_b = None
        batches = []
        for c0 in range(0, len(inst), B):
            x = torch.tensor(imgs[c0:c0 + B], device="cuda")
            y = model.forward(x)
            amp = y.abs().amax(dim=(1, 2), keepdim=True)
            gen = torch.Generator(device="cuda").manual_seed(n * 1000 + c0)
            y = (y + 0.01 * amp * torch.randn(y.shape, device="cuda", generator=gen)).contiguous()
            if first_b is None:
                first_b = y[0].cpu().numpy()
            rec_nn_with_TV_reg(model, y, 1, reg)  # plan/graph warm-up
            torch.cuda.synchronize()
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            rec = rec_nn_with_TV_reg(model, y, n_iter, reg)[0]
            z.record()
            torch.cuda.synchronize()
            ms_grid += a.elapsed_time(z)
            if n == min(grids) and c0 == 0:
                rec0 = rec[0].cpu().numpy().astype(np.float64)
            if args.tv_concurrent:
                batches.append(y)
        per_grid[str(n)] = {"instances": len(inst), "ms": ms_grid,
                            "recons_per_s": len(inst) / (ms_grid / 1e3), "autotune": tuning}
        total_ms += ms_grid
        if n == min(grids) and not args.no_oracle:
            ref, t_cpu = oracle_tv_solve(model, first_b, n_iter, reg, os.cpu_count() or 1)
            acc = {"grid": n, "rel_error_vs_fp64": float(np.linalg.norm(rec0 - ref) /
                                                         np.linalg.norm(ref)),
                   "cpu_fp64_s_per_recon": t_cpu}
        if args.tv_concurrent:
            jobs.append((model, batches))
        else:
            del model
            torch.cuda.empty_cache()
    n_all = n_wl * n_fr
    out = {"mode": "tv_multigrid", "metric": "TV-NNLS recons/s (mixed grids)",
           "value": n_all / (total_ms / 1e3), "unit": "recons/s", "instances": n_all,
           "iterations": n_iter, "lambda_tv": reg, "per_grid": per_grid, "accuracy": acc,
           "data": "synthetic multispectral disk+vessel phantoms, 1% noise",
           "note": f"batched per grid size (max {B} per call); not one persistent launch"}
    if args.tv_concurrent:
        # the grid sizes at once: one host thread per grid (the library call
        # releases the interpreter), each solve on its own stream; whole-job
        # wall time between device synchronisations
        from concurrent.futures import ThreadPoolExecutor

        def run_grid(job):
            model, batches = job
            torch.cuda.set_device(0)
            for y in batches:
                rec_nn_with_TV_reg(model, y, n_iter, reg)

        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(run_grid, jobs))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        out["serial_value"] = out["value"]
        out["value"] = n_all / wall
        out["note"] = ("grid sizes solved concurrently (one host thread and stream per grid, "
                       "batches of up to 64 per call); serial_value: one grid after another")
    return out


def _event_ms(fn):
    import torch
    a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record()
    out = fn()
    z.record()
    torch.cuda.synchronize()
    return out, a.elapsed_time(z)


def run_warmstart(args):
    """Learned warm start of the L2-NNLS solve: U-Net (4 levels, 32 base
    channels, BF16 weights, FP32 accumulate) trained on pairs the plain GPU
    solver generates (plain iterate after ws_input_iters iterations ->
    200-iteration solution, seeded disk + vessel phantoms, 1 % noise), then on
    ws_frames held-out frames: the accuracy target is the 200-iteration plain
    solve's relative distance to a 1000-iteration solve; the warm solve
    (input iterations + network + warm iterations) is scanned for the fewest
    warm iterations that reach it."""
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, reconstruct_dmas_cf, \
        rec_nn_with_L2_reg
    from msot_gb300 import _lib
    from msot_gb300.synthetic import gauss_pulse_eir, phantom_batch
    from msot_gb300.warmstart import LearnedWarmStart
    n, F, P = args.ws_grid, args.ws_frames, args.ws_pairs
    h = min(0.2e-3 * (n - 1) / 2, 0.2e-3 * 127 / 2)
    probe = Probe(n_det=N_DET, radius=0.040, angular_coverage=135.0, fs=4e7, n_samples=N_T,
                  delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
    model = MSOTmodel(probe, Discretization([-h, h], n), 1500.0, False, True, 0, 1e5, 12e6, None,
                      max_batch=64)
    ws = LearnedWarmStart(model, LAMBDA, levels=4, base_channels=32, max_batch=16,
                          input_iters=args.ws_input_iters, backprojection=args.ws_backprojection)
    L = _lib.load()
    imgs = phantom_batch(model.Discretization, P + F, seed=11)
    (f, t, b), pair_ms = _event_ms(lambda: ws.make_pairs(imgs, 200, seed=12))
    losses, train_ms = _event_ms(lambda: ws.fit(f[:P], t[:P], args.ws_train_steps, batch=16,
                                                lr=2e-3))
    del f, t
    bt = b[P:].contiguous()
    del b

    def solve(k):
        return torch.cat([rec_nn_with_L2_reg(model, bt[i:i + 64], k, LAMBDA)[0]
                          for i in range(0, F, 64)])
    xs = solve(1000)
    err = lambda x: float((x - xs).norm() / xs.norm())
    x200, plain_ms = _event_ms(lambda: solve(200))
    target = err(x200)
    # warm: input iterations + network + consistent multiplier, then k iterations
    ws.start(bt[:64])  # warm-up (graph capture of the input iterations)
    (w0, v0, fell), start_ms = _event_ms(lambda: ws.start(bt))
    net_ms = _event_ms(lambda: ws.net.forward(ws.features(bt)[0]))[1]
    rec_nn_with_L2_reg(model, bt[:64], 1, LAMBDA, x0=w0[:64], v0=v0[:64])  # warm-up
    scan, found = [], None
    for k in (5, 10, 20, 50, 100, 150, 200, 300):
        def warm():
            return torch.cat([rec_nn_with_L2_reg(model, bt[i:i + 64], k, LAMBDA, x0=w0[i:i + 64],
                                                 v0=v0[i:i + 64])[0] for i in range(0, F, 64)])
        r, ms = _event_ms(warm)
        e = err(r)
        scan.append({"warm_iterations": k, "rel_err": e, "ms": ms})
        if found is None and e <= target:
            found = (k, ms)
            break
    # iterations each start needs for the accuracy of k plain iterations
    plain_scan = []
    for k in (5, 10, 20, 50, 100, 150, 200):
        r, ms = _event_ms(lambda: solve(k))
        plain_scan.append({"iterations": k, "rel_err": err(r), "ms": ms})
    warm_errs = []
    for k in (0, 1, 2, 5, 10, 20, 50, 100, 150, 200, 300):
        if k == 0:
            warm_errs.append((0, err(w0)))
            continue
        r = torch.cat([rec_nn_with_L2_reg(model, bt[i:i + 64], k, LAMBDA, x0=w0[i:i + 64],
                                          v0=v0[i:i + 64])[0] for i in range(0, F, 64)])
        warm_errs.append((k, err(r)))
    crossover = []
    for p in plain_scan:
        need = next((k for k, e in warm_errs if e <= p["rel_err"]), None)
        crossover.append({"plain_iterations": p["iterations"], "rel_err": p["rel_err"],
                          "learned_input_plus_warm_iterations":
                              None if need is None else args.ws_input_iters + need})
    n0 = L.msot_launch_count()
    dm_ms = _event_ms(lambda: reconstruct_dmas_cf(model, bt))[1]
    dm_launches = L.msot_launch_count() - n0
    eq = err(solve(args.ws_input_iters + 10))
    warm_ms = start_ms + found[1] if found else None
    return {
        "metric": "learned-warm-start L2-NNLS recons/s at the 200-iteration plain accuracy",
        "value": F / (warm_ms / 1e3) if warm_ms else None, "unit": "recons/s",
        "plain_value": F / (plain_ms / 1e3), "higher_is_better": True,
        "iterations": {"plain": 200,
                       "warm": (args.ws_input_iters + found[0]) if found else None,
                       "saved": (200 - args.ws_input_iters - found[0]) if found else None},
        "accuracy_target_rel_err_vs_1000_it": target, "warm_scan": scan,
        "plain_scan": plain_scan, "iterations_to_plain_accuracy": crossover,
        "fallback_instances": int(fell.sum()),
        "equal_iterations": {"total": args.ws_input_iters + 10,
                             "plain_rel_err": eq, "warm_rel_err": scan[1]["rel_err"]
                             if len(scan) > 1 else None},
        "network_ms": net_ms, "start_ms": start_ms,
        "training": {"pairs": P, "pair_generation_s": pair_ms / 1e3, "steps": len(losses),
                     "batch": 16, "ms_per_step": train_ms / max(1, len(losses)),
                     "loss_first": float(np.mean(losses[:20])),
                     "loss_last": float(np.mean(losses[-100:]))},
        "dmas_cf": {"frames": F, "ms": dm_ms, "frames_per_s": F / (dm_ms / 1e3)},
        "dtype": "f32 solver; U-Net BF16 weights, FP32 accumulate",
        "data": "synthetic seeded disk+vessel phantoms, 1% noise",
        "config": {"workload": f"learned warm start, {n}x{n} px, {F} frames, 256-el arc, "
                               f"2030 samples, lambdaL2={LAMBDA}",
                   "grid": [n, n], "frames": F, "train_pairs": P,
                   "input_iterations": args.ws_input_iters,
                   "input": ("plain iterate" if args.ws_input_iters else
                             {"transpose": "A'b", "waveeq": "backproject_waveeq"}[
                                 args.ws_backprojection]),
                   "target_iterations": 200},
        "gpu_launches_dmas_cf": dm_launches,
    }


def unet_flops(L, c0, side):
    """Multiply-adds x 2 of one forward pass of the U-Net on one image."""
    ch = [c0 << l for l in range(L)]
    macs = 0
    for l in range(L):
        px = (side >> l) ** 2
        macs += px * 9 * ((1 if l == 0 else ch[l - 1]) * ch[l] + ch[l] * ch[l])
        if l + 1 < L:
            macs += px * 9 * ((ch[l + 1] + ch[l]) * ch[l] + ch[l] * ch[l])
    macs += side * side * c0
    return 2 * macs


def run_unet(args):
    """U-Net training step (forward + backward + Adam) and forward pass at
    batch 16 through the C-ABI, CUDA events; FLOPs of the 3x3/1x1
    convolutions (a training step counts 3x the forward)."""
    import torch
    from msot_gb300 import _lib
    from msot_gb300.warmstart import UNet
    S, B = args.unet_side, 16
    net = UNet(4, 32, S, B, seed=0)
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn((B, 1, S, S), device="cuda", generator=g)
    t = torch.randn((B, 1, S, S), device="cuda", generator=g)
    L = _lib.load()
    for _ in range(args.warmup):
        net.train_step(x, t, 1e-4)
    net.check()
    n0 = L.msot_launch_count()
    train_ms = _event_ms(lambda: [net.train_step(x, t, 1e-4) for _ in range(args.steps)])[1]
    launches = (L.msot_launch_count() - n0) // max(1, args.steps)
    fwd_ms = _event_ms(lambda: [net.forward(x) for _ in range(args.steps)])[1]
    net.check()
    train_ms /= args.steps
    fwd_ms /= args.steps
    fl = unet_flops(4, 32, S) * B
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            bf16 = float(json.load(f)["bf16_tflops"])
    except Exception:
        bf16 = None
    return {"metric": "U-Net training images/s", "value": B / (train_ms / 1e3), "unit": "images/s",
            "ms_per_step": train_ms, "forward_ms": fwd_ms,
            "forward_images_per_s": B / (fwd_ms / 1e3),
            "train_tflops": 3 * fl / (train_ms * 1e9), "forward_tflops": fl / (fwd_ms * 1e9),
            "peak_bf16_tflops_measured": bf16,
            "peak_tf32_tflops_est": bf16 / 2 if bf16 else None,
            "gpu_launches_per_step": launches,
            "higher_is_better": True, "steps": args.steps, "warmup": args.warmup,
            "dtype": "TF32 tensor-core convolutions (BF16 weights), FP32 accumulate",
            "data": "synthetic Gaussian images",
            "config": {"workload": f"U-Net 4 levels, 32 base channels, {S}x{S}, batch {B}"}}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank)
    elif args.op:
        import torch
        torch.cuda.set_device(0)
        out = run_operator(args)
    elif args.tv:
        import torch
        torch.cuda.set_device(0)
        out = run_tv(args)
    elif args.sweep:
        import torch
        torch.cuda.set_device(0)
        out = run_sweep(args)
    elif args.warmstart:
        import torch
        torch.cuda.set_device(0)
        out = run_warmstart(args)
    elif args.unet:
        import torch
        torch.cuda.set_device(0)
        out = run_unet(args)
    elif args.l1:
        import torch
        torch.cuda.set_device(0)
        out = run_l1(args)
    elif args.prep:
        import torch
        torch.cuda.set_device(0)
        out = run_prep(args)
    elif args.bp:
        import torch
        torch.cuda.set_device(0)
        out = run_bp(args)
    else:
        if world > 1:
            import torch
            import torch.distributed as dist
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
            dist.init_process_group("nccl")
        out = run_ours(args, rank, world)
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
    if rank == 0 and out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
