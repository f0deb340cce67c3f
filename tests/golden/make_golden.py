"""Generate the golden vectors of the four operator MEX functions.

Runs the reference's own forwardDelayAndSumMex / transposeDelayAndSumMex /
forwardMex / transposeMex, compiled unmodified from the reference sources into
oracle/_ref/libmsotref.so (``make -C oracle ref``; x86_64 only), on small
seeded inputs, and stores inputs and FP64 outputs in mex_golden.npz.

    python tests/golden/make_golden.py

The reference has no test suite or fixtures of its own, so these vectors are
the pin of the oracle (oracle/msot_oracle.c must reproduce them bit for bit)
and of the GPU kernels (within FP32 tolerance).
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import native  # noqa: E402


def small_geometry(nx=24, nz=20, n_det=16, R=0.010, cov=150.0, c=1500.0, fs=4e7, pitch=0.15e-3):
    ang = np.deg2rad((180 - cov) / 2 + cov / (n_det - 1) * np.arange(n_det))
    xd, zd = R * np.cos(ang), -R * np.sin(ang)
    x = (np.arange(nx) - (nx - 1) / 2) * pitch
    z = (np.arange(nz) - (nz - 1) / 2) * pitch
    X, Z = np.repeat(x, nz), np.tile(z, nx)
    tau = np.hypot(xd[:, None] - X[None], zd[:, None] - Z[None]) / c * fs
    r = pitch * fs / c
    return np.ascontiguousarray(tau), r


def main():
    if not native.ref_available():
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    ref = native.ref()
    rng = np.random.default_rng(20261203)
    tau, r = small_geometry()
    D, P = tau.shape
    T = int(np.ceil(tau.max() + r)) + 40
    out = {"tau": tau, "radius": np.float64(r), "T": np.int32(T)}
    for W in (1, 5):
        img = rng.random((P, W))
        sig = rng.standard_normal((D, T, W))
        out[f"das_img_w{W}"] = img
        out[f"das_sig_w{W}"] = sig
        out[f"das_fwd_w{W}"] = ref.forward_das(img, tau, T, r)
        out[f"das_adj_w{W}"] = ref.transpose_das(sig, tau, r)
    # SIR: synthetic columns; travel times shifted so that some SIR taps fall
    # outside [0, T) and exercise the bounds check of forwardMex.cpp:139.
    S, NS = 31, 12
    sir = rng.standard_normal((NS, S))
    se = np.zeros((NS, 2), dtype=np.int32)
    for k in range(NS):
        a = int(rng.integers(1, S // 2))
        b = int(rng.integers(S // 2, S + 1))
        se[k] = (a, b)
    idx = rng.integers(1, NS + 1, size=(D, P)).astype(np.int32)
    tau_s = tau - (tau.min() - 3.0)  # earliest pixel 3 samples after t = 0
    Ts = int(np.ceil(tau_s.max())) + 5  # latest taps run past the end
    out.update(sir=sir, sir_se=se, sir_idx=idx, sir_tau=tau_s, sir_T=np.int32(Ts))
    for W in (1, 3):
        img = rng.random((P, W))
        sig = rng.standard_normal((D, Ts, W))
        out[f"sir_img_w{W}"] = img
        out[f"sir_sig_w{W}"] = sig
        out[f"sir_fwd_w{W}"] = ref.forward_sir(img, idx, tau_s, sir, Ts, se, r)
        out[f"sir_adj_w{W}"] = ref.transpose_sir(sig, idx, tau_s, sir, se, r)
    np.savez_compressed(os.path.join(HERE, "mex_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "mex_golden.npz"), {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
