"""Matched (GPU product, FP64 oracle) model pairs for the GPU parity tests."""
import numpy as np

from oracle import model as M


def rel(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_pair(n=128, n_det=256, n_samples=2030, radius=0.040, coverage=135.0, eir_taps=256,
              norm=2.0e-5, max_batch=4, fov_half=0.0127, sir_tables=None, c=1500.0):
    from msot_gb300 import Discretization, MSOTmodel, Probe
    eir = M.gauss_pulse_eir(n_taps=eir_taps) if eir_taps else None
    L = eir.size if eir is not None else 257
    op = M.ArcProbe(n_det=n_det, radius=radius, coverage_deg=coverage, n_samples=n_samples,
                    eir=eir, eir_length=L)
    og = M.Grid(n, n, (-fov_half, fov_half, -fov_half, fov_half))
    include_sir = sir_tables is not None
    om = M.Model(op, og, c=c, norm=norm, include_sir=include_sir, sir_tables=None)
    pp = Probe(n_det=n_det, radius=radius, angular_coverage=coverage, n_samples=n_samples,
               eir=eir, eir_length=L)
    pd = Discretization([-fov_half, fov_half], n)
    pm = MSOTmodel(pp, pd, c, include_sir=include_sir, model_normalization_factor=norm,
                   max_batch=max_batch,
                   sir_tables=None if sir_tables is None else
                   (sir_tables[0], sir_tables[1], sir_tables[2]))
    if include_sir:
        om.sir_tables = (sir_tables[0], sir_tables[1], sir_tables[2])
    return pm, om
