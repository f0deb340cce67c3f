"""SPMR table generator on the GPU against the FP64 numpy restatement, and the
SIR operator built on the generated tables against the oracle operator.

The reference's own tables come from Field II (absent), so the generator is
pinned to oracle/sir.py; the operator bars are the usual ones (1e-5
relative, adjoint test 1e-6)."""
import numpy as np
import pytest

from oracle import sir as Q
from pairs import make_pair, rel

pytestmark = pytest.mark.gpu


def _geometry(n, D, fov_half, n_samples=2030):
    from msot_gb300 import Discretization, Probe
    p = Probe(n_det=D, radius=0.040, angular_coverage=135.0, n_samples=n_samples)
    d = Discretization([-fov_half, fov_half], n)
    return p, d


@pytest.mark.parametrize("n,D,elev", [(24, 24, 0.040), (20, 16, 0.0)])
def test_spmr_tables_match_oracle(cuda, n, D, elev):
    from msot_gb300.sir import spmr_tables
    p, d = _geometry(n, D, 0.0127)
    sir, se, idx, meta = spmr_tables(p, d, 1500.0, element=(0.25e-3, 10e-3, elev), sub=(4, 4),
                                     half_window=60)
    ref, rse, ridx, info = Q.spmr_tables(D, 0.040, 135.0, d.x, d.z, 1500.0, p.fs, d.sigma,
                                         0.25e-3, 10e-3, elev, 4, 4,
                                         half_window=meta["half_window"])
    assert meta["n_dist"] == info["n_dist"] and meta["n_angle"] == info["n_angle"]
    assert abs(meta["d_min"] - info["d_min"]) <= 1e-15
    assert sir.shape == ref.shape
    assert rel(sir, ref) <= 1e-9
    assert np.array_equal(se, rse)
    assert np.array_equal(idx, ridx)


def test_sir_operator_on_generated_tables(cuda):
    # config-2 style: 8 x 8 sub-element sampling of a 0.25 mm x 10 mm element
    import torch
    from msot_gb300.sir import spmr_tables
    n, D, fov_half = 40, 64, 0.004
    p, d = _geometry(n, D, fov_half)
    sir, se, idx, _ = spmr_tables(p, d, 1500.0, element=(0.25e-3, 10e-3, 0.0), sub=(8, 8))
    pm, om = make_pair(n=n, n_det=D, n_samples=2030, max_batch=2, fov_half=fov_half,
                       sir_tables=(sir, se, idx))
    rng = np.random.default_rng(3)
    x = rng.random((2, n, n))
    y = pm.forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < 1e-5
    s = rng.standard_normal((2, D, 2030))
    xa = pm.transpose(torch.tensor(s, dtype=torch.float32)).cpu().numpy()
    assert rel(xa, om.transpose(s)) < 1e-5
    # adjoint test on the GPU operator
    lhs = float(np.vdot(y, s))
    rhs = float(np.vdot(x, xa))
    assert abs(lhs - rhs) / (np.linalg.norm(y) * np.linalg.norm(s)) < 1e-6
