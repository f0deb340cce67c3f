"""GPU parity of the analytic reconstructors against the FP64 oracle.

Bars: dmas_cf 1e-5 relative per output image (FP32 in/out, FP64 sums);
backproject_waveeq 1e-4 relative (its kernel product is an FP32 GEMM and the
divergence differentiates neighbouring pixels)."""
import numpy as np
import pytest

from oracle import backprojection as B
from pairs import rel

pytestmark = pytest.mark.gpu

GEOM = dict(c=1500.0, fs=4e7, n_crop=3.0, coverage=135.0, R=0.015)


def _data(W, D, T, seed):
    rng = np.random.default_rng(seed)
    sig = rng.standard_normal((W, D, T)).astype(np.float32)
    x = np.linspace(-0.003, 0.003, 30)
    z = np.linspace(-0.0028, 0.0028, 26)
    return sig, x, z


def test_dmas_cf_matches_oracle(cuda):
    import torch
    from msot_gb300 import dmas_cf
    sig, x, z = _data(2, 64, 900, 1)
    g = GEOM
    got = dmas_cf(torch.tensor(sig), x, z, g["c"], g["fs"], g["n_crop"], g["coverage"], g["R"])
    ref = B.dmas_cf(sig.astype(np.float64), x, z, g["c"], g["fs"], g["n_crop"], g["coverage"],
                    g["R"])
    for a, b in zip(got, ref):
        assert rel(a.cpu().numpy(), b) < 1e-5


def test_dmas_cf_rejects_index_outside_sinogram(cuda):
    import torch
    from msot_gb300 import _lib, dmas_cf
    sig, x, z = _data(1, 64, 300, 2)  # 300 samples do not reach the far pixels
    g = GEOM
    with pytest.raises(_lib.MsotError) as e:
        dmas_cf(torch.tensor(sig), x, z, g["c"], g["fs"], g["n_crop"], g["coverage"], g["R"])
    assert e.value.code == -2


def test_backproject_waveeq_matches_oracle(cuda):
    import torch
    from msot_gb300 import backproject_waveeq
    sig, x, z = _data(2, 48, 700, 3)
    g = GEOM
    Nt = 700 + int(g["n_crop"]) + 5
    t = np.arange(1, Nt + 1) / g["fs"]
    K = B.bp_kernel(t)
    psf = np.array([[1.0, 2.0, 1.0], [2.0, 4.0, 2.0], [1.0, 2.0, 1.0]])[:, :2]  # 3 x 2
    got = backproject_waveeq(torch.tensor(sig), x, z, g["c"], g["fs"], g["n_crop"],
                             g["coverage"], g["R"], psf, K).cpu().numpy()
    ref = B.backproject_waveeq(sig.astype(np.float64), x, z, g["c"], g["fs"], g["n_crop"],
                               g["coverage"], g["R"], psf, K)
    assert rel(got, ref) < 1e-4
