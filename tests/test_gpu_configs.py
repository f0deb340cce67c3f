"""The configured workloads under the GPU parity bar.  Each GPU solve is
checked against the FP64 oracle solve of the same algorithm on the same
data, at <= 1e-3 relative error per instance (the metric's bar):

  * rec_nn_with_L2_reg at the headline configuration: 128 x 128 px at
    0.2 mm, 256-element arc of radius 40 mm over 135 deg, 2030 samples at
    40 MHz, EIR 257 taps, cut-offs [0.1, 12] MHz, lambdaL2 = 1e-2, 50 outer
    iterations, four distinct disk + vessel phantoms (1 % noise) solved in
    one batched call (nnls_L2_less.m:51-72 per instance);
  * rec_nn_with_L1_eye_reg on the 400 x 400 px geometry of the mixed-
    precision configuration: 25.4 mm FOV, 512-element arc over 270 deg,
    4096 samples, regParam 1e-3; one instance, 3 outer iterations
    (nnls_L1_eye_matrix_less.m:38-54);
  * rec_nn_with_TV_reg at 256 x 256 and 400 x 400 px (25.4 mm FOV, the
    headline probe), lambda_TV = 5e-3; one instance each, 3 outer
    iterations (nnls_sparsa_based_reg_matrix_less.m:31-85).

The model normalisation is the GPU's power-iteration estimate, passed to the
oracle model as well, as one model factor serves both sides.
"""
import os

import numpy as np
import pytest

from oracle import model as M
from oracle import solvers as S
from pairs import rel

pytestmark = pytest.mark.gpu


def _models(n, n_det, n_t, coverage, max_batch, fov_half):
    """GPU MSOTmodel and the matching FP64 oracle model (same probe, grid,
    IR, cut-offs and normalisation factor)."""
    from msot_gb300 import Discretization, MSOTmodel, Probe
    from msot_gb300.synthetic import gauss_pulse_eir
    from oracle import native
    native.port().set_threads(os.cpu_count() or 1)
    eir = gauss_pulse_eir()
    probe = Probe(n_det=n_det, radius=0.040, angular_coverage=coverage, fs=4e7,
                  n_samples=n_t, delay=0.0, eir=eir, eir_length=257)
    disc = Discretization([-fov_half, fov_half], n)
    pm = MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, None, max_batch=max_batch)
    op = M.ArcProbe(n_det=n_det, radius=0.040, coverage_deg=coverage, fs=4e7, n_samples=n_t,
                    delay=0.0, eir=eir, eir_length=257)
    om = M.Model(op, M.Grid(n, n, disc.fov), c=1500.0, fmin=1e5, fmax=12e6, norm=pm.norm)
    return pm, om


def _data(om, W, seed):
    rng = np.random.default_rng(seed)
    return np.stack([M.noisy_sinogram(om, M.phantom(om.grid, rng), rng) for _ in range(W)])


def _ops(om, n, n_det):
    fwd = lambda v: om.forward(v.reshape(1, n, n)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, n_det, -1)).ravel()
    return fwd, adj


def test_l2_headline_configuration_four_phantoms(cuda):
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    n, D, T, iters, lam = 128, 256, 2030, 50, 1e-2
    pm, om = _models(n, D, T, 135.0, 4, 0.2e-3 * 127 / 2)
    b = _data(om, 4, 2031)
    rec, e_img, e_reg, _, _, _ = rec_nn_with_L2_reg(pm, torch.tensor(b, dtype=torch.float32),
                                                    iters, lam)
    rec = rec.cpu().numpy()
    fwd, adj = _ops(om, n, D)
    for w in range(4):
        ref, r_img, r_reg = S.rec_nn_with_L2_reg(fwd, adj, b[w].ravel(), n * n, iters, lam)
        assert rec[w].min() >= 0
        assert rel(rec[w], ref) <= 1e-3, w
        assert abs(e_img[w] - r_img) / r_img < 1e-3
        assert abs(e_reg[w] - r_reg) / r_reg < 1e-3
    # four distinct phantoms: the instances are not copies of one another
    assert min(rel(rec[i], rec[j]) for i in range(4) for j in range(i)) > 0.1


def test_l1_400px_512_elements_270deg_4096_samples(cuda):
    import torch
    from msot_gb300 import rec_nn_with_L1_eye_reg
    n, D, T, iters, reg = 400, 512, 4096, 3, 1e-3
    pm, om = _models(n, D, T, 270.0, 1, 0.0127)
    b = _data(om, 1, 4096)
    rec, e_img, _, _, _ = rec_nn_with_L1_eye_reg(pm, torch.tensor(b, dtype=torch.float32),
                                                 iters, reg)
    fwd, adj = _ops(om, n, D)
    ref, r_img, _ = S.rec_nn_with_L1_eye_reg(fwd, adj, b[0].ravel(), iters, reg)
    assert rel(rec[0].cpu().numpy(), ref) <= 1e-3
    assert abs(e_img[0] - r_img) / r_img < 1e-3


@pytest.mark.parametrize("n", [256, 400])
def test_tv_at_configured_grid_sizes(cuda, n):
    import torch
    from msot_gb300 import rec_nn_with_TV_reg
    D, T, iters, reg = 256, 2030, 3, 5e-3
    pm, om = _models(n, D, T, 135.0, 1, 0.0127)
    b = _data(om, 1, 5000 + n)
    rec = rec_nn_with_TV_reg(pm, torch.tensor(b, dtype=torch.float32), iters, reg)[0]
    fwd, adj = _ops(om, n, D)
    ref = S.rec_nn_with_TV_reg(fwd, adj, b[0].ravel(), n, n, 1, iters, reg)[0]
    assert rel(rec[0].cpu().numpy(), ref.reshape(n, n)) <= 1e-3
