"""Reduced-precision storage (msot_plan_set_storage): BF16 or scaled FP16
storage of the DAS forward's interpolation input with FP32 accumulation,
and the L1 solver's FP32 refinement iterations.  The operator differs from
the FP32 one by the rounding of the stored values (2^-9 relative for BF16,
2^-12 for FP16); the solves with it stay within the solves' 1e-3 bar of the
FP64 oracle: L1 on the 512-element, 270 deg, 4096-sample geometry of the
mixed-precision configuration, L2 (FP16) on the headline's probe."""
import os

import numpy as np
import pytest

from oracle import model as M
from oracle import solvers as S
from pairs import make_pair, rel

pytestmark = pytest.mark.gpu


def test_bf16_storage_changes_the_forward_by_bf16_rounding_only(cuda):
    torch = cuda
    pm, om = make_pair(n=96, n_det=128, n_samples=1600, radius=0.03, fov_half=0.0095,
                       norm=1.0, max_batch=8)
    x = torch.rand((8, 96, 96), device="cuda", generator=torch.Generator("cuda").manual_seed(5))
    y32 = pm.forward(x).cpu().numpy()
    pm.set_storage(True)
    y16 = pm.forward(x).cpu().numpy()
    pm.set_storage(False)
    assert np.array_equal(pm.forward(x).cpu().numpy(), y32)
    e = rel(y16, y32)
    assert 0 < e < 5e-3
    # the adjoint does not read the stored image
    s = torch.randn((8, 128, 1600), device="cuda")
    a32 = pm.transpose(s).cpu().numpy()
    pm.set_storage(True)
    assert np.array_equal(pm.transpose(s).cpu().numpy(), a32)


@pytest.mark.parametrize("n,iters,refine", [(80, 20, 0), (80, 20, 5), (400, 3, 0)])
def test_l1_with_bf16_storage_meets_the_solve_bar(cuda, n, iters, refine):
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, rec_nn_with_L1_eye_reg
    from msot_gb300.synthetic import gauss_pulse_eir
    from oracle import native
    native.port().set_threads(os.cpu_count() or 1)
    D, T = 512, 4096
    eir = gauss_pulse_eir()
    probe = Probe(n_det=D, radius=0.040, angular_coverage=270.0, fs=4e7, n_samples=T,
                  delay=0.0, eir=eir, eir_length=257)
    disc = Discretization([-0.0127, 0.0127], n)
    pm = MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, None, max_batch=1)
    op = M.ArcProbe(n_det=D, radius=0.040, coverage_deg=270.0, fs=4e7, n_samples=T, delay=0.0,
                    eir=eir, eir_length=257)
    om = M.Model(op, M.Grid(n, n, disc.fov), c=1500.0, fmin=1e5, fmax=12e6, norm=pm.norm)
    rng = np.random.default_rng(800 + n)
    b = M.noisy_sinogram(om, M.phantom(om.grid, rng), rng)[None]
    pm.set_storage(True, refine)
    rec = rec_nn_with_L1_eye_reg(pm, torch.tensor(b, dtype=torch.float32), iters, 1e-3)[0]
    fwd = lambda v: om.forward(v.reshape(1, n, n)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, D, -1)).ravel()
    ref = S.rec_nn_with_L1_eye_reg(fwd, adj, b[0].ravel(), iters, 1e-3)[0]
    assert rel(rec[0].cpu().numpy(), ref) <= 1e-3


def test_fp16_storage_rounding_and_power_of_two_scaling(cuda):
    # FP16 of the values times a power-of-two scale per instance: the
    # forward differs from FP32 by FP16 rounding only, and scaling an
    # instance by 2^+-60 (outside FP16's range unscaled) scales its output
    # exactly
    torch = cuda
    pm, om = make_pair(n=96, n_det=128, n_samples=1600, radius=0.03, fov_half=0.0095,
                       norm=1.0, max_batch=8)
    x = torch.rand((8, 96, 96), device="cuda", generator=torch.Generator("cuda").manual_seed(6))
    y32 = pm.forward(x).cpu().numpy()
    pm.set_storage("fp16")
    y16 = pm.forward(x).cpu().numpy()
    e = rel(y16, y32)
    assert 0 < e < 1e-3
    c = torch.tensor([2.0 ** 60, 2.0 ** -60, 1.0, 2.0 ** 20, 1.0, 1.0, 2.0 ** -30, 1.0],
                     device="cuda").view(8, 1, 1)
    yc = pm.forward(x * c).cpu().numpy()
    assert np.array_equal(yc, y16 * c.cpu().numpy().reshape(8, 1, 1))
    pm.set_storage("fp32")
    assert np.array_equal(pm.forward(x).cpu().numpy(), y32)
    with pytest.raises(ValueError):
        pm.set_storage("fp8")


def test_l2_with_fp16_storage_meets_the_solve_bar(cuda):
    # the headline's probe (256 elements, 135 deg, 2030 samples) at 64 x 64 px
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    n, D, T, iters, lam = 64, 256, 2030, 50, 1e-2
    pm, om = make_pair(n=n, n_det=D, n_samples=T, radius=0.040, fov_half=0.2e-3 * (n - 1) / 2,
                       max_batch=2)
    rng = np.random.default_rng(77)
    b = np.stack([M.noisy_sinogram(om, M.phantom(om.grid, rng), rng) for _ in range(2)])
    pm.set_storage("fp16")
    rec = rec_nn_with_L2_reg(pm, torch.tensor(b, dtype=torch.float32), iters, lam)[0]
    fwd = lambda v: om.forward(v.reshape(1, n, n)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, D, -1)).ravel()
    for w in range(2):
        ref = S.rec_nn_with_L2_reg(fwd, adj, b[w].ravel(), n * n, iters, lam)[0]
        assert rel(rec[w].cpu().numpy(), ref) <= 1e-3


def test_l1_with_fp16_storage_meets_the_solve_bar(cuda):
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, rec_nn_with_L1_eye_reg
    from msot_gb300.synthetic import gauss_pulse_eir
    from oracle import native
    native.port().set_threads(os.cpu_count() or 1)
    n, D, T, iters = 80, 512, 4096, 20
    eir = gauss_pulse_eir()
    probe = Probe(n_det=D, radius=0.040, angular_coverage=270.0, fs=4e7, n_samples=T,
                  delay=0.0, eir=eir, eir_length=257)
    disc = Discretization([-0.0127, 0.0127], n)
    pm = MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, None, max_batch=1)
    op = M.ArcProbe(n_det=D, radius=0.040, coverage_deg=270.0, fs=4e7, n_samples=T, delay=0.0,
                    eir=eir, eir_length=257)
    om = M.Model(op, M.Grid(n, n, disc.fov), c=1500.0, fmin=1e5, fmax=12e6, norm=pm.norm)
    rng = np.random.default_rng(880)
    b = M.noisy_sinogram(om, M.phantom(om.grid, rng), rng)[None]
    pm.set_storage("fp16")
    rec = rec_nn_with_L1_eye_reg(pm, torch.tensor(b, dtype=torch.float32), iters, 1e-3)[0]
    fwd = lambda v: om.forward(v.reshape(1, n, n)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, D, -1)).ravel()
    ref = S.rec_nn_with_L1_eye_reg(fwd, adj, b[0].ravel(), iters, 1e-3)[0]
    assert rel(rec[0].cpu().numpy(), ref) <= 1e-3
