"""GPU solvers against the FP64 oracle solve of the same algorithm.
Bar (the headline metric's): relative error <= 1e-3 per instance."""
import numpy as np
import pytest

from oracle import model as M
from oracle import solvers as S
from pairs import make_pair, rel

pytestmark = pytest.mark.gpu


def _data(om, n, W, seed):
    rng = np.random.default_rng(seed)
    imgs, bs = [], []
    for _ in range(W):
        img = M.phantom(om.grid, rng)
        imgs.append(img)
        bs.append(M.noisy_sinogram(om, img, rng))
    return np.stack(imgs), np.stack(bs)


@pytest.fixture(scope="module")
def norm_pair(cuda):
    pm, om = make_pair(n=64, n_det=128, n_samples=1200, radius=0.02, fov_half=0.0063,
                       norm=1.0, max_batch=4)
    s = pm.estimate_sigma_max(100)
    pm2, om2 = make_pair(n=64, n_det=128, n_samples=1200, radius=0.02, fov_half=0.0063,
                         norm=s, max_batch=4)
    return pm2, om2


def test_l2_nnls_matches_fp64_oracle(norm_pair):
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    pm, om = norm_pair
    _, b = _data(om, 64, 3, 21)
    rec, e_img, e_reg, _, _, _ = rec_nn_with_L2_reg(pm, torch.tensor(b, dtype=torch.float32),
                                                    50, 1e-2)
    rec = rec.cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(1, 64, 64)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, 128, -1)).ravel()
    for w in range(3):
        ref, ref_img, ref_reg = S.rec_nn_with_L2_reg(fwd, adj, b[w].ravel(), 64 * 64, 50, 1e-2)
        assert rec[w].min() >= 0
        assert rel(rec[w], ref) <= 1e-3
        assert abs(e_img[w] - ref_img) / ref_img < 1e-3
        assert abs(e_reg[w] - ref_reg) / ref_reg < 1e-3


def test_l2_nnls_coupled_wavelengths(norm_pair):
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    pm, om = norm_pair
    _, b = _data(om, 64, 2, 22)
    rec = rec_nn_with_L2_reg(pm, torch.tensor(b, dtype=torch.float32), 20, 1e-2,
                             coupled=True)[0].cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(2, 64, 64)).ravel()
    adj = lambda y: om.transpose(y.reshape(2, 128, -1)).ravel()
    ref = S.rec_nn_with_L2_reg(fwd, adj, b.ravel(), 2 * 64 * 64, 20, 1e-2)[0]
    assert rel(rec, ref) <= 1e-3


def test_l2_warm_start_is_used(norm_pair):
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    pm, om = norm_pair
    img, b = _data(om, 64, 1, 23)
    bt = torch.tensor(b, dtype=torch.float32)
    cold = rec_nn_with_L2_reg(pm, bt, 2, 1e-2)[0]
    warm = rec_nn_with_L2_reg(pm, bt, 2, 1e-2, x0=torch.tensor(img, dtype=torch.float32))[0]
    assert rel(warm.cpu().numpy(), cold.cpu().numpy()) > 1e-2


def test_l1_nnls_matches_fp64_oracle(norm_pair):
    import torch
    from msot_gb300 import rec_nn_with_L1_eye_reg
    pm, om = norm_pair
    _, b = _data(om, 64, 2, 24)
    rec, e_img, e_reg, _, _ = rec_nn_with_L1_eye_reg(pm, torch.tensor(b, dtype=torch.float32),
                                                     15, 1e-3)
    rec = rec.cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(1, 64, 64)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, 128, -1)).ravel()
    for w in range(2):
        ref, ref_img, ref_reg = S.rec_nn_with_L1_eye_reg(fwd, adj, b[w].ravel(), 15, 1e-3)
        assert rel(rec[w], ref) <= 1e-3
        assert abs(e_img[w] - ref_img) / ref_img < 1e-3


def test_l2_warm_start_with_consistent_multiplier(norm_pair):
    # Seeding w alone restarts the splitting multiplier v at zero and the
    # iterates leave even an exact solution; seeding v from the fixed-point
    # relation (kkt_multiplier) keeps them there.
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.solvers import kkt_multiplier
    pm, om = norm_pair
    _, b = _data(om, 64, 2, 25)
    bt = torch.tensor(b, dtype=torch.float32)
    ref = rec_nn_with_L2_reg(pm, bt, 300, 1e-2)[0]
    w0, v0 = kkt_multiplier(pm, bt, ref, 1e-2)
    warm = rec_nn_with_L2_reg(pm, bt, 5, 1e-2, x0=w0, v0=v0)[0].cpu().numpy()
    w_only = rec_nn_with_L2_reg(pm, bt, 5, 1e-2, x0=w0)[0].cpu().numpy()
    r = ref.cpu().numpy()
    assert rel(warm, r) < 1e-2
    assert rel(warm, r) < 0.5 * rel(w_only, r)


def test_l1_nnls_512_elements_270deg_4096_samples(cuda):
    # the mixed-geometry L1 configuration (512-element arc over 270 degrees,
    # 4096 samples at 40 MHz, 25.4 mm FOV) on an 80 x 80 grid the oracle
    # solves in seconds; the full 400 x 400, 64-instance case is measured by
    # bench.py --l1 against the same oracle
    import torch
    from msot_gb300 import rec_nn_with_L1_eye_reg
    kw = dict(n=80, n_det=512, n_samples=4096, radius=0.040, coverage=270.0, fov_half=0.0127,
              max_batch=2)
    pm, _ = make_pair(norm=1.0, **kw)
    pm, om = make_pair(norm=pm.estimate_sigma_max(100), **kw)
    _, b = _data(om, 80, 2, 26)
    rec = rec_nn_with_L1_eye_reg(pm, torch.tensor(b, dtype=torch.float32), 20, 1e-3)[0]
    rec = rec.cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(1, 80, 80)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, 512, -1)).ravel()
    for w in range(2):
        ref = S.rec_nn_with_L1_eye_reg(fwd, adj, b[w].ravel(), 20, 1e-3)[0]
        assert rel(rec[w], ref) <= 1e-3


@pytest.mark.parametrize("shape", [(3, 37, 29), (1, 3, 5), (1, 2, 6), (2, 4, 4)])
def test_laplacian_per_wavelength_matches_oracle(cuda, shape):
    # MATLAB del2 semantics: interior second differences, ends extrapolated
    # linearly (n > 3), copied (n == 3), zero (n < 3); / 4
    import torch
    from msot_gb300.solvers import laplacian_per_wavelength
    x = np.random.default_rng(sum(shape)).standard_normal(shape)
    got = laplacian_per_wavelength(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    ref = S.laplacian_per_wavelength(x, shape[1], shape[2]).reshape(shape)
    assert np.max(np.abs(got - ref)) <= 1e-5 * max(1.0, np.abs(ref).max())


def test_l2_nnls_two_regularisers_matches_fp64_oracle(norm_pair):
    # the overview script's lambdaL2 = 5e-4 (identity) and lambdaL2_2 = 5e-3
    # (Laplacian, passed as its own transpose)
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.solvers import laplacian_per_wavelength
    pm, om = norm_pair
    _, b = _data(om, 64, 2, 27)
    rec, e_img, e_reg, e_reg2, _, _ = rec_nn_with_L2_reg(
        pm, torch.tensor(b, dtype=torch.float32), 30, 5e-4, "identity", "identity", 5e-3,
        laplacian_per_wavelength, laplacian_per_wavelength)
    rec = rec.cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(1, 64, 64)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, 128, -1)).ravel()
    for w in range(2):
        ref, r_img, r_reg, r_reg2 = S.rec_nn_with_L2_reg(fwd, adj, b[w].ravel(), 64 * 64, 30,
                                                         5e-4, lambdaL2_2=5e-3, shape=(64, 64))
        assert rel(rec[w], ref) <= 1e-3
        assert abs(e_img[w] - r_img) / r_img < 1e-3
        assert abs(e_reg[w] - r_reg) / r_reg < 1e-3
        assert abs(e_reg2[w] - r_reg2) / r_reg2 < 1e-3
    # the Laplacian changes the solution
    plain = rec_nn_with_L2_reg(pm, torch.tensor(b, dtype=torch.float32), 30, 5e-4)[0]
    assert rel(rec, plain.cpu().numpy()) > 1e-3


def test_l2_second_regulariser_needs_the_first(norm_pair):
    # incorporate_l2_reg_into_model_functions.m:8-22: with lambdaL2 = 0 the
    # Laplacian term is not used at all
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300.solvers import laplacian_per_wavelength
    pm, om = norm_pair
    _, b = _data(om, 64, 1, 28)
    bt = torch.tensor(b, dtype=torch.float32)
    a = rec_nn_with_L2_reg(pm, bt, 5, 0.0, None, None, 5e-3, laplacian_per_wavelength,
                           laplacian_per_wavelength)[0]
    p = rec_nn_with_L2_reg(pm, bt, 5, 0.0)[0]
    assert torch.equal(a, p)


def test_l2_solver_reports_nonfinite_data(norm_pair):
    """A NaN in one instance's sinogram: the solve returns MSOT_ENONFINITE
    naming that instance (the reference would return a NaN image silently),
    and the plan solves finite data normally afterwards."""
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    from msot_gb300._lib import MsotError
    pm, om = norm_pair
    _, b = _data(om, 64, 3, 23)
    bad = torch.tensor(b, dtype=torch.float32)
    bad[1, 5, 100] = float("nan")
    with pytest.raises(MsotError, match="non-finite residual .* instance 1"):
        rec_nn_with_L2_reg(pm, bad, 5, 1e-2)
    rec, e_img, _, _, _, _ = rec_nn_with_L2_reg(pm, torch.tensor(b, dtype=torch.float32), 5, 1e-2)
    assert torch.isfinite(rec).all() and np.isfinite(e_img).all()


def test_l1_solver_reports_nonfinite_data(norm_pair):
    """As for L2: a NaN in one instance's sinogram gives MSOT_ENONFINITE
    naming it, and finite data solve normally afterwards."""
    import torch
    from msot_gb300 import rec_nn_with_L1_eye_reg
    from msot_gb300._lib import MsotError
    pm, om = norm_pair
    _, b = _data(om, 64, 3, 24)
    bad = torch.tensor(b, dtype=torch.float32)
    bad[2, 7, 300] = float("inf")
    with pytest.raises(MsotError, match="non-finite residual .* instance 2"):
        rec_nn_with_L1_eye_reg(pm, bad, 3, 1e-3)
    rec, e_img, _, _, _ = rec_nn_with_L1_eye_reg(pm, torch.tensor(b, dtype=torch.float32), 3,
                                                 1e-3)
    assert torch.isfinite(rec).all() and np.isfinite(e_img).all()
