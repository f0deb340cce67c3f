"""TV-regularised NNLS and its pieces on the GPU against the FP64 oracle.

  SB_ITV2 (split-Bregman isotropic TV prox) and ITV against
  oracle.solvers.sb_itv2 / itv; rec_nn_with_TV_reg against
  oracle.solvers.rec_nn_with_TV_reg (per instance and coupled wavelengths).
Bar: relative error <= 1e-3 (the headline metric's bar) for the
reconstructions and the prox; 1e-5 for the TV value itself.
"""
import numpy as np
import pytest

from oracle import model as M
from oracle import solvers as S
from pairs import make_pair, rel

pytestmark = pytest.mark.gpu


def _noisy_blocks(n, W, seed):
    rng = np.random.default_rng(seed)
    out = np.zeros((W, n, n))
    for w in range(W):
        for _ in range(4):
            a, b = sorted(rng.integers(0, n, 2))
            c, d = sorted(rng.integers(0, n, 2))
            out[w, a:b + 1, c:d + 1] += rng.uniform(0.3, 1.0)
        out[w] += 0.1 * rng.standard_normal((n, n))
    return out


# sizes cover the shared-memory cluster kernels (1 or 4 z-pixels per
# thread) with 1, 2, 4 (ragged last slab), 8 and 16 CTAs per image, and the
# 16-CTA cluster with its vectors in global memory (300)
@pytest.mark.parametrize("n,mu", [(32, 0.05), (64, 0.1), (50, 0.02), (90, 0.05), (128, 0.05),
                                  (200, 0.03), (300, 0.05)])
def test_sb_itv2_matches_oracle(cuda, n, mu):
    import torch
    from msot_gb300 import SB_ITV2
    W = 3 if n <= 128 else 1
    g = _noisy_blocks(n, W, 100 + n)
    u = SB_ITV2(torch.tensor(g, dtype=torch.float32), mu).cpu().numpy()
    B, Bt, BtB = S.diff_oper(n)
    for w in range(W):
        # images are [nx][nz] (p = ix*nz + iz): the oracle's column-major n x n view
        ref = S.sb_itv2(g[w].T, mu, B, Bt, BtB).reshape(n, n, order="F").T
        assert rel(u[w], ref) <= 1e-3


@pytest.mark.parametrize("n", [48, 128])
def test_sb_itv2_global_memory_kernel(cuda, n):
    # the fallback for images too large for shared memory, forced at small sizes
    import torch
    from msot_gb300 import SB_ITV2, _lib
    L = _lib.load()
    g = _noisy_blocks(n, 2, 300 + n)
    _lib.check(L.msot_tv_prox_path(1))
    try:
        u_glob = SB_ITV2(torch.tensor(g, dtype=torch.float32), 0.05).cpu().numpy()
    finally:
        _lib.check(L.msot_tv_prox_path(0))
    u_cl = SB_ITV2(torch.tensor(g, dtype=torch.float32), 0.05).cpu().numpy()
    B, Bt, BtB = S.diff_oper(n)
    for w in range(2):
        ref = S.sb_itv2(g[w].T, 0.05, B, Bt, BtB).reshape(n, n, order="F").T
        assert rel(u_glob[w], ref) <= 1e-3
        assert rel(u_cl[w], u_glob[w]) <= 1e-3


def test_sb_itv2_zero_mu(cuda):
    # mu = 0: no shrinkage; the iteration approaches g and stops at the
    # 1e-3 relative-change test, as the reference's does
    import torch
    from msot_gb300 import SB_ITV2
    n = 24
    g = _noisy_blocks(n, 2, 7)
    u = SB_ITV2(torch.tensor(g, dtype=torch.float32), 0.0).cpu().numpy()
    B, Bt, BtB = S.diff_oper(n)
    for w in range(2):
        ref = S.sb_itv2(g[w].T, 0.0, B, Bt, BtB).reshape(n, n, order="F").T
        assert rel(u[w], ref) <= 1e-3
        assert rel(u[w], g[w]) <= 2e-2


def test_sb_itv2_constant_image(cuda):
    # B u = 0 everywhere: the shrinkage meets |Bu + b| = 0 (0/0 in SB_ITV2.m:34)
    import torch
    from msot_gb300 import SB_ITV2
    g = np.full((1, 16, 16), 0.7)
    u = SB_ITV2(torch.tensor(g, dtype=torch.float32), 0.1).cpu().numpy()
    assert np.all(np.isfinite(u))
    assert rel(u, g) <= 1e-6


def test_itv_matches_oracle(cuda):
    import torch
    from msot_gb300 import ITV
    g = _noisy_blocks(40, 3, 5)
    v = ITV(torch.tensor(g, dtype=torch.float32))
    for w in range(3):
        assert abs(v[w] - S.itv(g[w].T)) / S.itv(g[w].T) <= 1e-5


@pytest.fixture(scope="module")
def tv_pair(cuda):
    pm, _ = make_pair(n=48, n_det=128, n_samples=1200, radius=0.02, fov_half=0.0063,
                      norm=1.0, max_batch=4)
    s = pm.estimate_sigma_max(100)
    return make_pair(n=48, n_det=128, n_samples=1200, radius=0.02, fov_half=0.0063,
                     norm=s, max_batch=4)


def _data(om, W, seed):
    rng = np.random.default_rng(seed)
    bs = []
    for _ in range(W):
        img = M.phantom(om.grid, rng)
        bs.append(M.noisy_sinogram(om, img, rng))
    return np.stack(bs)


def test_tv_nnls_matches_fp64_oracle(tv_pair):
    import torch
    from msot_gb300 import rec_nn_with_TV_reg
    pm, om = tv_pair
    n = 48
    b = _data(om, 2, 31)
    rec, e_img, e_reg, _, _ = rec_nn_with_TV_reg(pm, torch.tensor(b, dtype=torch.float32), 8,
                                                 2.5e-2)
    rec = rec.cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(1, n, n)).ravel()
    adj = lambda y: om.transpose(y.reshape(1, 128, -1)).ravel()
    for w in range(2):
        ref, ref_img, ref_reg = S.rec_nn_with_TV_reg(fwd, adj, b[w].ravel(), n, n, 1, 8, 2.5e-2)
        assert rec[w].min() >= 0
        assert rel(rec[w], ref) <= 1e-3
        assert abs(e_img[w] - ref_img) / ref_img < 1e-3
        assert abs(e_reg[w] - ref_reg) / ref_reg < 1e-3


def test_tv_nnls_coupled_wavelengths(tv_pair):
    import torch
    from msot_gb300 import rec_nn_with_TV_reg
    pm, om = tv_pair
    n = 48
    b = _data(om, 2, 32)
    rec = rec_nn_with_TV_reg(pm, torch.tensor(b, dtype=torch.float32), 5, 2.5e-2,
                             coupled=True)[0].cpu().numpy()
    fwd = lambda v: om.forward(v.reshape(2, n, n)).ravel()
    adj = lambda y: om.transpose(y.reshape(2, 128, -1)).ravel()
    ref = S.rec_nn_with_TV_reg(fwd, adj, b.ravel(), n, n, 2, 5, 2.5e-2)[0]
    assert rel(rec, ref) <= 1e-3


def test_tv_rejects_non_square_grid(cuda):
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe, rec_nn_with_TV_reg
    from msot_gb300._lib import MsotError
    eir = M.gauss_pulse_eir(n_taps=64)
    pm = MSOTmodel(Probe(n_det=64, radius=0.02, angular_coverage=135.0, n_samples=1000, eir=eir,
                         eir_length=eir.size),
                   Discretization([-0.003, 0.003, -0.0025, 0.0025], (48, 40)), 1500.0,
                   model_normalization_factor=1.0, max_batch=1)
    b = torch.zeros((1, 64, 1000), dtype=torch.float32, device="cuda")
    with pytest.raises(MsotError, match="square"):
        rec_nn_with_TV_reg(pm, b, 1, 1e-2)
