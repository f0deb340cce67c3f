"""GPU parity of the operator A / A^T against the oracle (FP32 vs FP64).

Bars: 1e-5 relative (L2 norm of the difference over the norm of the
reference output) for the MEX kernels and the full operator; adjoint test
|<Ax,y> - <x,A^T y>| / (||Ax|| ||y||) < 1e-6."""
import ctypes as C

import numpy as np
import pytest

from oracle import model as M
from oracle import native
from pairs import make_pair, rel

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


@pytest.mark.parametrize("W", [1, 5])
def test_mex_das_contract_matches_reference(cuda, golden, W):
    from msot_gb300 import _lib
    L = _lib.load()
    tau, r, T = golden["tau"], float(golden["radius"]), int(golden["T"])
    D, P = tau.shape
    img = np.ascontiguousarray(golden[f"das_img_w{W}"])
    out = np.empty((D, T, W))
    _lib.check(L.msot_mex_forwardDelayAndSum(_dp(img), W, P, _dp(tau), D, T, r, _dp(out)))
    assert rel(out, golden[f"das_fwd_w{W}"]) < TOL
    sig = np.ascontiguousarray(golden[f"das_sig_w{W}"])
    x = np.empty((P, W))
    _lib.check(L.msot_mex_transposeDelayAndSum(_dp(sig), W, T, D, _dp(tau), P, r, _dp(x)))
    assert rel(x, golden[f"das_adj_w{W}"]) < TOL


@pytest.mark.parametrize("W", [1, 3])
def test_mex_sir_contract_matches_reference(cuda, golden, W):
    from msot_gb300 import _lib
    L = _lib.load()
    g = golden
    r, T = float(g["radius"]), int(g["sir_T"])
    tau, idx, sir, se = g["sir_tau"], g["sir_idx"], g["sir"], g["sir_se"]
    D, P = tau.shape
    NS, S = sir.shape
    img = np.ascontiguousarray(g[f"sir_img_w{W}"])
    out = np.empty((D, T, W))
    _lib.check(L.msot_mex_forward(_dp(img), W, P, _ip(idx), _dp(tau), D, _dp(sir), S, NS, T,
                                  _ip(se), r, _dp(out)))
    assert rel(out, g[f"sir_fwd_w{W}"]) < TOL
    sig = np.ascontiguousarray(g[f"sir_sig_w{W}"])
    x = np.empty((P, W))
    _lib.check(L.msot_mex_transpose(_dp(sig), W, T, D, _ip(idx), _dp(tau), P, _dp(sir), S, NS,
                                    _ip(se), r, _dp(x)))
    assert rel(x, g[f"sir_adj_w{W}"]) < TOL


def test_mex_das_rejects_out_of_range(cuda, golden):
    from msot_gb300 import _lib
    L = _lib.load()
    tau = golden["tau"].copy()
    r, T = float(golden["radius"]), int(golden["T"])
    D, P = tau.shape
    tau[2, 5] = -1.0
    img = np.ones((P, 1))
    out = np.empty((D, T, 1))
    assert L.msot_mex_forwardDelayAndSum(_dp(img), 1, P, _dp(tau), D, T, r, _dp(out)) == -2


@pytest.fixture(scope="module")
def cfg1_pair(cuda):
    return make_pair(n=128, max_batch=4)


def test_interp_operator_config1_matches_port(cfg1_pair):
    import torch
    pm, om = cfg1_pair
    rng = np.random.default_rng(7)
    x = rng.random((2, 128 * 128))
    y = pm.interp_forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    ref = native.port().forward_das(x.T, om.travel, om.n_t, om.radius)
    assert rel(y, np.transpose(ref, (2, 0, 1))) < TOL
    s = rng.standard_normal((2, 256, 2030))
    xa = pm.interp_transpose(torch.tensor(s, dtype=torch.float32)).cpu().numpy()
    refa = native.port().transpose_das(np.ascontiguousarray(np.transpose(s, (1, 2, 0))),
                                       om.travel, om.radius)
    assert rel(xa, refa.T) < TOL


def test_full_operator_config1_matches_oracle(cfg1_pair):
    import torch
    pm, om = cfg1_pair
    rng = np.random.default_rng(8)
    x = rng.random((3, 128, 128))
    y = pm.Funcs.applyForward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < TOL
    s = rng.standard_normal((3, 256, 2030))
    xa = pm.Funcs.applyTranspose(torch.tensor(s, dtype=torch.float32)).cpu().numpy()
    assert rel(xa, om.transpose(s)) < TOL


def test_full_operator_adjoint_config1(cfg1_pair):
    import torch
    pm, _ = cfg1_pair
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.rand((4, 128, 128), device="cuda", generator=g)
    y = torch.randn((4, 256, 2030), device="cuda", generator=g)
    Ax = pm.forward(x).double()
    Aty = pm.transpose(y).double()
    lhs = (Ax * y.double()).sum().item()
    rhs = (x.double() * Aty).sum().item()
    err = abs(lhs - rhs) / (Ax.norm().item() * y.double().norm().item())
    assert err < 1e-6


def test_batch_equals_single_instances(cfg1_pair):
    import torch
    pm, _ = cfg1_pair
    x = torch.rand((4, 128, 128), device="cuda")
    yb = pm.forward(x)
    for w in range(4):
        ys = pm.forward(x[w:w + 1])
        assert rel(ys.cpu().numpy(), yb[w:w + 1].cpu().numpy()) < 1e-6


@pytest.mark.parametrize("n", [200, 101])
def test_full_operator_other_grids_match_oracle(cuda, n):
    import torch
    pm, om = make_pair(n=n, max_batch=2)
    rng = np.random.default_rng(n)
    x = rng.random((2, n, n))
    y = pm.forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < TOL
    s = rng.standard_normal((2, 256, 2030))
    xa = pm.transpose(torch.tensor(s, dtype=torch.float32)).cpu().numpy()
    assert rel(xa, om.transpose(s)) < TOL


def test_sir_operator_matches_oracle(cuda):
    import torch
    rng = np.random.default_rng(11)
    n, D = 48, 64
    S, NS = 41, 20
    sir = rng.standard_normal((NS, S))
    se = np.stack([rng.integers(1, 10, NS), rng.integers(S - 10, S + 1, NS)], 1).astype(np.int32)
    idx = rng.integers(1, NS + 1, (D, n * n)).astype(np.int32)
    pm, om = make_pair(n=n, n_det=D, n_samples=2030, max_batch=2, fov_half=0.005,
                       sir_tables=(sir, se, idx))
    x = rng.random((2, n, n))
    y = pm.forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < TOL
    s = rng.standard_normal((2, D, 2030))
    xa = pm.transpose(torch.tensor(s, dtype=torch.float32)).cpu().numpy()
    assert rel(xa, om.transpose(s)) < TOL


def test_norm_estimate_matches_oracle(cuda):
    pm, om = make_pair(n=64, n_det=128, n_samples=1600, norm=1.0, max_batch=1, fov_half=0.006)
    s_gpu = pm.estimate_sigma_max(200)
    s_ref = M.estimate_sigma_max(om.forward, om.transpose, (1, 64, 64), iters=200)
    assert abs(s_gpu - s_ref) / s_ref < 1e-4


def test_travel_times_on_gpu_match_oracle(cuda):
    # MSOTmodel.m:350-382 (single speed of sound) in FP64 on the GPU
    from msot_gb300 import Discretization, Probe
    from msot_gb300.model import travel_times
    for n, crop in ((128, 0), (57, 3)):
        tau = travel_times(Probe(), Discretization([-0.0127, 0.0127], n), 1500.0, crop)
        ref = M.travel_time_indices(M.config1_probe(), M.config_grid(n), 1500.0, crop)
        assert tau.shape == ref.shape
        assert np.max(np.abs(tau - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_autotune_keeps_results(cuda):
    # the autotuner only picks among variants that differ in float summation
    # order: the operator still matches the oracle, the solve its untuned self
    import torch
    from msot_gb300 import rec_nn_with_L2_reg
    pm, om = make_pair(n=48, n_det=64, n_samples=1200, radius=0.02, fov_half=0.0063, norm=1.0,
                       max_batch=8)
    rng = np.random.default_rng(8)
    x = rng.random((8, 48, 48))
    b = torch.tensor(om.forward(x), dtype=torch.float32)
    before = rec_nn_with_L2_reg(pm, b, 10, 1e-2)[0].cpu().numpy()
    t = pm.autotune(8)
    assert t["fwd_wt"] in (2, 4, 8) and t["conv_min_blocks"] in (1, 3, 4)
    assert t["adj_wt"] in (1, 2)
    assert t["tv_cluster"] in (0, 1, 2, 4, 8, 16)
    assert t["fwd_ms"] > 0 and t["transpose_ms"] > 0 and t["tv_prox_ms"] > 0
    y = pm.forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < 1e-5
    after = rec_nn_with_L2_reg(pm, b, 10, 1e-2)[0].cpu().numpy()
    assert rel(after, before) < 1e-5


def test_model_tables_from_disk_cache(cuda, tmp_path):
    # a second model of the same geometry loads the travel-time table written
    # by the first (acoustic_file_<key>.npz) and applies the same operator
    import os
    import torch
    from msot_gb300 import Discretization, MSOTmodel, Probe
    p = Probe(n_det=32, radius=0.02, n_samples=1200)
    d = Discretization([-0.004, 0.004], 32)
    m1 = MSOTmodel(p, d, 1500.0, model_normalization_factor=1.0, cache_dir=str(tmp_path))
    files = os.listdir(tmp_path)
    assert len(files) == 1 and files[0].startswith("acoustic_file_")
    m2 = MSOTmodel(p, d, 1500.0, model_normalization_factor=1.0, cache_dir=str(tmp_path))
    assert np.array_equal(m1.travel, m2.travel)
    x = torch.rand((1, 32, 32))
    assert torch.equal(m1.forward(x), m2.forward(x))


@pytest.mark.parametrize("W,fmt", [(8, "fp32"), (4, "fp32"), (16, "fp16"), (2, "fp32")])
def test_interleaved_entry_table_forward_is_bit_identical(cuda, W, fmt):
    # k_das_fwd3 on the per-warp interleaved entry table reads the same
    # entries of each bucket in the same order as on the CSR table
    import torch
    from msot_gb300 import _lib
    L = _lib.load()
    pm, _ = make_pair(n=64, n_det=128, n_samples=1200, radius=0.02, fov_half=0.0063,
                      max_batch=W)
    pm.set_storage(fmt)
    x = torch.rand((W, 64, 64), device="cuda", generator=torch.Generator("cuda").manual_seed(9))
    _lib.check(L.msot_tune_set(b"fwd_staged", 0))
    _lib.check(L.msot_tune_set(b"fwd_ell", 0))
    try:
        y_csr = pm.forward(x).cpu().numpy()
        _lib.check(L.msot_tune_set(b"fwd_ell", 1))
        y_ell = pm.forward(x).cpu().numpy()
    finally:
        _lib.check(L.msot_tune_set(b"fwd_ell", 1))
        _lib.check(L.msot_tune_set(b"fwd_staged", 1))
    assert np.array_equal(y_csr, y_ell)


def test_staged_forward_matches_the_per_detector_forward(cuda):
    # the staged kernel (pixel unions in shared memory, packed FMAs) sums the
    # same bucket moments as k_das_fwd3 on the CSR table
    import torch
    from msot_gb300 import _lib
    L = _lib.load()
    pm, _ = make_pair(n=64, n_det=128, n_samples=1200, radius=0.02, fov_half=0.0063,
                      max_batch=8)
    x = torch.rand((8, 64, 64), device="cuda", generator=torch.Generator("cuda").manual_seed(4))
    _lib.check(L.msot_tune_set(b"fwd_ell", 0))
    try:
        _lib.check(L.msot_tune_set(b"fwd_staged", 0))
        y_csr = pm.forward(x).cpu().numpy()
        _lib.check(L.msot_tune_set(b"fwd_staged", 1))
        y_st = pm.forward(x).cpu().numpy()
    finally:
        _lib.check(L.msot_tune_set(b"fwd_staged", 1))
        _lib.check(L.msot_tune_set(b"fwd_ell", 1))
    assert rel(y_st, y_csr) <= 1e-6
