"""Raw-sinogram pre-processing on the GPU (crop, Butterworth window,
zero-phase Butterworth filter) against the FP64 restatement
(oracle/preprocess.py).  Bar: 1e-5 relative (FP32 data, FP32 GEMM)."""
import numpy as np
import pytest

from oracle import preprocess as Q
from pairs import rel

pytestmark = pytest.mark.gpu

FS, FMIN, FMAX = 4e7, 1e5, 12e6


def _raw(W, D, T, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(T)
    # a few band-limited pulses on an offset, plus noise
    x = 0.3 + 0.01 * rng.standard_normal((W, D, T))
    for _ in range(4):
        t0 = rng.uniform(0.2 * T, 0.8 * T)
        x += rng.uniform(0.5, 1.5) * np.exp(-((t - t0) / 6.0) ** 2) * np.cos(0.8 * (t - t0))
    return x.astype(np.float32)


@pytest.mark.parametrize("T_raw,n_crop", [(2033, 3), (780, 3), (1024, 0)])
def test_preprocess_chain_matches_oracle(cuda, T_raw, n_crop):
    from msot_gb300.preprocess import Preprocessor
    x = _raw(2, 16, T_raw, T_raw)
    T = T_raw - n_crop
    win = (2, 300.0, T - 200.0) if T > 600 else (2, 40.0, T - 40.0)
    got = Preprocessor(T_raw, n_crop, win, FS, FMIN, FMAX, max_cols=32)(x).cpu().numpy()
    ref = Q.preprocess(x, n_crop, win, FS, FMIN, FMAX)
    assert got.shape == ref.shape
    assert rel(got, ref) <= 1e-5


def test_preprocess_stages_alone(cuda):
    from msot_gb300.preprocess import (apply_butterworth_window_to_sinogram,
                                       crop_first_n_signals, filter_butter_zero_phase)
    x = _raw(1, 8, 2030, 5)
    assert np.array_equal(crop_first_n_signals(x, 7).cpu().numpy(), x[..., 7:])
    w = apply_butterworth_window_to_sinogram(x, 2, 300, 1830).cpu().numpy()
    assert rel(w, Q.apply_butterworth_window_to_sinogram(x, 2, 300, 1830)) <= 1e-6
    for fmin, fmax in [(FMIN, FMAX), (0.0, FMAX), (FMIN, 0.0)]:
        f = filter_butter_zero_phase(x, FS, (fmin, fmax)).cpu().numpy()
        assert rel(f, Q.filter_butter_zero_phase(x, FS, fmin, fmax)) <= 1e-5
    with pytest.raises(NotImplementedError):
        filter_butter_zero_phase(x, FS, (FMIN, FMAX), use_fft=False)


def test_preprocess_for_model_chain(cuda):
    # reconstruction_example_script.m:24-26 with a model's crop and cut-offs
    from msot_gb300 import Discretization, MSOTmodel, Probe
    from msot_gb300.preprocess import preprocess_raw_data
    from msot_gb300.synthetic import gauss_pulse_eir
    probe = Probe(n_det=16, radius=0.040, angular_coverage=135.0, fs=FS, n_samples=2030,
                  delay=0.0, eir=gauss_pulse_eir(), eir_length=257)
    model = MSOTmodel(probe, Discretization([-0.003, 0.003], 32), 1500.0, False, True, 4,
                      FMIN, FMAX, 1.0, max_batch=1)
    x = _raw(1, 16, 2034, 9)
    got = preprocess_raw_data(model, x).cpu().numpy()
    ref = Q.preprocess(x, 4, (2, 300.0, 1830.0), FS, FMIN, FMAX)
    assert rel(got, ref) <= 1e-5


def test_preprocess_rejects_bad_arguments(cuda):
    from msot_gb300._lib import MsotError
    from msot_gb300.preprocess import Preprocessor
    with pytest.raises(MsotError):
        Preprocessor(100, 0, (2, 50.0, 40.0))          # low >= high
    with pytest.raises(MsotError):
        Preprocessor(100, 0, None, FS, 0.0, 0.6 * FS)  # above Nyquist
    with pytest.raises(MsotError):
        Preprocessor(10, 9)                             # fewer than 2 samples left
