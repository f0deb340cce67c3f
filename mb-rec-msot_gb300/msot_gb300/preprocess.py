"""Raw-sinogram pre-processing on the GPU (msot_prep_*), mirroring the
reference's load_and_preprocess functions and the order in which
reconstruction_example_script.m:24-26 applies them.

Arrays are batches of columns with time last: a sinogram batch [W][D][T] is
MATLAB's T x D x W with the reference's first (time) axis fastest.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .model import _stream_ptr


def _columns(x):
    t = torch.as_tensor(x)
    if not t.is_cuda:
        t = t.cuda()
    return t.to(torch.float32).contiguous()


class Preprocessor:
    """msot_prep_create(T_raw, n_crop, window_order, window_low, window_high,
    fs, fmin, fmax, max_cols): crop, Butterworth window, zero-phase
    Butterworth filter (see include/msot_gpu.h)."""

    def __init__(self, n_samples_raw: int, n_crop: int = 0, window=None, fs: float = 0.0,
                 fmin: float = 0.0, fmax: float = 0.0, max_cols: int = 256 * 64):
        order, lo, hi = window if window is not None else (0, 0.0, 0.0)
        h = C.c_void_p()
        _lib.check(_lib.load().msot_prep_create(int(n_samples_raw), int(n_crop), int(order),
                                                float(lo), float(hi), float(fs), float(fmin),
                                                float(fmax), int(max_cols), C.byref(h)))
        self._h = h
        self.n_samples_raw, self.n_crop, self.max_cols = int(n_samples_raw), int(n_crop), max_cols

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.load().msot_prep_destroy(self._h)
            self._h = None

    def __call__(self, data_raw, out=None, stream=None):
        x = _columns(data_raw)
        if x.shape[-1] != self.n_samples_raw:
            raise ValueError(f"last axis {x.shape[-1]} != {self.n_samples_raw} samples")
        n_cols = x.numel() // self.n_samples_raw
        T = self.n_samples_raw - self.n_crop
        if out is None:
            out = torch.empty((*x.shape[:-1], T), device=x.device, dtype=torch.float32)
        flat_in, flat_out = x.reshape(n_cols, -1), out.reshape(n_cols, T)
        for c0 in range(0, n_cols, self.max_cols):
            c1 = min(n_cols, c0 + self.max_cols)
            _lib.check(_lib.load().msot_prep_apply(
                self._h, C.c_void_p(flat_in[c0:c1].data_ptr()),
                C.c_void_p(flat_out[c0:c1].data_ptr()), c1 - c0, _stream_ptr(stream)))
        return out


def crop_first_n_signals(data_raw, n_signals_to_crop: int):
    """crop_first_n_signals.m:1-3 (time is the last axis here)."""
    x = _columns(data_raw)
    return x[..., int(n_signals_to_crop):].contiguous()


def apply_butterworth_window_to_sinogram(sinograms, n_butter: int, low_cutoff: float,
                                         high_cutoff: float):
    """apply_butterworth_window_to_sinogram.m:1-10: cut-offs in samples."""
    x = _columns(sinograms)
    p = Preprocessor(x.shape[-1], 0, (n_butter, low_cutoff, high_cutoff),
                     max_cols=max(1, x.numel() // x.shape[-1]))
    return p(x)


def filter_butter_zero_phase(signal_matrix, sampling_frequency: float, filter_frequencies,
                             use_fft: bool = True):
    """filter_butter_zero_phase.m:1-53 with use_fft = true (the filtfilt
    branch is not provided)."""
    if not use_fft:
        raise NotImplementedError("only the FFT-domain (use_fft = true) branch is provided")
    fmin, fmax = (float(v) for v in filter_frequencies)
    x = _columns(signal_matrix)
    if fmin <= 0 and fmax <= 0:
        return x.clone()
    p = Preprocessor(x.shape[-1], 0, None, sampling_frequency, fmin, fmax,
                     max_cols=max(1, x.numel() // x.shape[-1]))
    return p(x)


def preprocess_raw_data(model, data_raw, window_order: int = 2, window_low: float = 300.0,
                        window_margin: float = 200.0):
    """reconstruction_example_script.m:24-26 for an MSOTmodel: crop the
    model's cropped samples, window with the order-2 band-pass [300, T - 200],
    zero-phase filter with the model's cut-offs."""
    x = _columns(data_raw)
    T = x.shape[-1] - int(model.n_crop)
    p = Preprocessor(x.shape[-1], int(model.n_crop), (window_order, window_low, T - window_margin),
                     model.Probe.fs, model.fmin, model.fmax,
                     max_cols=max(1, x.numel() // x.shape[-1]))
    return p(x)


def butter_response(order: int, btype: str, wn, n: int, whole: bool = False) -> np.ndarray:
    """|H| of the library's Butterworth design (msot_butter_response; host
    only, no GPU needed)."""
    types = {"low": 0, "high": 1, "bandpass": 2}
    w = np.atleast_1d(np.asarray(wn, dtype=np.float64))
    out = np.empty(int(n), dtype=np.float64)
    _lib.check(_lib.load().msot_butter_response(
        int(order), types[btype], float(w[0]), float(w[1]) if w.size > 1 else 0.0, int(n),
        1 if whole else 0, out.ctypes.data_as(C.POINTER(C.c_double))))
    return out
