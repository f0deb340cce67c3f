"""FP64 numpy restatement of the reference's raw-sinogram pre-processing.

TEST INFRASTRUCTURE ONLY ("the oracle"): imported by tests/ only.

  * crop_first_n_signals.m:1-3
  * apply_butterworth_window_to_sinogram.m:1-10 (butter band-pass, zp2tf,
    freqz at T points of [0, pi), |h|)
  * filter_butter_zero_phase.m:16-48 (use_fft = true), via
    oracle.model.filter_butter_zero_phase
  * the chain of reconstruction_example_script.m:24-26

Arrays are (..., T) with time last (the reference's first axis).  The
Butterworth designs come from scipy.signal (the published bilinear design
MATLAB's butter also follows); no MATLAB run pins them (parity unpinned
against MATLAB itself).
"""
from __future__ import annotations

import numpy as np
import scipy.signal as sps

from . import model as M


def crop_first_n_signals(x, n):
    return np.asarray(x, dtype=np.float64)[..., int(n):]


def butter_window(T, n_butter, low, high):
    """|freqz(zp2tf(butter(n, [low high] / T, 'bandpass')), T)|."""
    z, p, k = sps.butter(n_butter, [low / T, high / T], "bandpass", output="zpk")
    b, a = sps.zpk2tf(z, p, k)
    _, h = sps.freqz(b, a, worN=T)
    return np.abs(h)


def apply_butterworth_window_to_sinogram(x, n_butter, low, high):
    x = np.asarray(x, dtype=np.float64)
    w = butter_window(x.shape[-1], n_butter, low, high)
    m = x.mean(axis=-1, keepdims=True)
    return m + (x - m) * w


def filter_butter_zero_phase(x, fs, fmin, fmax):
    x = np.asarray(x, dtype=np.float64)
    y = M.filter_butter_zero_phase(np.moveaxis(x, -1, 0), fs, fmin, fmax)
    return np.moveaxis(y, 0, -1)


def preprocess(x, n_crop, window, fs, fmin, fmax):
    """reconstruction_example_script.m:24-26; window = (order, low, high) or
    None."""
    y = crop_first_n_signals(x, n_crop)
    if window is not None:
        y = apply_butterworth_window_to_sinogram(y, *window)
    if fmin > 0 or fmax > 0:
        y = filter_butter_zero_phase(y, fs, fmin, fmax)
    return y
