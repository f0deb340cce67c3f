"""FP64 numpy restatement of the reference's analytic reconstructors.

TEST INFRASTRUCTURE ONLY ("the oracle"): imported by tests/ only.

  dmas_cf            <- reconstruction_backprojection/dmas_cf.m:19-107
  backproject_waveeq <- reconstruction_backprojection/backproject_waveeq.m:1-50
  bp_kernel          <- reconstruction_backprojection/bp_kernel.m:1-12

MATLAB built-ins restated: round (half away from zero), cumtrapz, convn
'same', gradient/divergence (central differences inside, one-sided at the
borders, with the coordinate vectors), fliplr; besselh(0, .) is
scipy.special.hankel1(0, .).

Arrays follow the MATLAB layouts through numpy C-order views: sinogram
(W, D, T) == T x D x W; images (W, nx, nz) == Nz x Nx x W; the pixel grid is
the meshgrid of the coordinate vectors x (columns) and z (rows).
"""
from __future__ import annotations

import numpy as np
from scipy import special


def _round(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def transducer_angles(n_det, coverage):
    off = (180.0 - coverage) / 2.0
    step = coverage / (n_det - 1)
    return -(off + step * np.arange(n_det)) * np.pi / 180.0


def _sample_index(x, z, n_t, c, fs, n_crop, coverage, R, n_det):
    """(D, nx, nz) 0-based nearest sample indices (dmas_cf.m:69-74)."""
    ang = transducer_angles(n_det, coverage)
    acq1 = (1 + n_crop) / fs
    X, Z = np.meshgrid(x, z, indexing="ij")  # (nx, nz)
    idx = np.empty((n_det, X.shape[0], X.shape[1]), dtype=np.int64)
    for p in range(n_det):
        dist = np.sqrt(np.abs(X - np.cos(ang[p]) * R) ** 2 + np.abs(Z - np.sin(ang[p]) * R) ** 2)
        idx[p] = _round((dist / c - acq1) * fs + 1).astype(np.int64) - 1
    if idx.min() < 0 or idx.max() >= n_t:
        raise IndexError("sample index outside the sinogram (MATLAB would error)")
    return idx


def dmas_cf(sig_wdt, x, z, c, fs, n_crop, coverage, R):
    """Returns (dmas_cf, dmas, cf, das), each (W, nx, nz)."""
    sig = np.asarray(sig_wdt, dtype=np.float64)
    W, D, T = sig.shape
    sig = sig / np.abs(sig).max()
    ssq = np.sign(sig) * np.sqrt(np.abs(sig))
    idx = _sample_index(x, z, T, c, fs, n_crop, coverage, R, D)
    out = [np.zeros((W, len(x), len(z))) for _ in range(4)]
    for w in range(W):
        sos = np.zeros((len(x), len(z)))
        sqs = np.zeros_like(sos)
        num = np.zeros_like(sos)
        den = np.zeros_like(sos)
        for p in range(D):
            v = sig[w, p][idx[p]]
            vs = ssq[w, p][idx[p]]
            sos += vs ** 2
            sqs += vs
            num += v
            den += v ** 2
        das = num.copy()
        dmas = 0.5 * (sqs ** 2 - sos)
        cf = num ** 2 / (1e-6 + D * den)
        out[0][w], out[1][w], out[2][w], out[3][w] = dmas * cf, dmas, cf, das
    return tuple(out)


def cumtrapz_cols(t, y):
    """cumtrapz(t, y, 1) on (..., T) arrays (integration along the last axis)."""
    dt = np.diff(t)
    inc = 0.5 * dt * (y[..., 1:] + y[..., :-1])
    return np.concatenate([np.zeros(y.shape[:-1] + (1,)), np.cumsum(inc, axis=-1)], axis=-1)


def convn_same_td(sig_wdt, psf):
    """convn(sigMat, psf, 'same') with psf (m x n) over MATLAB's T x D
    dimensions of each wavelength; sig is (W, D, T), psf is MATLAB m x n
    (m along T, n along D)."""
    psf = np.atleast_2d(np.asarray(psf, dtype=np.float64))
    m, n = psf.shape
    W, D, T = sig_wdt.shape
    out = np.zeros_like(sig_wdt, dtype=np.float64)
    om, on = m // 2, n // 2
    for a in range(m):
        for b in range(n):
            # out[t][d] += psf[a][b] * sig[t + om - a][d + on - b]
            st, sd = om - a, on - b
            t0, t1 = max(0, -st), min(T, T - st)
            d0, d1 = max(0, -sd), min(D, D - sd)
            if t0 >= t1 or d0 >= d1:
                continue
            out[:, d0:d1, t0:t1] += psf[a, b] * sig_wdt[:, d0 + sd:d1 + sd, t0 + st:t1 + st]
    return out


def gradient_1d(f, h, axis):
    """MATLAB gradient along one axis with coordinate vector h."""
    f = np.moveaxis(f, axis, -1)
    g = np.empty_like(f)
    g[..., 1:-1] = (f[..., 2:] - f[..., :-2]) / (h[2:] - h[:-2])
    g[..., 0] = (f[..., 1] - f[..., 0]) / (h[1] - h[0])
    g[..., -1] = (f[..., -1] - f[..., -2]) / (h[-1] - h[-2])
    return np.moveaxis(g, -1, axis)


def backproject_waveeq(sig_wdt, x, z, c, fs, n_crop, coverage, R, psf, K):
    """backproject_waveeq.m:1-50 with fov_x = meshgrid of x (columns) and
    fov_y = meshgrid of z (rows).  K is the full kernel matrix
    (bp_kernel of the acquisition times including the cropped samples)."""
    sig = np.asarray(sig_wdt, dtype=np.float64)
    W, D, T = sig.shape
    dt = 1.0 / fs
    ang = transducer_angles(D, coverage)
    acq_samples = np.arange(1, T + 1) + int(round(n_crop))
    acq = acq_samples * dt
    s = cumtrapz_cols(acq, sig / c) / acq
    s = convn_same_td(s, psf) / np.asarray(psf, dtype=np.float64).sum()
    Kt = np.asarray(K, dtype=np.float64)[np.ix_(acq_samples - 1, acq_samples - 1)]
    idx = _sample_index(x, z, T, c, fs, n_crop, coverage, R, D)
    out = np.zeros((W, len(x), len(z)))
    for w in range(W):
        swl = (Kt @ s[w].T) * dt  # (T, D)
        px = np.zeros((len(x), len(z)))
        py = np.zeros_like(px)
        for p in range(D):
            v = swl[idx[p], p]
            px += v * np.cos(ang[p]) * dt * c
            py += v * np.sin(ang[p]) * dt * c
        # divergence: d(px)/dx along x (MATLAB columns) + d(py)/dy along z (rows)
        div = gradient_1d(px, np.asarray(x, dtype=np.float64), 0) + \
            gradient_1d(py, np.asarray(z, dtype=np.float64), 1)
        out[w] = div[::-1, :]  # fliplr: reverse the columns (x)
    return out


def bp_kernel(t):
    """bp_kernel.m:1-12: K = -imag(trapz(lambda, H0(t lambda) conj(H0(t' lambda)) lambda))."""
    t = np.asarray(t, dtype=np.float64).ravel()
    Nt = t.size
    dl = np.pi / (t[-1] - t[0])
    lam = dl * np.arange(1, Nt + 1)
    H = special.hankel1(0, t[:, None] * lam[None, :])  # (Nt, Nl)
    w = np.full(Nt, dl)
    w[0] = w[-1] = dl / 2  # trapezoid weights
    # K[j,k] = -Im sum_l w_l lam_l H[j,l] conj(H[k,l])
    M = (H * (w * lam)[None, :]) @ np.conj(H).T
    return -np.imag(M)
