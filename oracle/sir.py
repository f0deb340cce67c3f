"""FP64 numpy restatement of the SPMR (spatial pixel model response) table
generator.

TEST INFRASTRUCTURE ONLY ("the oracle"): imported by tests/ only.

Follows is_tir_derivation/calculate_polarSPMR.m:21-184 and
MSOTmodel.m:463-480, 586-613 (2-D, single speed of sound).  The reference
takes the element's spatial impulse response from Field II (calc_h), which
is not available; as in the GPU generator it is the Rayleigh integral over
sub_x x sub_y point sources (weight area / (2 pi R)).  Parity with the
reference's own tables is therefore unpinned; the GPU generator is pinned to
this restatement.
"""
from __future__ import annotations

import numpy as np

FSF = 5e9  # calculate_polarSPMR.m:35
NF = 1 << 16


def nshape_filtered(sigma, c, fs):
    """calculate_polarSPMR.m:56-75: q(t) = phi(c t)(-t) at 5 GHz, times the
    squared magnitude of the order-8 Butterworth low pass at fs/2 (bilinear
    form: 1 / (1 + (tan(pi f/fsF) / tan(pi fc/fsF))^16)), circular on NF
    points.  Returns (g, M) with g[m + M] for m = -M .. M + 1."""
    phi = lambda r: np.exp(-r * r / (2.0 * sigma * sigma))
    hq = 200
    if not abs(phi(hq / FSF * c)) < 1e-3:
        for tb in np.arange(1.0, 5.0001, 0.25) * 1e-7:
            if abs(phi(tb * c)) < 1e-3:
                hq = int(np.ceil(tb * FSF))
                break
    a = np.zeros(NF)
    j = np.arange(-hq, hq + 1)
    t = j / FSF
    a[j % NF] = phi(t * c) * (-t)
    A = np.fft.fft(a)
    f = np.arange(NF) / NF
    with np.errstate(divide="ignore", over="ignore"):
        ratio = np.tan(np.pi * f) / np.tan(np.pi * (fs / 2.0) / FSF)
        h2 = 1.0 / (1.0 + ratio ** 16)
    h2[NF // 2] = 0.0
    g = np.real(np.fft.ifft(A * h2))
    M = NF // 2 - 1
    m = np.arange(-M, M + 2)
    return g[m % NF], M


def sources(width, height, elev_radius, sx, sy):
    """Sub-element centres (x along the array, y elevation, z towards the
    field) and areas; curved in elevation with radius elev_radius (0 = flat)."""
    dx, dy = width / sx, height / sy
    out = []
    for i in range(sx):
        for jj in range(sy):
            x = -width / 2 + (i + 0.5) * dx
            y = -height / 2 + (jj + 0.5) * dy
            z, area = 0.0, dx * dy
            if elev_radius > 0:
                s = np.sqrt(elev_radius ** 2 - y * y)
                z = elev_radius - s
                area = dx * dy * elev_radius / s
            out.append((x, y, z, area))
    return np.array(out)


def _round(v):
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def spmr_tables(n_det, radius, coverage_deg, x, z, c, fs, sigma, width, height, elev_radius,
                sx, sy, half_window=45, virtual=None):
    """Returns (sir [NS][S], start_end [NS][2] 1-based, idx [D][P] 1-based,
    info dict).  virtual = (virt_x, virt_z) [D][P] replaces the pixels in the
    polar mapping (two speeds of sound, MSOTmodel.m:579-596; c is then the
    coupling medium's speed)."""
    x = np.asarray(x, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    off = (180.0 - coverage_deg) / 2.0
    ang = (off + coverage_deg / (n_det - 1) * np.arange(n_det)) * np.pi / 180.0
    xd, zd = radius * np.cos(ang), -radius * np.sin(ang)
    X, Z = np.meshgrid(x, z, indexing="ij")
    X, Z = X.ravel(), Z.ravel()  # p = ix * nz + iz
    if virtual is not None:
        ax = xd[:, None] - np.asarray(virtual[0], dtype=np.float64)
        az = zd[:, None] - np.asarray(virtual[1], dtype=np.float64)
    else:
        ax = xd[:, None] - X[None, :]
        az = zd[:, None] - Z[None, :]
    r = np.sqrt(ax * ax + az * az)
    nd = np.sqrt(xd * xd + zd * zd)[:, None]
    th = np.arccos(np.clip((ax * xd[:, None] + az * zd[:, None]) / (nd * r), -1.0, 1.0))
    # MSOTmodel.m:600-613
    res = min(x[1] - x[0], z[1] - z[0])
    d_step = res * (1450.0 / c)
    d_min, d_max = r.min() - d_step, r.max() + d_step
    a_step = np.arctan2(d_step, d_max) / np.pi * 180.0
    a_max = np.ceil((th.max() / np.pi * 180.0) * a_step) / a_step
    n_dist = int(np.ceil((d_max - d_min) / d_step)) + 1
    n_angle = int(np.ceil(a_max / a_step)) + 1
    H = half_window
    S0 = 2 * H + 1
    g, M = nshape_filtered(sigma, c, fs)
    src = sources(width, height, elev_radius, sx, sy)
    NS = n_dist * n_angle
    tab = np.zeros((NS, S0))
    n = np.arange(-H, H + 1)
    for c0 in range(0, NS, 512):
        cols = np.arange(c0, min(NS, c0 + 512))
        di, ai = cols // n_angle, cols % n_angle
        rr = d_min + di * d_step
        tt = ai * a_step * np.pi / 180.0
        px, pz = rr * np.sin(tt), rr * np.cos(tt)
        t = rr[:, None] / c + n[None, :] / fs  # (cols, S0)
        acc = np.zeros((cols.size, S0))
        for (sxk, syk, szk, area) in src:
            R = np.sqrt((px - sxk) ** 2 + syk ** 2 + (pz - szk) ** 2)
            a = area / (2.0 * np.pi * R)
            u = (t - (R / c)[:, None]) * FSF
            fl = np.floor(u)
            m = fl.astype(np.int64)
            ok = (m >= -M) & (m < M)
            mm = np.clip(m, -M, M - 1)
            w = u - fl
            gv = (1.0 - w) * g[mm + M] + w * g[mm + 1 + M]
            acc += np.where(ok, a[:, None] * gv, 0.0)
        tab[cols] = acc
    # calculate_polarSPMR.m:151-160, 179-183
    mx = np.abs(tab).max(axis=1, keepdims=True)
    tab[np.abs(tab) < mx * 1e-4] = 0.0
    nz_ = tab != 0
    st = nz_.argmax(axis=1) + 1
    en = S0 - nz_[:, ::-1].argmax(axis=1)
    if np.any(st == 1) or np.any(en == S0):
        raise ValueError("a column reaches the window edge; widen half_window")
    hmax = int(max((H + 1 - st).max(), (en - H - 1).max())) + 1
    h = min(hmax, H)
    shift = H - h
    sir = tab[:, shift:shift + 2 * h + 1]
    se = np.stack([st - shift, en - shift], axis=1).astype(np.int32)
    # MSOTmodel.m:472-477
    dix = _round(1 + (r - d_min) / d_step)
    aix = 1 + _round(th * 180.0 / np.pi / a_step)
    idx = ((dix - 1) * n_angle + aix).astype(np.int32)
    info = dict(d_min=d_min, d_step=d_step, a_step_deg=a_step, n_dist=n_dist, n_angle=n_angle)
    return sir, se, idx, info
