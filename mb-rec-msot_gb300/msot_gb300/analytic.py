"""The reference's analytic reconstructors on the GPU, with its MATLAB
signatures (reconstruction_backprojection/).

Layouts: sigMat [W, D, T] (== MATLAB T x D x W) as a torch CUDA tensor or
numpy array; fov given by the pixel coordinate vectors x (columns) and z
(rows) of the meshgrid (Discretization.m:28-34), or by the meshgrid matrices
themselves as the reference passes them (region.xPositionsFov /
zPositionsFov, Nz x Nx, reconstruct_dmas_cf.m:6-7); images [W, nx, nz].
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .model import _dptr, _stream_ptr


def _sig(sigMat):
    s = torch.as_tensor(sigMat)
    if not s.is_cuda:
        s = s.cuda()
    s = s.to(torch.float32)
    if s.dim() == 2:
        s = s[None]
    return s.contiguous()


def _vec(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())


def _fov_axis(v, axis: str) -> np.ndarray:
    """The coordinate vector of one fov argument: a vector as given, or from
    an Nz x Nx meshgrid matrix its first row (x: constant down each column)
    or its first column (z: constant along each row)."""
    a = np.asarray(v, dtype=np.float64)
    if a.ndim <= 1 or min(a.shape) == 1:
        return _vec(a)
    if a.ndim != 2:
        raise ValueError(f"fov_{axis} must be a vector or an Nz x Nx meshgrid matrix")
    vec = a[0, :] if axis == "x" else a[:, 0]
    grid = np.broadcast_to(vec[None, :] if axis == "x" else vec[:, None], a.shape)
    if not np.array_equal(a, grid):
        raise ValueError(f"fov_{axis} is not a meshgrid of {axis} coordinates")
    return _vec(vec)


def dmas_cf(sigMat, x, z, speed_of_sound, sampling_frequency,
            cropped_or_unrecorded_signals_at_sinogram_start, angular_coverage, detector_radius,
            stream=None):
    """dmas_cf.m:19: returns (p0_rec_dmas_cf, p0_rec_dmas, cf, p0_rec_das)."""
    s = _sig(sigMat)
    W, D, T = s.shape
    xv, zv = _fov_axis(x, "x"), _fov_axis(z, "z")
    outs = [torch.empty((W, xv.size, zv.size), device=s.device) for _ in range(4)]
    _lib.check(_lib.load().msot_dmas_cf(
        C.c_void_p(s.data_ptr()), W, D, T, _dptr(xv), xv.size, _dptr(zv), zv.size,
        float(speed_of_sound), float(sampling_frequency),
        float(cropped_or_unrecorded_signals_at_sinogram_start), float(angular_coverage),
        float(detector_radius), *[C.c_void_p(o.data_ptr()) for o in outs], _stream_ptr(stream)))
    return tuple(outs)


def reconstruct_dmas_cf(model, sinogram, stream=None):
    """reconstruct_dmas_cf.m:1-14 for a single-SoS MSOTmodel."""
    d = model.Discretization
    return dmas_cf(sinogram, d.x, d.z, model.c, model.Probe.fs,
                   model.n_crop + model.Probe.delay, model.Probe.angular_coverage,
                   model.Probe.radius, stream=stream)


def backproject_waveeq(sigMat, x, z, speed_of_sound, sampling_frequency,
                       cropped_or_unrecorded_signals_at_sinogram_start, angular_coverage,
                       detector_radius, psf, K, stream=None):
    """backproject_waveeq.m:1.  psf: MATLAB m x n array (numpy (m, n), m along
    time); K: the bp_kernel matrix of the full acquisition times (numpy (Nt, Nt)
    with K[j, k] = MATLAB K(j, k), or a CUDA tensor already in column-major
    order as returned by bp_kernel_device).  The image is the reference's,
    mirrored in x by its final fliplr (backproject_waveeq.m:49)."""
    s = _sig(sigMat)
    W, D, T = s.shape
    xv, zv = _fov_axis(x, "x"), _fov_axis(z, "z")
    psf = np.atleast_2d(np.asarray(psf, dtype=np.float64))
    psf_cm = np.ascontiguousarray(psf.T)  # column-major m x n
    if isinstance(K, torch.Tensor) and K.is_cuda:
        Kd = K.to(torch.float32).contiguous()
        Kn = int(round(Kd.numel() ** 0.5))
    else:
        Kh = np.asarray(K, dtype=np.float64)
        Kn = Kh.shape[0]
        Kd = torch.tensor(np.ascontiguousarray(Kh.T), dtype=torch.float32, device=s.device)
    out = torch.empty((W, xv.size, zv.size), device=s.device)
    _lib.check(_lib.load().msot_backproject_waveeq(
        C.c_void_p(s.data_ptr()), W, D, T, _dptr(xv), xv.size, _dptr(zv), zv.size,
        float(speed_of_sound), float(sampling_frequency),
        float(cropped_or_unrecorded_signals_at_sinogram_start), float(angular_coverage),
        float(detector_radius), _dptr(psf_cm), psf.shape[0], psf.shape[1],
        C.c_void_p(Kd.data_ptr()), Kn, C.c_void_p(out.data_ptr()), _stream_ptr(stream)))
    return out


def bp_kernel(t) -> np.ndarray:
    """bp_kernel.m:1-12: K(t, t') = -Im trapz_lambda(H0(t lambda)
    conj(H0(t' lambda)) lambda) with lambda = dl (1 .. Nt), dl = pi / (t_end -
    t_1), H0 the Hankel function of the first kind.  With H0 = J0 + i Y0 the
    imaginary part is real-valued: K = M - M^T, M = J0(t lambda) diag(w
    lambda) Y0(t' lambda)^T (w the trapezoid weights) -- two real GEMMs on
    the host in FP64."""
    from scipy import special
    t = np.asarray(t, dtype=np.float64).ravel()
    n = t.size
    dl = np.pi / (t[-1] - t[0])
    lam = dl * np.arange(1, n + 1)
    w = np.full(n, dl)
    w[0] = w[-1] = dl / 2.0
    arg = t[:, None] * lam[None, :]
    J = special.j0(arg)
    Y = special.y0(arg)
    M = (J * (w * lam)[None, :]) @ Y.T
    return M - M.T


def bp_kernel_device(t, device="cuda"):
    """bp_kernel(t) as the FP32 column-major CUDA tensor backproject_waveeq
    takes directly."""
    K = bp_kernel(t)
    return torch.tensor(np.ascontiguousarray(K.T), dtype=torch.float32, device=device)
