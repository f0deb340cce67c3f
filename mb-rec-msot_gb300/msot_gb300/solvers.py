"""Non-negative solvers with the reference's MATLAB signatures, running on
the GPU through the CUDA library.

Inputs/outputs are torch tensors (CUDA) or numpy arrays in the layouts of
model.py: data_filt [W, n_det, n_t], images [W, nx, nz].  By default the W
slices are W independent reconstructions (one reference call each); with
``coupled=True`` they are the wavelengths of ONE reference call (the
reference's lsqr/cgs then see one stacked vector).  ``x0`` is an optional
warm start (the reference's L2/TV cores always start from zero,
nnls_L2_less.m:28-29).
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np
import torch

from . import _lib
from .model import MSOTmodel, _stream_ptr


def _prep(model: MSOTmodel, data_filt, x0):
    b = torch.as_tensor(data_filt)
    if not b.is_cuda:
        b = b.cuda()
    b = b.to(torch.float32).reshape(-1, *model.sinogram_shape).contiguous()
    W = b.shape[0]
    if W > model.max_batch:
        raise ValueError(f"batch {W} > model.max_batch {model.max_batch}")
    x0p = None
    if x0 is not None:
        x0p = torch.as_tensor(x0).to(device=b.device, dtype=torch.float32)
        x0p = x0p.reshape(W, *model.image_shape).contiguous()
    rec = torch.empty((W, *model.image_shape), device=b.device, dtype=torch.float32)
    return b, W, x0p, rec


def kkt_multiplier(model: MSOTmodel, data_filt, w0, lambdaL2: float = 0.0, beta: float = 1e-3):
    """The splitting multiplier v consistent with an image w0 (nnls_L2_less's
    fixed point): v = (A'(A w0 - b) + lambdaL2 w0) / beta where w0 <= 0
    (clipped at 0), 0 elsewhere.  Costs one A and one A'."""
    b = torch.as_tensor(data_filt)
    if not b.is_cuda:
        b = b.cuda()
    b = b.to(torch.float32).reshape(-1, *model.sinogram_shape)
    w = torch.as_tensor(w0).to(device=b.device, dtype=torch.float32).clamp_min(0)
    w = w.reshape(b.shape[0], *model.image_shape).contiguous()
    g = model.transpose(model.forward(w) - b)
    if lambdaL2 and lambdaL2 > 0:
        g = g + lambdaL2 * w
    v = torch.where(w > 0, torch.zeros_like(g), (g / beta).clamp_min(0))
    return w, v.contiguous()


def rec_nn_with_L2_reg(model: MSOTmodel, data_filt, num_iter_nn_outer: int, lambdaL2: float = 0.0,
                       RegL2="identity", RegL2T="identity", lambdaL2_2=None, RegL2_2=None,
                       RegL2T_2=None, *, x0=None, v0=None, v_out=None, coupled: bool = False,
                       stream=None):
    """rec_nn_with_L2_reg.m:1.  Returns (rec_img, lCurveErrImg, lCurveErrReg,
    lCurveErrReg_2, err, t) like the reference.  x0 / v0 start the splitting
    from an image and multiplier; v_out (a CUDA tensor of the image batch's
    size) receives the final multiplier, so a solve can be continued from
    (rec_img, v_out).  RegL2 is the identity;
    RegL2_2 / RegL2T_2 (with lambdaL2_2 > 0 and lambdaL2 > 0, as the reference
    requires) is laplacian_per_wavelength.  lCurveErr* are per-instance
    numpy arrays (one value when coupled), err is empty (the reference only
    fills it when calculate_objective_per_iter is set, which it hard-codes
    to false) and t is the wall time of the solve in seconds."""
    if lambdaL2 and lambdaL2 > 0 and RegL2 not in ("identity", None):
        raise NotImplementedError("only the identity L2 regulariser is supported")
    two = bool(lambdaL2_2 and lambdaL2_2 > 0)
    if two and not (_is_laplacian(RegL2_2) and _is_laplacian(RegL2T_2 or RegL2_2)):
        raise NotImplementedError("the second L2 regulariser must be laplacian_per_wavelength")
    b, W, x0p, rec = _prep(model, data_filt, x0)
    e1 = np.zeros(W)
    e2 = np.zeros(W)
    e3 = np.zeros(W)
    t0 = time.perf_counter()
    if two:
        if v0 is not None or v_out is not None:
            raise NotImplementedError("v0 / v_out with the second regulariser")
        _lib.check(_lib.load().msot_rec_nn_with_L2_reg_2(
            model.plan, C.c_void_p(b.data_ptr()), C.c_void_p(rec.data_ptr()), W,
            int(num_iter_nn_outer), float(lambdaL2 or 0.0), float(lambdaL2_2),
            C.c_void_p(x0p.data_ptr()) if x0p is not None else None, 1 if coupled else 0,
            e1.ctypes.data_as(C.POINTER(C.c_double)), e2.ctypes.data_as(C.POINTER(C.c_double)),
            e3.ctypes.data_as(C.POINTER(C.c_double)), _stream_ptr(stream)))
    elif v_out is not None:
        if not (v_out.is_cuda and v_out.dtype == torch.float32 and v_out.is_contiguous()
                and v_out.numel() == rec.numel()):
            raise ValueError("v_out: a contiguous float32 CUDA tensor of the images' size")
        if v0 is not None and x0p is None:
            raise ValueError("v0 needs x0")
        v0p = None
        if v0 is not None:
            v0p = torch.as_tensor(v0).to(device=b.device, dtype=torch.float32)
            v0p = v0p.reshape(W, *model.image_shape).contiguous()
        _lib.check(_lib.load().msot_rec_nn_with_L2_reg_state(
            model.plan, C.c_void_p(b.data_ptr()), C.c_void_p(rec.data_ptr()),
            C.c_void_p(v_out.data_ptr()), W, int(num_iter_nn_outer), float(lambdaL2 or 0.0),
            C.c_void_p(x0p.data_ptr()) if x0p is not None else None,
            C.c_void_p(v0p.data_ptr()) if v0p is not None else None, 1 if coupled else 0,
            e1.ctypes.data_as(C.POINTER(C.c_double)), e2.ctypes.data_as(C.POINTER(C.c_double)),
            _stream_ptr(stream)))
    elif v0 is not None:
        if x0p is None:
            raise ValueError("v0 needs x0")
        v0p = torch.as_tensor(v0).to(device=b.device, dtype=torch.float32)
        v0p = v0p.reshape(W, *model.image_shape).contiguous()
        _lib.check(_lib.load().msot_rec_nn_with_L2_reg_warm(
            model.plan, C.c_void_p(b.data_ptr()), C.c_void_p(rec.data_ptr()), W,
            int(num_iter_nn_outer), float(lambdaL2 or 0.0), C.c_void_p(x0p.data_ptr()),
            C.c_void_p(v0p.data_ptr()), 1 if coupled else 0,
            e1.ctypes.data_as(C.POINTER(C.c_double)), e2.ctypes.data_as(C.POINTER(C.c_double)),
            _stream_ptr(stream)))
    else:
        _lib.check(_lib.load().msot_rec_nn_with_L2_reg(
            model.plan, C.c_void_p(b.data_ptr()), C.c_void_p(rec.data_ptr()), W,
            int(num_iter_nn_outer), float(lambdaL2 or 0.0),
            C.c_void_p(x0p.data_ptr()) if x0p is not None else None, 1 if coupled else 0,
            e1.ctypes.data_as(C.POINTER(C.c_double)), e2.ctypes.data_as(C.POINTER(C.c_double)),
            _stream_ptr(stream)))
    t = time.perf_counter() - t0
    if coupled:
        e1, e2, e3 = np.array([e1.sum()]), np.array([e2.sum()]), np.array([e3.sum()])
    return rec, e1, e2, e3, np.zeros(0), t


def laplacian_per_wavelength(x, *, stream=None):
    """laplacian_per_wavelength.m:1-9: MATLAB del2(x(:, :, wl), 1) for every
    image of a batch (W, nx, nz) on the GPU (msot_laplacian_per_wavelength)."""
    t = torch.as_tensor(x)
    if not t.is_cuda:
        t = t.cuda()
    t = t.to(torch.float32).contiguous()
    if t.dim() == 2:
        t = t.unsqueeze(0)
    out = torch.empty_like(t)
    _lib.check(_lib.load().msot_laplacian_per_wavelength(
        C.c_void_p(t.data_ptr()), C.c_void_p(out.data_ptr()), t.shape[0], t.shape[1], t.shape[2],
        _stream_ptr(stream)))
    return out


def _is_laplacian(reg) -> bool:
    return reg is laplacian_per_wavelength or reg == "laplacian"


def rec_nn_with_L1_eye_reg(model: MSOTmodel, data_filt, num_iter: int, regParam: float, *,
                           x0=None, coupled: bool = False, stream=None):
    """rec_nn_with_L1_eye_reg.m:1.  Returns (rec_img, lCurveErrImg,
    lCurveErrReg, err, t); the start value is A^T b unless x0 is given."""
    b, W, x0p, rec = _prep(model, data_filt, x0)
    e1 = np.zeros(W)
    e2 = np.zeros(W)
    t0 = time.perf_counter()
    _lib.check(_lib.load().msot_rec_nn_with_L1_eye_reg(
        model.plan, C.c_void_p(b.data_ptr()), C.c_void_p(rec.data_ptr()), W, int(num_iter),
        float(regParam), C.c_void_p(x0p.data_ptr()) if x0p is not None else None,
        1 if coupled else 0, e1.ctypes.data_as(C.POINTER(C.c_double)),
        e2.ctypes.data_as(C.POINTER(C.c_double)), _stream_ptr(stream)))
    t = time.perf_counter() - t0
    if coupled:
        e1, e2 = np.array([e1.sum()]), np.array([e2.sum()])
    return rec, e1, e2, np.zeros(0), t


def rec_nn_with_TV_reg(model: MSOTmodel, data_filt, num_iter: int, regParam: float, *,
                       sparsa_iter: int = 2, x0=None, coupled: bool = False, stream=None):
    """rec_nn_with_TV_reg.m:1 (square grids only).  Returns (rec_img,
    lCurveErrImg, lCurveErrReg, err, t); lCurveErrReg is ITV of each
    reconstruction.  sparsa_iter is SpaRSA's MaxiterA (the reference passes
    2, nnls_sparsa_based_reg_matrix_less.m:64)."""
    b, W, x0p, rec = _prep(model, data_filt, x0)
    e1 = np.zeros(W)
    e2 = np.zeros(W)
    t0 = time.perf_counter()
    _lib.check(_lib.load().msot_rec_nn_with_TV_reg(
        model.plan, C.c_void_p(b.data_ptr()), C.c_void_p(rec.data_ptr()), W, int(num_iter),
        float(regParam), int(sparsa_iter), C.c_void_p(x0p.data_ptr()) if x0p is not None else None,
        1 if coupled else 0, e1.ctypes.data_as(C.POINTER(C.c_double)),
        e2.ctypes.data_as(C.POINTER(C.c_double)), _stream_ptr(stream)))
    t = time.perf_counter() - t0
    if coupled:
        e1, e2 = np.array([e1.sum()]), np.array([e2.sum()])
    return rec, e1, e2, np.zeros(0), t


def SB_ITV2(g, mu: float, B=None, Bt=None, BtB=None, *, stream=None):
    """SB_ITV2.m:1 on a batch of square images g [W, n, n] (or one [n, n]).

    B, Bt, BtB: the reference's caller passes DiffOper(n) (PsiForTVReg.m:6,
    rec_nn_with_TV_reg.m:41); the kernel applies that operator itself, so
    they are accepted for the signature and only their shapes are checked."""
    t = torch.as_tensor(g)
    if t.dim() < 2 or t.shape[-1] != t.shape[-2]:
        raise ValueError("SB_ITV2 needs square images")
    n2 = t.shape[-1] * t.shape[-1]
    for name, op, shape in (("B", B, (2 * n2, n2)), ("Bt", Bt, (n2, 2 * n2)),
                            ("BtB", BtB, (n2, n2))):
        if op is not None and tuple(op.shape) != shape:
            raise ValueError(f"{name} must be DiffOper({t.shape[-1]}) of shape {shape}")
    if not t.is_cuda:
        t = t.cuda()
    squeeze = t.dim() == 2
    t = t.to(torch.float32).reshape(-1, t.shape[-2], t.shape[-1]).contiguous()
    u = torch.empty_like(t)
    _lib.check(_lib.load().msot_sb_itv2(C.c_void_p(t.data_ptr()), C.c_void_p(u.data_ptr()),
                                        t.shape[0], t.shape[-1], float(mu), _stream_ptr(stream)))
    return u[0] if squeeze else u


def SB_ITV(g, mu: float, *, stream=None):
    """SB_ITV.m:1: SB_ITV2 with the difference operator built inside (the
    denoising library's own entry point; its progress prints are not
    reproduced)."""
    return SB_ITV2(g, mu, stream=stream)


def ITV(x, *, stream=None):
    """ITV.m:1 for a batch of square images x [W, n, n]; returns [W] numpy."""
    t = torch.as_tensor(x)
    if not t.is_cuda:
        t = t.cuda()
    t = t.to(torch.float32).reshape(-1, t.shape[-2], t.shape[-1]).contiguous()
    out = np.zeros(t.shape[0])
    _lib.check(_lib.load().msot_itv(C.c_void_p(t.data_ptr()),
                                    out.ctypes.data_as(C.POINTER(C.c_double)), t.shape[0],
                                    t.shape[-1], _stream_ptr(stream)))
    return out
