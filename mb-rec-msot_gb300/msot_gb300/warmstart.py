"""Learned warm start for the L2-NNLS solve (no counterpart in the
reference): a U-Net on the project's CUDA kernels (msot_unet_*), trained on
pairs the plain GPU solver generates, whose prediction seeds both splitting
variables of rec_nn_with_L2_reg (image w and multiplier v, kkt_multiplier).

The network input f is a backprojection of the sinogram b (input_iters =
0): A'b, or the backproject_waveeq image (backprojection = "waveeq", with
the bp_kernel of the acquisition times and its x mirror undone) -- or the
plain solver's iterate after input_iters iterations.  Input f / s, output
x / (kappa s), with s = rms(f) per instance and kappa = median rms(x) /
rms(f) over the training pairs, so one network serves any data scale; with
``residual`` (an iterate as input, kappa = 1) the network predicts the
correction x / s - f / s.  The plain solver stays
the fallback, twice: an instance whose prediction has a larger objective
|A x0 - b|^2 + lambda |x0|^2 than the zero start (|b|^2) is started from
zero, and (solve) an instance whose data residual |A x - b|^2 rose during the
warm iterations above that of its start is solved again from zero.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .model import _stream_ptr
from .solvers import rec_nn_with_L2_reg


class UNet:
    """msot_unet_create_ch(levels, base_channels, in_channels, side, max_batch,
    seed): input (n, in_channels, side, side), output (n, 1, side, side)."""

    def __init__(self, levels=4, base_channels=32, side=128, max_batch=16, seed=0,
                 in_channels=1):
        self.levels, self.base, self.side, self.max_batch = levels, base_channels, side, max_batch
        self.in_channels = int(in_channels)
        h = C.c_void_p()
        _lib.check(_lib.load().msot_unet_create_ch(levels, base_channels, self.in_channels, side,
                                                   max_batch, seed, C.byref(h)))
        self._h = h
        n = C.c_size_t()
        _lib.check(_lib.load().msot_unet_param_count(h, C.byref(n)))
        self.n_params = n.value
        self.step_count = 0

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.load().msot_unet_destroy(self._h)
            self._h = None

    def check(self):
        """Synchronise and raise if a tensor-core convolution timed out."""
        _lib.check(_lib.load().msot_unet_check(self._h))

    def get_params(self) -> np.ndarray:
        p = np.empty(self.n_params, dtype=np.float32)
        _lib.check(_lib.load().msot_unet_get_params(self._h, p.ctypes.data_as(
            C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        _lib.check(_lib.load().msot_unet_set_params(self._h, p.ctypes.data_as(
            C.POINTER(C.c_float))))

    def _dev(self, x, channels=None):
        t = torch.as_tensor(x)
        if not t.is_cuda:
            t = t.cuda()
        c = self.in_channels if channels is None else channels
        return t.to(torch.float32).reshape(-1, c, self.side, self.side).contiguous()

    def forward(self, x, stream=None):
        x = self._dev(x)
        out = torch.empty((x.shape[0], 1, self.side, self.side), device=x.device,
                          dtype=torch.float32)
        for c0 in range(0, x.shape[0], self.max_batch):
            xs = x[c0:c0 + self.max_batch]
            _lib.check(_lib.load().msot_unet_forward(self._h, C.c_void_p(xs.data_ptr()),
                                                     C.c_void_p(out[c0:].data_ptr()),
                                                     xs.shape[0], _stream_ptr(stream)))
        return out

    def gradients(self, x, target, stream=None):
        x, t = self._dev(x), self._dev(target, 1)
        loss = C.c_double()
        g = np.empty(self.n_params, dtype=np.float32)
        _lib.check(_lib.load().msot_unet_gradients(self._h, C.c_void_p(x.data_ptr()),
                                                   C.c_void_p(t.data_ptr()), x.shape[0],
                                                   C.byref(loss),
                                                   g.ctypes.data_as(C.POINTER(C.c_float)),
                                                   _stream_ptr(stream)))
        return loss.value, g

    def train_step(self, x, target, lr=1e-3, stream=None):
        x, t = self._dev(x), self._dev(target, 1)
        loss = C.c_double()
        _lib.check(_lib.load().msot_unet_gradients(self._h, C.c_void_p(x.data_ptr()),
                                                   C.c_void_p(t.data_ptr()), x.shape[0],
                                                   C.byref(loss), None, _stream_ptr(stream)))
        self.step_count += 1
        _lib.check(_lib.load().msot_unet_adam_step(self._h, float(lr), self.step_count,
                                                   _stream_ptr(stream)))
        return loss.value


class LearnedWarmStart:
    """Warm start of rec_nn_with_L2_reg(model, b, iters, lambdaL2) from a
    U-Net prediction (see the module docstring)."""

    def __init__(self, model, lambdaL2: float = 0.0, net: UNet | None = None, levels=4,
                 base_channels=32, max_batch=16, seed=0, beta=1e-3, input_iters=0,
                 residual=None, backprojection: str = "transpose", trajectory: int = 0):
        nx, nz = model.image_shape
        if nx != nz:
            raise ValueError("the warm-start network needs a square grid")
        self.model, self.lam, self.beta = model, float(lambdaL2 or 0.0), beta
        self.trajectory = int(trajectory)
        if self.trajectory and not 0 < self.trajectory < int(input_iters):
            raise ValueError("the trajectory input needs 0 < trajectory < input_iters")
        self.net = net or UNet(levels, base_channels, nx, max_batch, seed,
                               in_channels=2 if self.trajectory else 1)
        self.input_iters = int(input_iters)
        self.residual = bool(self.input_iters > 0 if residual is None else residual)
        if self.residual and self.input_iters <= 0:
            raise ValueError("the residual form needs an iterate as input (input_iters > 0)")
        self.kappa = 1.0 if self.residual else None
        if backprojection not in ("transpose", "waveeq"):
            raise ValueError("backprojection: 'transpose' or 'waveeq'")
        self.backprojection = backprojection
        self._K = None

    def _chunks(self, W):
        m = self.model.max_batch
        return [(i, min(W, i + m)) for i in range(0, W, m)]

    def _sino(self, b):
        b = torch.as_tensor(b)
        if not b.is_cuda:
            b = b.cuda()
        return b.to(torch.float32).reshape(-1, *self.model.sinogram_shape).contiguous()

    def features(self, b):
        """(f / s as (W, 1, n, n), s (W,)); f = the plain iterate, A'b or the
        backproject_waveeq image (see the module docstring).  With
        ``trajectory`` = m a second channel holds (x_k - x_{k-m}) / s, the last
        m steps of the plain iteration (k = input_iters; the solve runs k - m
        iterations, keeps its multiplier, and continues for m: k in all)."""
        b = self._sino(b)
        d = None
        if self.input_iters > 0 and self.trajectory:
            fs, ds = [], []
            for i, j in self._chunks(b.shape[0]):
                v = torch.empty((j - i, *self.model.image_shape), device=b.device,
                                dtype=torch.float32)
                wa = rec_nn_with_L2_reg(self.model, b[i:j], self.input_iters - self.trajectory,
                                        self.lam, v_out=v)[0]
                wk = rec_nn_with_L2_reg(self.model, b[i:j], self.trajectory, self.lam, x0=wa,
                                        v0=v.clone(), v_out=v)[0]
                fs.append(wk)
                ds.append(wk - wa)
            f, d = torch.cat(fs), torch.cat(ds)
        elif self.input_iters > 0:
            f = torch.cat([rec_nn_with_L2_reg(self.model, b[i:j], self.input_iters, self.lam)[0]
                           for i, j in self._chunks(b.shape[0])])
        elif self.backprojection == "waveeq":
            f = self._waveeq(b)
        else:
            f = torch.cat([self.model.transpose(b[i:j]) for i, j in self._chunks(b.shape[0])])
        s = f.flatten(1).pow(2).mean(1).sqrt().clamp_min(1e-30)
        feat = (f / s.view(-1, 1, 1)).unsqueeze(1)
        if d is not None:
            feat = torch.cat([feat, (d / s.view(-1, 1, 1)).unsqueeze(1)], dim=1)
        return feat.contiguous(), s

    def _waveeq(self, b):
        """backproject_waveeq of b on the model's grid and probe (psf = 1),
        with the x mirror of backproject_waveeq.m:49 undone so that the image
        lines up with the model's pixels."""
        from .analytic import backproject_waveeq, bp_kernel_device
        m, d, p = self.model, self.model.Discretization, self.model.Probe
        crop = m.n_crop + p.delay
        if self._K is None:
            nt = m.n_t + int(round(crop))
            self._K = bp_kernel_device(np.arange(1, nt + 1) / p.fs)
        out = backproject_waveeq(b, d.x, d.z, m.c, p.fs, crop, p.angular_coverage, p.radius,
                                 np.array([[1.0]]), self._K)
        return out.flip(1).contiguous()

    def make_pairs(self, images, iters=200, noise=0.01, seed=0):
        """Training pairs from phantoms (W, nx, nz): sinograms A x + noise
        (``noise`` x rms of A x, Gaussian), the plain solver's ``iters``
        iteration reconstruction as the target.  Returns (inputs, targets,
        sinograms); sets kappa on the first call."""
        images = torch.as_tensor(images).cuda().to(torch.float32)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(int(seed))
        bs, recs = [], []
        for i, j in self._chunks(images.shape[0]):
            y = self.model.forward(images[i:j].contiguous())
            r = y.flatten(1).pow(2).mean(1).sqrt().view(-1, 1, 1)
            y = y + noise * r * torch.randn(y.shape, generator=gen, device="cuda")
            bs.append(y)
            recs.append(rec_nn_with_L2_reg(self.model, y, iters, self.lam)[0])
        b, rec = torch.cat(bs), torch.cat(recs)
        f, s = self.features(b)
        if self.kappa is None:
            ratio = rec.flatten(1).pow(2).mean(1).sqrt() / s
            self.kappa = float(ratio.median())
        t = (rec / (self.kappa * s.view(-1, 1, 1))).unsqueeze(1)
        if self.residual:
            t = t - f[:, :1]
        return f, t.contiguous(), b

    def fit(self, inputs, targets, steps, batch=16, lr=1e-3, lr_final=1e-5, seed=0):
        """Adam on random minibatches with a cosine learning-rate decay;
        returns the per-step losses."""
        batch = min(batch, self.net.max_batch)
        g = torch.Generator(device="cuda")
        g.manual_seed(int(seed))
        W = inputs.shape[0]
        losses = []
        for k in range(steps):
            idx = torch.randint(0, W, (batch,), generator=g, device="cuda")
            a = lr_final + 0.5 * (lr - lr_final) * (1 + np.cos(np.pi * k / max(1, steps)))
            losses.append(self.net.train_step(inputs[idx], targets[idx], lr=a))
        return losses

    def predict(self, b):
        """x0 = kappa s relu(net(A'b / s)), (W, nx, nz)."""
        if self.kappa is None:
            raise RuntimeError("kappa unset: make_pairs (or set kappa) before predicting")
        f, s = self.features(b)
        out = self.net.forward(f)
        if self.residual:
            out = out + f[:, :1]
        return (out.squeeze(1).clamp_min(0) * (self.kappa * s.view(-1, 1, 1))).contiguous()

    def start(self, b, x0=None):
        """(w0, v0, fallback mask): the prediction, its consistent multiplier
        and which instances were put back to the zero start."""
        b = self._sino(b)
        w = self.predict(b) if x0 is None else torch.as_tensor(x0).cuda().to(torch.float32)
        v = torch.empty_like(w)
        fell = torch.zeros(b.shape[0], dtype=torch.bool, device="cuda")
        res0 = torch.empty(b.shape[0], dtype=torch.float64, device="cuda")
        for i, j in self._chunks(b.shape[0]):
            r = self.model.forward(w[i:j].contiguous()) - b[i:j]
            res0[i:j] = r.flatten(1).double().pow(2).sum(1)
            obj = r.flatten(1).pow(2).sum(1) + self.lam * w[i:j].flatten(1).pow(2).sum(1)
            fell[i:j] = obj >= b[i:j].flatten(1).pow(2).sum(1)
            g = self.model.transpose(r.contiguous())
            if self.lam > 0:
                g = g + self.lam * w[i:j]
            v[i:j] = torch.where(w[i:j] > 0, torch.zeros_like(g), (g / self.beta).clamp_min(0))
        keep = (~fell).view(-1, 1, 1).to(torch.float32)
        # data residual of each start (|b|^2 for a zero start), for solve()
        self.start_residual = torch.where(fell, b.flatten(1).double().pow(2).sum(1), res0)
        return (w * keep).contiguous(), (v * keep).contiguous(), fell

    def solve(self, b, iters, x0=None, restart_iters=None):
        """rec_nn_with_L2_reg from the learned start; an instance whose data
        residual rose above its start's is solved again from zero with
        ``restart_iters`` (default ``iters``) plain iterations.  Returns (rec,
        fallback mask: objective test at the start or residual rise)."""
        b = self._sino(b)
        w, v, fell = self.start(b, x0)
        recs, res = [], []
        for i, j in self._chunks(b.shape[0]):
            out = rec_nn_with_L2_reg(self.model, b[i:j], iters, self.lam, x0=w[i:j], v0=v[i:j])
            recs.append(out[0])
            res.append(torch.as_tensor(out[1], dtype=torch.float64, device="cuda"))
        rec = torch.cat(recs)
        rose = torch.cat(res) > self.start_residual
        if bool(rose.any()):
            idx = torch.nonzero(rose).flatten()
            again = torch.cat([rec_nn_with_L2_reg(self.model, b[idx[i:j]].contiguous(),
                                                  restart_iters or iters, self.lam)[0]
                               for i, j in self._chunks(idx.numel())])
            rec[idx] = again
        return rec, fell | rose
