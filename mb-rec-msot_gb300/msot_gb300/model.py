"""Host-side mirror of the reference's model classes (Probe, Discretization,
MSOTmodel) on top of the CUDA library.

The model tables are built once on the host in FP64 (geometry, IR,
prefilter) and handed to a device-resident plan; every apply runs on the GPU.
Tensor layouts (torch, CUDA, float32) are memory-identical to the MATLAB
arrays of the reference:
    image     [W, nx, nz]      == MATLAB Nz x Nx x W   (pixel p = ix*nz + iz)
    sinogram  [W, n_det, n_t]  == MATLAB T x D x W
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np
import torch
from scipy import signal as sps

from . import _lib


def _dptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("FP64 C-contiguous array required at the C ABI")
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a: np.ndarray):
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError("int32 C-contiguous array required at the C ABI")
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _stream_ptr(stream=None):
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream)


# ----------------------------------------------------------------------------
# Probe (Probe.m)
# ----------------------------------------------------------------------------
@dataclass
class Probe:
    """Arc array: elements evenly over ``angular_coverage`` degrees centred
    on the -z axis (Probe.m:112-116).  ``eir`` None -> identity EIR of
    ``eir_length`` taps (Probe.m:57-59)."""

    n_det: int = 256
    radius: float = 0.040
    angular_coverage: float = 135.0
    fs: float = 4e7
    n_samples: int = 2030
    delay: float = 0.0
    eir: np.ndarray | None = None
    eir_length: int = 257
    # dual speed of sound (Probe.membrane, Probe.coupling.speedOfSound): the
    # membrane z = sum_k membrane[k] x^k (metres; up to 8 coefficients) and the
    # speed of sound of the coupling medium between membrane and detectors
    membrane: tuple | None = None
    coupling_speed_of_sound: float | None = None

    @classmethod
    def example_system(cls, eir=None):
        """The reference's 'example_system' entry (Probe.m:101-127)."""
        return cls(n_det=256, radius=0.060, angular_coverage=145.0, fs=4e7, n_samples=2030,
                   delay=500.0, eir=eir, eir_length=201)

    def detector_positions(self):
        off = (180.0 - self.angular_coverage) / 2.0
        step = self.angular_coverage / (self.n_det - 1)
        ang = np.deg2rad(off + step * np.arange(self.n_det))
        return self.radius * np.cos(ang), -self.radius * np.sin(ang)

    def eir_taps(self) -> np.ndarray:
        if self.eir is None:
            e = np.zeros(self.eir_length)
            e[self.eir_length // 2] = 1.0
            return e
        e = np.asarray(self.eir, dtype=np.float64).ravel()
        if e.size % 2 != 1:
            raise ValueError("EIR length must be odd")
        return e

    # Read-only views under the MATLAB class's field names (Probe.m:101-127),
    # for code written against the reference's model struct.
    @property
    def detector(self):
        xd, zd = self.detector_positions()
        return SimpleNamespace(numOfTransducers=self.n_det, radius=self.radius,
                               angularCoverage=self.angular_coverage,
                               xPositionsOfTransducers=xd, zPositionsOfTransducers=zd,
                               EIR=self.eir_taps())

    @property
    def DAC(self):
        return SimpleNamespace(numRecordedSamplesPerTransducer=self.n_samples,
                               delayBeforeRecording=self.delay, frequency=self.fs)

    @property
    def coupling(self):
        return SimpleNamespace(speedOfSound=self.coupling_speed_of_sound)

    @property
    def eirLength(self) -> int:
        return int(self.eir_taps().size)


# ----------------------------------------------------------------------------
# Discretization (Discretization.m)
# ----------------------------------------------------------------------------
class Discretization:
    """Pixel grid (Discretization.m:19-35) and the Gaussian pixel model's
    shift-invariant prefilter (Discretization.m:41-51) as separable circular
    taps."""

    def __init__(self, field_of_view, size_of_pixel_grid):
        fov = list(field_of_view)
        if len(fov) <= 2:
            fov = [fov[0], fov[1], fov[0], fov[1]]
        if np.isscalar(size_of_pixel_grid):
            size_of_pixel_grid = (size_of_pixel_grid, size_of_pixel_grid)
        self.nx, self.nz = int(size_of_pixel_grid[0]), int(size_of_pixel_grid[1])
        self.fov = tuple(float(v) for v in fov)
        self.x = np.linspace(fov[0], fov[1], self.nx)
        self.z = np.linspace(fov[2], fov[3], self.nz)
        self.dx = self.x[1] - self.x[0]
        self.dz = self.z[1] - self.z[0]
        self.sigma = round(min(self.dx, self.dz) / 2 * 1e6) / 1e6
        # region.xPositionsFov / zPositionsFov: the Nz x Nx meshgrid matrices
        # of Discretization.m:34, for code written against the MATLAB class
        X, Z = np.meshgrid(self.x, self.z)
        self.region = SimpleNamespace(xPositionsFov=X, zPositionsFov=Z)
        self.sizeOfPixelGrid = (self.nx, self.nz)

    @property
    def numberOfPixels(self) -> int:
        return self.nx * self.nz

    @property
    def number_of_pixels(self) -> int:
        return self.nx * self.nz

    def pixel_model(self, r):
        return np.exp(-np.asarray(r) ** 2 / (2 * self.sigma ** 2))

    def pixel_coordinates(self):
        """(x, z) of pixel p = ix*nz + iz."""
        return np.repeat(self.x, self.nz), np.tile(self.z, self.nx)

    def _axis_taps(self, n, h, tol=1e-13, kmax=64):
        # 1-D factor of conj(phi_hat / F{autocorr}) with lattice [1 1]
        lin = h * np.arange(np.floor(-n / 2), np.floor(n / 2 - 1) + 1)
        g = np.fft.fftshift(self.pixel_model(lin))
        gh = np.fft.fft(g)
        pre = np.conj(gh / np.fft.fft(np.real(np.fft.ifft(np.abs(gh) ** 2))))
        kern = np.real(np.fft.ifft(pre))
        big = np.abs(kern) > tol * abs(kern[0])
        K = 0
        for k in range(1, (n - 1) // 2 + 1):
            if big[k] or big[-k]:
                K = k
        K = min(K, kmax)
        return kern[np.arange(-K, K + 1) % n].copy()

    def prefilter_taps(self):
        """(taps_x, taps_z): centred circular kernels along x and z."""
        return self._axis_taps(self.nx, self.dx), self._axis_taps(self.nz, self.dz)


# ----------------------------------------------------------------------------
# Impulse response (MSOTmodel.m:320-348, filter_butter_zero_phase.m)
# ----------------------------------------------------------------------------
def butter_zero_phase(sig: np.ndarray, fs: float, fmin: float, fmax: float) -> np.ndarray:
    """Zero-phase Butterworth filtering in the FFT domain along axis 0
    (filter_butter_zero_phase.m:16-48): demean when fmin > 0, |H|^2 of an
    order-8 low-pass (fmax) and order-2 high-pass (fmin) on the whole circle."""
    x = np.asarray(sig, dtype=np.float64)
    if fmin > 0:
        x = x - x.mean(axis=0, keepdims=True)
    zs, ps, k = [], [], 1.0
    if fmax > 0:
        z, p, g = sps.butter(8, 2 * fmax / fs, "low", output="zpk")
        zs.append(z); ps.append(p); k *= g
    if fmin > 0:
        z, p, g = sps.butter(2, 2 * fmin / fs, "high", output="zpk")
        zs.append(z); ps.append(p); k *= g
    if not zs:
        return x
    sos = sps.zpk2sos(np.concatenate(zs), np.concatenate(ps), k)
    _, h = sps.sosfreqz(sos, worN=x.shape[0], whole=True)
    H2 = (np.abs(h) ** 2).reshape((-1,) + (1,) * (x.ndim - 1))
    return np.real(np.fft.ifft(H2 * np.fft.fft(x, axis=0), axis=0))


def model_impulse_response(probe: Probe, disc: Discretization, c: float, fmin: float,
                           fmax: float, include_sir: bool) -> np.ndarray:
    eir = probe.eir_taps()
    if include_sir:
        return butter_zero_phase(eir, probe.fs, fmin, fmax)
    L = eir.size
    h = (L - 1) // 2
    t = np.arange(-h, h + 1) / probe.fs
    pixel_response = disc.pixel_model(t * c) * (-t)  # time derivative of the pixel
    ir = np.convolve(eir, pixel_response)[h:h + L]
    return butter_zero_phase(ir, probe.fs, fmin, fmax)


# ----------------------------------------------------------------------------
# MSOTmodel
# ----------------------------------------------------------------------------
class _Funcs:
    def __init__(self, model):
        self.applyForward = model.forward
        self.applyTranspose = model.transpose


def travel_times(probe: Probe, disc: Discretization, c: float, n_crop: int = 0) -> np.ndarray:
    """[n_det][nx*nz] FP64 fractional sample indices |x_p - x_d| / c * fs -
    delay - n_crop (MSOTmodel.m:350-382, single speed of sound), computed by
    msot_travel_times on the GPU."""
    out = np.empty((probe.n_det, disc.nx * disc.nz), dtype=np.float64)
    x = np.ascontiguousarray(disc.x, dtype=np.float64)
    z = np.ascontiguousarray(disc.z, dtype=np.float64)
    P = C.POINTER(C.c_double)
    _lib.check(_lib.load().msot_travel_times(
        int(probe.n_det), float(probe.radius), float(probe.angular_coverage),
        x.ctypes.data_as(P), x.size, z.ctypes.data_as(P), z.size, float(c), float(probe.fs),
        float(probe.delay), float(n_crop), out.ctypes.data_as(P)))
    return out


def travel_times_dual(probe: Probe, disc: Discretization, c_below: float, c_above: float,
                      membrane, n_crop: int = 0, virtual: bool = False):
    """([n_det][nx*nz] fractional sample indices, membrane intersections x_m)
    for two speeds of sound split by the membrane (refraction.m:8-24,
    fermat_principle.m:17-24; MSOTmodel.m:380-381), computed by
    msot_travel_times_dual on the GPU (FP64 Fermat minimisation); with
    ``virtual`` also the virtual sources (virt_x, virt_z) of
    MSOTmodel.m:585-594."""
    P = disc.nx * disc.nz
    out = np.empty((probe.n_det, P), dtype=np.float64)
    xm = np.empty((probe.n_det, P), dtype=np.float64)
    vx = np.empty((probe.n_det, P), dtype=np.float64) if virtual else None
    vz = np.empty((probe.n_det, P), dtype=np.float64) if virtual else None
    x = np.ascontiguousarray(disc.x, dtype=np.float64)
    z = np.ascontiguousarray(disc.z, dtype=np.float64)
    a = np.ascontiguousarray(np.atleast_1d(membrane), dtype=np.float64)
    D = C.POINTER(C.c_double)
    _lib.check(_lib.load().msot_travel_times_dual(
        int(probe.n_det), float(probe.radius), float(probe.angular_coverage),
        x.ctypes.data_as(D), x.size, z.ctypes.data_as(D), z.size, float(c_below),
        float(c_above), a.ctypes.data_as(D), a.size, float(probe.fs), float(probe.delay),
        float(n_crop), out.ctypes.data_as(D), xm.ctypes.data_as(D),
        vx.ctypes.data_as(D) if virtual else None, vz.ctypes.data_as(D) if virtual else None))
    return (out, xm, vx, vz) if virtual else (out, xm)


class MSOTmodel:
    """MSOTmodel(probe, discretization, speed_of_sound, include_sir,
    use_single_speed_of_sound, num_cropped_samples_at_sinogram_start,
    filt_cutoff_min, filt_cutoff_max, model_normalization_factor)
    (MSOTmodel.m:18); dual speed of sound (use_single_speed_of_sound False)
    takes the membrane and coupling speed from the probe.  cache_dir keeps
    the travel-time tables on disk (msot_gb300.cache).  SIR tables, when
    include_sir, are given as ``sir_tables=(SPMR [NS, S], start_end [NS, 2]
    1-based, SPMRIndices [n_det, P] 1-based)``.  ``max_batch`` sizes the
    plan's scratch for batched applies and solves."""

    def __init__(self, probe: Probe, discretization: Discretization, speed_of_sound: float,
                 include_sir: bool = False, use_single_speed_of_sound: bool = True,
                 num_cropped_samples_at_sinogram_start: int = 0, filt_cutoff_min: float = 1e5,
                 filt_cutoff_max: float = 12e6, model_normalization_factor: float | None = None,
                 sir_tables=None, max_batch: int = 1, norm_iterations: int = 100,
                 cache_dir: str | None = None):
        self.use_single_speed_of_sound = bool(use_single_speed_of_sound)
        if not self.use_single_speed_of_sound:
            if probe.membrane is None or probe.coupling_speed_of_sound is None:
                raise ValueError("dual speed of sound needs probe.membrane and "
                                 "probe.coupling_speed_of_sound")
        self.Probe = probe
        self.Discretization = discretization
        self.c = float(speed_of_sound)
        self.include_sir = bool(include_sir)
        self.n_crop = int(num_cropped_samples_at_sinogram_start)
        self.fmin, self.fmax = float(filt_cutoff_min), float(filt_cutoff_max)
        self.n_t = int(probe.n_samples - self.n_crop)
        self.max_batch = int(max_batch)
        disc = discretization
        # travel-time indices (MSOTmodel.m:380-381; straight rays, refraction.m:20-24,
        # or refracted at the membrane), computed on the GPU in FP64
        if self.use_single_speed_of_sound:
            compute = lambda: (travel_times(probe, disc, self.c, self.n_crop), None)
            c_ir = self.c
        else:
            compute = lambda: travel_times_dual(probe, disc, self.c, probe.coupling_speed_of_sound,
                                                probe.membrane, self.n_crop)
            c_ir = float(probe.coupling_speed_of_sound)  # MSOTmodel.m:331-335
        if cache_dir:
            # acoustic_file_<hash> of MSOTmodel.m:350-379
            from . import cache
            self.travel, self.x_membrane_intersections = cache.acoustic_tables(
                cache_dir, probe, disc, self.c, self.n_crop, self.use_single_speed_of_sound,
                compute)
        else:
            self.travel, self.x_membrane_intersections = compute()
        # interpolation radius (MSOTmodel.m:36-38)
        self.radius = float(disc.dz / (self.c / probe.fs))
        self.ir = np.ascontiguousarray(
            model_impulse_response(probe, disc, c_ir, self.fmin, self.fmax, self.include_sir),
            dtype=np.float64)
        self.pre_x, self.pre_z = (np.ascontiguousarray(t, dtype=np.float64)
                                  for t in disc.prefilter_taps())
        self.sir_tables = None
        if self.include_sir:
            if sir_tables is None:
                raise ValueError("include_sir needs sir_tables (SPMR, start/end, indices)")
            sir, se, idx = sir_tables
            self.sir_tables = (np.ascontiguousarray(sir, dtype=np.float64),
                               np.ascontiguousarray(se, dtype=np.int32),
                               np.ascontiguousarray(idx, dtype=np.int32))
        self._plan = None
        self.norm = 1.0
        self._make_plan(1.0)
        if model_normalization_factor is None:
            self.norm = self.estimate_sigma_max(norm_iterations)
        else:
            self.norm = float(model_normalization_factor)
        self._make_plan(self.norm)
        self.Funcs = _Funcs(self)

    # --- plan -------------------------------------------------------------------
    def _make_plan(self, norm: float):
        L = _lib.load()
        if self._plan:
            L.msot_plan_destroy(self._plan)
            self._plan = None
        d = _lib.PlanDesc()
        disc = self.Discretization
        d.nx, d.nz = disc.nx, disc.nz
        d.n_det, d.n_t = self.Probe.n_det, self.n_t
        d.radius = self.radius
        self._keep = [self.travel, self.ir, self.pre_x, self.pre_z]
        d.travel = _dptr(self.travel)
        d.ir_len = self.ir.size
        d.ir = _dptr(self.ir)
        d.pre_len_x, d.pre_len_z = self.pre_x.size, self.pre_z.size
        d.pre_x, d.pre_z = _dptr(self.pre_x), _dptr(self.pre_z)
        d.norm = norm
        if self.sir_tables is not None:
            sir, se, idx = self.sir_tables
            self._keep += [sir, se, idx]
            d.sir_len, d.n_sir = sir.shape[1], sir.shape[0]
            d.sir, d.sir_start_end, d.sir_idx = _dptr(sir), _iptr(se), _iptr(idx)
        d.max_batch = self.max_batch
        h = C.c_void_p()
        _lib.check(L.msot_plan_create(C.byref(d), C.byref(h)))
        self._plan = h

    def __del__(self):
        try:
            if self._plan:
                _lib.load().msot_plan_destroy(self._plan)
        except Exception:
            pass

    @property
    def plan(self):
        return self._plan

    def autotune(self, batch: int | None = None, stream=None) -> dict:
        """msot_autotune: time the kernel variants on this model's geometry at
        ``batch`` instances (default max_batch) and keep the fastest."""
        t = _lib.Tuning()
        _lib.check(_lib.load().msot_autotune(self.plan, int(batch or self.max_batch),
                                             _stream_ptr(stream), C.byref(t)))
        return {f: getattr(t, f) for f, _ in t._fields_}

    def set_storage(self, image_format=False, refine_every: int = 0) -> None:
        """msot_plan_set_storage: 16-bit storage of the DAS forward's
        interpolation input (FP32 accumulation) -- image_format "bf16" (or
        True), "fp16" (scaled per instance), or "fp32" (or False) -- and in
        the L1 solver every ``refine_every``-th outer iteration with the FP32
        input."""
        fmts = {False: 0, "fp32": 0, True: 1, "bf16": 1, "fp16": 2}
        if image_format not in fmts:
            raise ValueError("image_format: 'fp32', 'bf16' or 'fp16'")
        _lib.check(_lib.load().msot_plan_set_storage(self.plan, fmts[image_format],
                                                     int(refine_every)))

    def estimate_sigma_max(self, iters: int = 100, seed: int = 0) -> float:
        out = C.c_double()
        _lib.check(_lib.load().msot_estimate_norm(self._plan, int(iters), int(seed),
                                                  C.byref(out), _stream_ptr()))
        return float(out.value)

    # --- the reference's model struct fields (MSOTmodel.m:18-48), read-only -------
    @property
    def Medium(self):
        return SimpleNamespace(speedOfSound=self.c)

    @property
    def DataPreprocessing(self):
        return SimpleNamespace(numCroppedSamplesAtSinogramStart=self.n_crop,
                               filtCutoffMin=self.fmin, filtCutoffMax=self.fmax)

    @property
    def Data(self):
        """numTimeSamplesPerTransducer, absoluteTravelTimeIndices ([n_det][P],
        memory-identical to MATLAB's P x D) and
        circularInterpolationRadiusInSamples."""
        return SimpleNamespace(numTimeSamplesPerTransducer=self.n_t,
                               absoluteTravelTimeIndices=self.travel,
                               circularInterpolationRadiusInSamples=self.radius)

    @property
    def useSingleSpeedOfSound(self) -> bool:
        return self.use_single_speed_of_sound

    @property
    def includeSir(self) -> bool:
        return self.include_sir

    # --- operators ----------------------------------------------------------------
    @property
    def image_shape(self):
        return (self.Discretization.nx, self.Discretization.nz)

    @property
    def sinogram_shape(self):
        return (self.Probe.n_det, self.n_t)

    def _as_batch(self, x, inner):
        t = torch.as_tensor(x)
        if not t.is_cuda:
            t = t.cuda()
        t = t.to(torch.float32).reshape(-1, *inner).contiguous()
        if t.shape[0] > self.max_batch:
            raise ValueError(f"batch {t.shape[0]} > max_batch {self.max_batch}")
        return t

    def forward(self, p0, out=None, stream=None):
        """Funcs.applyForward: [W, nx, nz] -> [W, n_det, n_t] (MSOTmodel.m:285)."""
        x = self._as_batch(p0, self.image_shape)
        W = x.shape[0]
        if out is None:
            out = torch.empty((W, *self.sinogram_shape), device=x.device, dtype=torch.float32)
        _lib.check(_lib.load().msot_forward(self._plan, C.c_void_p(x.data_ptr()),
                                            C.c_void_p(out.data_ptr()), W, _stream_ptr(stream)))
        return out

    def transpose(self, sig, out=None, stream=None):
        """Funcs.applyTranspose: [W, n_det, n_t] -> [W, nx, nz] (MSOTmodel.m:286)."""
        y = self._as_batch(sig, self.sinogram_shape)
        W = y.shape[0]
        if out is None:
            out = torch.empty((W, *self.image_shape), device=y.device, dtype=torch.float32)
        _lib.check(_lib.load().msot_transpose(self._plan, C.c_void_p(y.data_ptr()),
                                              C.c_void_p(out.data_ptr()), W,
                                              _stream_ptr(stream)))
        return out

    def interp_forward(self, coeffs, stream=None):
        """The bare MEX operator (forwardDelayAndSumMex / forwardMex) on device."""
        x = self._as_batch(coeffs, (self.Discretization.number_of_pixels,))
        out = torch.empty((x.shape[0], *self.sinogram_shape), device=x.device)
        _lib.check(_lib.load().msot_interp_forward(self._plan, C.c_void_p(x.data_ptr()),
                                                   C.c_void_p(out.data_ptr()), x.shape[0],
                                                   _stream_ptr(stream)))
        return out

    def interp_transpose(self, sig, stream=None):
        y = self._as_batch(sig, self.sinogram_shape)
        out = torch.empty((y.shape[0], self.Discretization.number_of_pixels), device=y.device)
        _lib.check(_lib.load().msot_interp_transpose(self._plan, C.c_void_p(y.data_ptr()),
                                                     C.c_void_p(out.data_ptr()), y.shape[0],
                                                     _stream_ptr(stream)))
        return out
