"""FP64 numpy restatement of the reference's operator wrapper (MSOTmodel).

TEST INFRASTRUCTURE ONLY ("the oracle"): imported by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
product.  It restates, in FP64:

  * the arc probe geometry            Probe.m:110-116
  * the pixel grid                    Discretization.m:19-35
  * the Gaussian pixel model          Discretization.m:41-44, :112-118
  * the shift-invariant prefilter     Discretization.m:46-51, :74-86,
                                      shift_inv_proj.m:66-71
  * project / transpose-project       Discretization.m:54-72
  * single-SoS travel-time indices    MSOTmodel.m:350-382, refraction.m:20-24
  * dual-SoS (Fermat) travel times    refraction.m:8-24, fermat_principle.m:17-24
  * interpolation radius              MSOTmodel.m:35-38
  * the impulse response (no SIR)     MSOTmodel.m:329-348
  * the impulse response (with SIR)   MSOTmodel.m:320-327
  * zero-phase Butterworth filter     load_and_preprocess/filter_butter_zero_phase.m:16-48
  * IR convolution and its transpose  MSOTmodel.m:259-269
  * forward / transpose               MSOTmodel.m:189-257
  * normalisation by sigma_max        MSOTmodel.m:271-287

Layout: sinograms are numpy (W, D, T) C-order (== MATLAB T x D x W) and
images (W, Nx, Nz) C-order (== MATLAB Nz x Nx x W); pixel p = ix*Nz + iz.

Pins: the interpolation inside forward / transpose runs through the C
restatement of the MEX loops (msot_oracle.c), bit-identical to the
reference's compiled MEX code.  The MATLAB wrapper steps around it have no
MATLAB run to compare with (parity unpinned against MATLAB itself); they are
checked against independent computations in tests/test_oracle.py instead.
Those checks are: the separable prefilter against the 2-D FFT prefilter, the
FFT zero-phase filter against forward-backward IIR filtering, the adjoint
test, the power-iteration norm against an SVD, and one pixel's sinogram
located by both this model's transpose and the analytic reconstructors.

Deviations recorded for the synthetic probe used by this project: the EIR
length is a probe property (odd, e.g. 257) instead of the reference's fixed
201 (Probe.m:13); the crop uses floor(L/2) of that length, so the output keeps
T samples.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
from scipy import signal as sps

from . import native


# ----------------------------------------------------------------------------
# Probe and grid
# ----------------------------------------------------------------------------
@dataclass
class ArcProbe:
    """Arc detector array (Probe.m:110-127 with configurable values)."""

    n_det: int = 256
    radius: float = 0.040
    coverage_deg: float = 135.0
    fs: float = 4e7
    n_samples: int = 2030
    delay: float = 0.0
    eir: np.ndarray | None = None  # odd length; None -> identity (Probe.m:57-59)
    eir_length: int = 257
    # SIR element geometry (used by sir.py): in-plane width, elevation height
    element_width: float = 0.25e-3
    element_height: float = 10e-3

    def angles(self) -> np.ndarray:
        off = (180.0 - self.coverage_deg) / 2.0
        step = self.coverage_deg / (self.n_det - 1)
        return (off + step * np.arange(self.n_det)) * np.pi / 180.0

    def positions(self):
        a = self.angles()
        return self.radius * np.cos(a), -self.radius * np.sin(a)

    def eir_taps(self) -> np.ndarray:
        if self.eir is None:
            e = np.zeros(self.eir_length)
            e[self.eir_length // 2] = 1.0
            return e
        e = np.asarray(self.eir, dtype=np.float64)
        assert e.ndim == 1 and e.size % 2 == 1, "EIR length must be odd"
        return e


@dataclass
class Grid:
    """Pixel grid (Discretization.m:19-35); fov = [xmin, xmax, zmin, zmax]."""

    nx: int
    nz: int
    fov: tuple = (-0.0127, 0.0127, -0.0127, 0.0127)

    @property
    def n_pix(self) -> int:
        return self.nx * self.nz

    def vectors(self):
        x = np.linspace(self.fov[0], self.fov[1], self.nx)
        z = np.linspace(self.fov[2], self.fov[3], self.nz)
        return x, z

    def pixel_xz(self):
        """Flattened column-major pixel coordinates, p = ix*nz + iz."""
        x, z = self.vectors()
        X = np.repeat(x, self.nz)
        Z = np.tile(z, self.nx)
        return X, Z

    def spacing(self):
        x, z = self.vectors()
        return x[1] - x[0], z[1] - z[0]

    def sigma(self) -> float:
        """Gaussian pixel width, Discretization.m:42-43 (rounded to 1 um)."""
        dx, dz = self.spacing()
        return round(min(dx, dz) / 2 * 1e6) / 1e6


def gaussian_pixel_model(r, sigma):
    """Discretization.m:113-118."""
    return np.exp(-np.asarray(r) ** 2 / (2 * sigma ** 2))


# ----------------------------------------------------------------------------
# Prefilter (projection into the shift-invariant space)
# ----------------------------------------------------------------------------
def pixel_on_grid(grid: Grid) -> np.ndarray:
    """Discretization.m:74-86 with refinement 1: an (nz, nx) array."""
    dx, dz = grid.spacing()
    lx = dx * np.arange(np.floor(-grid.nx / 2), np.floor(grid.nx / 2 - 1) + 1)
    lz = dz * np.arange(np.floor(-grid.nz / 2), np.floor(grid.nz / 2 - 1) + 1)
    XX, ZZ = np.meshgrid(lx, lz)
    return gaussian_pixel_model(np.sqrt(XX ** 2 + ZZ ** 2), grid.sigma())


def prefilter(grid: Grid) -> np.ndarray:
    """shift_inv_proj.m:66-71 with lattice [1 1]; returns the (nz, nx) filter."""
    phi = np.fft.fftshift(pixel_on_grid(grid))
    phi_hat = np.fft.fft2(phi)
    autocorr = np.real(np.fft.ifft2(np.abs(phi_hat) ** 2))
    return np.conj(phi_hat / np.fft.fft2(autocorr))


def project(img_wxz: np.ndarray, pre: np.ndarray) -> np.ndarray:
    """Discretization.m:54-62 (circular filter per wavelength).

    img_wxz is (W, nx, nz); the MATLAB image is (nz, nx), i.e. the transpose
    of each numpy slice, so the filter is applied to (nz, nx) slices."""
    out = np.empty_like(img_wxz, dtype=np.float64)
    for w in range(img_wxz.shape[0]):
        m = img_wxz[w].T  # (nz, nx)
        out[w] = np.real(np.fft.ifft2(np.fft.fft2(m) * pre)).T
    return out


def project_transpose(img_wxz: np.ndarray, pre: np.ndarray) -> np.ndarray:
    """Discretization.m:64-72 (conjugate prefilter)."""
    return project(img_wxz, np.conj(pre))


def separable_prefilter_taps(n: int, spacing: float, sigma: float, tol: float = 1e-13,
                             kmax: int = 64) -> np.ndarray:
    """1-D circular kernel of the prefilter along one axis.

    The Gaussian pixel model is separable, phi(x, z) = g(x) g(z), so with
    lattice [1 1] the prefilter conj(phi_hat / |phi_hat|^2) factors into one
    circular filter per axis.  Returns taps h[-K..K] (length 2K+1, centre at
    index K) with |h[k]| < tol*|h[0]| for all dropped k."""
    lin = spacing * np.arange(np.floor(-n / 2), np.floor(n / 2 - 1) + 1)
    g = np.fft.fftshift(gaussian_pixel_model(lin, sigma))
    gh = np.fft.fft(g)
    ac = np.real(np.fft.ifft(np.abs(gh) ** 2))
    pre = np.conj(gh / np.fft.fft(ac))
    kern = np.real(np.fft.ifft(pre))  # circular kernel, index = offset mod n
    h0 = abs(kern[0])
    K = 0
    for k in range(1, n // 2):
        if abs(kern[k]) > tol * h0 or abs(kern[-k]) > tol * h0:
            K = k
    K = min(K, kmax, (n - 1) // 2)
    offs = np.arange(-K, K + 1)
    return kern[offs % n]


# ----------------------------------------------------------------------------
# Impulse response
# ----------------------------------------------------------------------------
def butter_zero_phase_response(n: int, fs: float, fmin: float, fmax: float) -> np.ndarray:
    """|H|^2 on n whole-circle bins (filter_butter_zero_phase.m:26-48):
    order-8 low-pass at fmax, order-2 high-pass at fmin, zp2sos, freqz."""
    zs, ps, k = [], [], 1.0
    if fmax > 0:
        z, p, kk = sps.butter(8, fmax * 2 / fs, "low", output="zpk")
        zs.append(z); ps.append(p); k *= kk
    if fmin > 0:
        z, p, kk = sps.butter(2, fmin * 2 / fs, "high", output="zpk")
        zs.append(z); ps.append(p); k *= kk
    if not zs:
        return np.ones(n)
    sos = sps.zpk2sos(np.concatenate(zs), np.concatenate(ps), k)
    _, h = sps.sosfreqz(sos, worN=n, whole=True)
    return np.abs(h) ** 2


def filter_butter_zero_phase(sig: np.ndarray, fs: float, fmin: float, fmax: float) -> np.ndarray:
    """filter_butter_zero_phase.m:16-48 with use_fft = true, along axis 0."""
    sig = np.asarray(sig, dtype=np.float64)
    if fmin > 0:
        sig = sig - sig.mean(axis=0, keepdims=True)
    H2 = butter_zero_phase_response(sig.shape[0], fs, fmin, fmax)
    H2 = H2.reshape((-1,) + (1,) * (sig.ndim - 1))
    return np.real(np.fft.ifft(H2 * np.fft.fft(sig, axis=0), axis=0))


def impulse_response(probe: ArcProbe, grid: Grid, c: float, fmin: float, fmax: float,
                     include_sir: bool = False) -> np.ndarray:
    """The model IR (MSOTmodel.m:320-348).  Without SIR it is the EIR
    convolved with the time derivative of the Gaussian pixel,
    phi(c t) * (-t), then zero-phase Butterworth filtered; with SIR only the
    EIR is filtered (the N-shape lives in the SIR table)."""
    eir = probe.eir_taps()
    if include_sir:
        return filter_butter_zero_phase(eir, probe.fs, fmin, fmax)
    L = eir.size
    h = (L - 1) // 2
    tk = np.arange(-h, h + 1) / probe.fs
    pmr = gaussian_pixel_model(tk * c, grid.sigma()) * (-tk)
    full = np.convolve(eir, pmr)  # convn(...,'same') keeps the centre
    ir = full[h:h + L]
    return filter_butter_zero_phase(ir, probe.fs, fmin, fmax)


def convolve_ir(sino_wdt: np.ndarray, ir: np.ndarray) -> np.ndarray:
    """MSOTmodel.m:259-263: linear FFT convolution, crop floor(L/2) each end."""
    T = sino_wdt.shape[-1]
    L = ir.size
    n = L + T - 1
    irh = np.fft.fft(ir, n)
    y = np.real(np.fft.ifft(np.fft.fft(sino_wdt, n, axis=-1) * irh, axis=-1))
    h = L // 2
    return y[..., h:n - h]


def convolve_ir_transpose(sino_wdt: np.ndarray, ir: np.ndarray) -> np.ndarray:
    """MSOTmodel.m:265-269: same with the flipped IR (exact adjoint)."""
    return convolve_ir(sino_wdt, ir[::-1].copy())


# ----------------------------------------------------------------------------
# Geometry tables
# ----------------------------------------------------------------------------
def travel_time_indices(probe: ArcProbe, grid: Grid, c: float, n_crop: int = 0) -> np.ndarray:
    """(D, P) fractional sample indices, MSOTmodel.m:380-381 with straight
    rays (refraction.m:23): |x_p - x_d| / c * fs - delay - n_crop."""
    xd, zd = probe.positions()
    X, Z = grid.pixel_xz()
    dist = np.sqrt((xd[:, None] - X[None, :]) ** 2 + (zd[:, None] - Z[None, :]) ** 2)
    return dist / c * probe.fs - probe.delay - n_crop


def travel_time_indices_dual(probe: ArcProbe, grid: Grid, c_below: float, c_above: float,
                             membrane, n_crop: int = 0):
    """(D, P) fractional sample indices and membrane intersections x_m for
    two speeds of sound separated by the membrane z = sum_k a_k x^k
    (refraction.m:8-24, fermat_principle.m:17-24, MSOTmodel.m:380-381).  A
    pixel with z > m(x) takes the path through (x_m, m(x_m)) that minimises
    |p - q| / c_below + |q - d| / c_above over [-R, R]: here a vectorised
    golden-section search to 1e-13 R, checked against scipy's bounded Brent
    method by the oracle tests; other pixels travel straight at c_above
    (x_m = NaN)."""
    a = np.asarray(membrane, dtype=np.float64)
    m = lambda x: np.polynomial.polynomial.polyval(x, a)
    xd, zd = probe.positions()
    X, Z = grid.pixel_xz()
    D, P = xd.size, X.size
    px, pz = np.broadcast_to(X[None, :], (D, P)), np.broadcast_to(Z[None, :], (D, P))
    dx, dz = np.broadcast_to(xd[:, None], (D, P)), np.broadcast_to(zd[:, None], (D, P))

    def T(x):
        mz = m(x)
        return (np.hypot(px - x, pz - mz) / c_below + np.hypot(x - dx, mz - dz) / c_above)

    R = probe.radius
    g = (np.sqrt(5.0) - 1.0) / 2.0
    lo, hi = np.full((D, P), -R), np.full((D, P), R)
    x1, x2 = hi - g * (hi - lo), lo + g * (hi - lo)
    f1, f2 = T(x1), T(x2)
    while np.max(hi - lo) > 1e-13 * R:
        left = f1 < f2
        hi = np.where(left, x2, hi)
        lo = np.where(left, lo, x1)
        xn = np.where(left, hi - g * (hi - lo), lo + g * (hi - lo))
        fn = T(xn)
        x2, f2, x1, f1 = (np.where(left, x1, xn), np.where(left, f1, fn),
                          np.where(left, xn, x2), np.where(left, fn, f2))
    xm = np.where(f1 < f2, x1, x2)
    t = np.minimum(f1, f2)
    below = pz > m(px)
    t = np.where(below, t, np.hypot(dx - px, dz - pz) / c_above)
    xm = np.where(below, xm, np.nan)
    return t * probe.fs - probe.delay - n_crop, xm


def virtual_sources(probe: ArcProbe, grid: Grid, c_below: float, c_above: float, membrane):
    """MSOTmodel.m:585-594: (virt_x, virt_z) [D][P], the point at distance
    t * c_above from the detector on its ray through the membrane
    intersection; the pixel itself where the path does not cross."""
    tau, xm = travel_time_indices_dual(probe, grid, c_below, c_above, membrane)
    t = (tau + probe.delay) / probe.fs
    xd, zd = probe.positions()
    X, Z = grid.pixel_xz()
    zm = np.polynomial.polynomial.polyval(xm, np.asarray(membrane, dtype=np.float64))
    qx, qz = xm - xd[:, None], zm - zd[:, None]
    n = np.hypot(qx, qz)
    vx = xd[:, None] + qx / n * t * c_above
    vz = zd[:, None] + qz / n * t * c_above
    nan = np.isnan(xm)
    vx = np.where(nan, np.broadcast_to(X[None, :], vx.shape), vx)
    vz = np.where(nan, np.broadcast_to(Z[None, :], vz.shape), vz)
    return vx, vz


def interpolation_radius(grid: Grid, probe: ArcProbe, c: float) -> float:
    """MSOTmodel.m:36-38."""
    _, z = grid.vectors()
    return (z[1] - z[0]) / (c / probe.fs)


# ----------------------------------------------------------------------------
# The operator
# ----------------------------------------------------------------------------
@dataclass
class Model:
    """FP64 MSOTmodel (single speed of sound).  ``norm`` is the
    model_normalization_factor (MSOTmodel.m:18); None -> 1 until
    :meth:`normalize` is called."""

    probe: ArcProbe
    grid: Grid
    c: float = 1500.0
    fmin: float = 1e5
    fmax: float = 12e6
    n_crop: int = 0
    include_sir: bool = False
    norm: float | None = None
    lib: object = None
    sir_tables: object = None  # (sir_ns, start_end_ns2, sir_idx_dp) when include_sir
    # dual speed of sound: membrane polynomial coefficients and the coupling
    # medium's speed of sound (Probe.membrane, Probe.coupling.speedOfSound)
    membrane: object = None
    c_coupling: float | None = None
    travel: np.ndarray = field(init=False)
    radius: float = field(init=False)
    ir: np.ndarray = field(init=False)
    pre: np.ndarray = field(init=False)

    def __post_init__(self):
        if self.membrane is None:
            self.travel = travel_time_indices(self.probe, self.grid, self.c, self.n_crop)
            c_ir = self.c
        else:
            self.travel, _ = travel_time_indices_dual(self.probe, self.grid, self.c,
                                                      self.c_coupling, self.membrane, self.n_crop)
            c_ir = self.c_coupling  # MSOTmodel.m:331-335
        self.radius = interpolation_radius(self.grid, self.probe, self.c)
        self.ir = impulse_response(self.probe, self.grid, c_ir, self.fmin, self.fmax,
                                   self.include_sir)
        self.pre = prefilter(self.grid)
        if self.lib is None:
            self.lib = native.port()

    @property
    def n_t(self) -> int:
        return int(self.probe.n_samples - self.n_crop)

    @property
    def shape_img(self):
        return (self.grid.nx, self.grid.nz)

    def _scale(self):
        return 1.0 / (self.norm if self.norm else 1.0)

    # --- raw MEX layer ------------------------------------------------------
    def mex_forward(self, coeffs_wp: np.ndarray) -> np.ndarray:
        """(W, P) -> (W, D, T) through the MEX operator."""
        x = np.ascontiguousarray(coeffs_wp.T)
        if self.include_sir:
            sir, se, idx = self.sir_tables
            y = self.lib.forward_sir(x, idx, self.travel, sir, self.n_t, se, self.radius)
        else:
            y = self.lib.forward_das(x, self.travel, self.n_t, self.radius)
        return np.ascontiguousarray(np.transpose(y, (2, 0, 1)))

    def mex_transpose(self, sino_wdt: np.ndarray) -> np.ndarray:
        y = np.ascontiguousarray(np.transpose(sino_wdt, (1, 2, 0)))
        if self.include_sir:
            sir, se, idx = self.sir_tables
            x = self.lib.transpose_sir(y, idx, self.travel, sir, se, self.radius)
        else:
            x = self.lib.transpose_das(y, self.travel, self.radius)
        return np.ascontiguousarray(x.T)

    # --- full operator -------------------------------------------------------
    def forward(self, img_wxz: np.ndarray) -> np.ndarray:
        """Funcs.applyForward (MSOTmodel.m:189-222, :285): (W,nx,nz)->(W,D,T)."""
        img = np.asarray(img_wxz, dtype=np.float64).reshape(-1, *self.shape_img)
        coeffs = project(img, self.pre).reshape(img.shape[0], -1)
        raw = self.mex_forward(coeffs)
        return convolve_ir(raw, self.ir) * self._scale()

    def transpose(self, sino_wdt: np.ndarray) -> np.ndarray:
        """Funcs.applyTranspose (MSOTmodel.m:224-257, :286): (W,D,T)->(W,nx,nz)."""
        s = np.asarray(sino_wdt, dtype=np.float64).reshape(-1, self.probe.n_det, self.n_t)
        s = convolve_ir_transpose(s, self.ir)
        x = self.mex_transpose(s).reshape(s.shape[0], *self.shape_img)
        return project_transpose(x, self.pre) * self._scale()

    def normalize(self, iters: int = 60, seed: int = 0) -> float:
        """sigma_max of the unnormalised operator (MSOTmodel.m:278 uses svds,
        50 iterations, tol 1e-8); here power iteration on A^T A in FP64."""
        self.norm = None
        self.norm = estimate_sigma_max(self.forward, self.transpose,
                                       (1,) + self.shape_img, iters, seed)
        return self.norm


def estimate_sigma_max(fwd, adj, shape, iters=60, seed=0) -> float:
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(shape)
    v /= np.linalg.norm(v)
    s = 0.0
    for _ in range(iters):
        u = adj(fwd(v))
        s = np.sqrt(np.linalg.norm(u))
        v = u / np.linalg.norm(u)
    return float(np.linalg.norm(fwd(v)))


# ----------------------------------------------------------------------------
# Synthetic inputs (seeded)
# ----------------------------------------------------------------------------
def gauss_pulse_eir(fs=4e7, fc=5e6, bw=0.6, n_taps=256, bwr=-6.0) -> np.ndarray:
    """Gaussian-modulated cosine (the published gausspulse definition):
    exp(-a t^2) cos(2 pi fc t), a = -(pi fc bw)^2 / (4 ln(10^(bwr/20))),
    sampled on n_taps taps centred at tap n_taps//2 and zero-padded to odd
    length n_taps+1 when n_taps is even."""
    ref = 10.0 ** (bwr / 20.0)
    a = -(np.pi * fc * bw) ** 2 / (4.0 * np.log(ref))
    k = np.arange(n_taps) - n_taps // 2
    t = k / fs
    e = np.exp(-a * t * t) * np.cos(2 * np.pi * fc * t)
    if n_taps % 2 == 0:
        e = np.concatenate([e, [0.0]])
    return e


def phantom(grid: Grid, rng: np.random.Generator, n_disks=(5, 15), r_disk=(0.3e-3, 3e-3),
            amp=(0.2, 1.0), n_vessels=3, vessel_width=0.2e-3) -> np.ndarray:
    """Disk + line-vessel phantom, (nx, nz) array (synthetic, seeded)."""
    X, Z = grid.pixel_xz()
    X = X.reshape(grid.nx, grid.nz)
    Z = Z.reshape(grid.nx, grid.nz)
    img = np.zeros((grid.nx, grid.nz))
    x0, x1, z0, z1 = grid.fov
    half = 0.8 * min(x1 - x0, z1 - z0) / 2
    for _ in range(int(rng.integers(n_disks[0], n_disks[1] + 1))):
        cx, cz = rng.uniform(-half, half, 2)
        rad = rng.uniform(*r_disk)
        a = rng.uniform(*amp)
        img[(X - cx) ** 2 + (Z - cz) ** 2 <= rad * rad] += a
    sig = vessel_width / 2.355  # FWHM = width
    for _ in range(n_vessels):
        px, pz = rng.uniform(-half, half, 2)
        th = rng.uniform(0, np.pi)
        nxv, nzv = -np.sin(th), np.cos(th)
        dist = (X - px) * nxv + (Z - pz) * nzv
        along = (X - px) * np.cos(th) + (Z - pz) * np.sin(th)
        L = rng.uniform(0.3, 0.8) * (x1 - x0)
        a = rng.uniform(*amp)
        img += a * np.exp(-dist ** 2 / (2 * sig * sig)) * (np.abs(along) <= L / 2)
    return img


def config1_probe(eir=True) -> ArcProbe:
    """256 elements, R = 40 mm, 135 deg, 2030 samples at 40 MHz, delay 0."""
    return ArcProbe(n_det=256, radius=0.040, coverage_deg=135.0, fs=4e7, n_samples=2030,
                    delay=0.0, eir=gauss_pulse_eir() if eir else None, eir_length=257)


def config_grid(n: int) -> Grid:
    """n x n grid over the fixed 25.4 mm FOV (0.2 mm pitch at n = 128)."""
    h = 0.2e-3 * 127 / 2
    return Grid(n, n, (-h, h, -h, h))


def noisy_sinogram(model: Model, img_xz: np.ndarray, rng, noise=0.01) -> np.ndarray:
    y = model.forward(img_xz[None])[0]
    return y + rng.standard_normal(y.shape) * noise * np.abs(y).max()
