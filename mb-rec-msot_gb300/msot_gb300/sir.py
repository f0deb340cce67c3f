"""SPMR (spatial pixel model response) tables for include_sir models.

The role of the reference's calculate_polarSPMR.m:21-184 and
MSOTmodel.get_SPMR_and_SPMR_indices (MSOTmodel.m:463-480), computed by
msot_spmr_query / msot_spmr_tables on the GPU.  The reference obtains the
element's spatial impulse response from Field II, which is not available;
here it is the Rayleigh integral over sub_x x sub_y point sources on the
element (flat, or curved in elevation).  The default element is the
0.25 mm x 10 mm element sampled 8 x 8.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _spec(probe, disc, c, element, sub, half_window, virtual=None):
    width, height, elev_radius = element
    x = np.ascontiguousarray(disc.x, dtype=np.float64)
    z = np.ascontiguousarray(disc.z, dtype=np.float64)
    s = _lib.SpmrSpec()
    s.n_det, s.radius, s.coverage_deg = int(probe.n_det), float(probe.radius), \
        float(probe.angular_coverage)
    s.x, s.nx = x.ctypes.data_as(_lib._dp), x.size
    s.z, s.nz = z.ctypes.data_as(_lib._dp), z.size
    s.c, s.fs, s.pixel_sigma = float(c), float(probe.fs), float(disc.sigma)
    s.elem_width, s.elem_height = float(width), float(height)
    s.elem_elev_radius = float(elev_radius or 0.0)
    s.sub_x, s.sub_y = int(sub[0]), int(sub[1])
    s.half_window = int(half_window)
    keep = [x, z]
    if virtual is not None:
        vx, vz = (np.ascontiguousarray(v, dtype=np.float64) for v in virtual)
        if vx.shape != (probe.n_det, disc.nx * disc.nz) or vz.shape != vx.shape:
            raise ValueError("virtual sources must be [n_det][nx*nz]")
        s.virt_x, s.virt_z = vx.ctypes.data_as(_lib._dp), vz.ctypes.data_as(_lib._dp)
        keep += [vx, vz]
    return s, keep


def spmr_tables(probe, disc, c: float, element=(0.25e-3, 10e-3, 0.0), sub=(8, 8),
                half_window: int = 45, virtual=None, cache_dir=None):
    """Returns (sir [NS][S], start_end [NS][2], sir_idx [n_det][P], info) in the
    layout MSOTmodel(include_sir=True, sir_tables=(sir, start_end, sir_idx))
    takes.  The half window grows (as calculate_polarSPMR.m:115-139 does) until
    every column's response fits.  With two speeds of sound pass c = the
    coupling medium's speed and virtual = (virt_x, virt_z) from
    virtual_sources (MSOTmodel.m:579-596).  cache_dir keeps the tables on
    disk keyed by every input (msot_gb300.cache)."""
    if cache_dir:
        from . import cache
        xd, zd = probe.detector_positions()
        fields = dict(detector_x=xd, detector_z=zd, x=disc.x, z=disc.z, c=c, fs=probe.fs,
                      sigma=disc.sigma, element=element, sub=sub, half_window=half_window)
        if virtual is not None:
            fields.update(virt_x=np.ravel(virtual[0]), virt_z=np.ravel(virtual[1]))
        return cache.spmr_tables(cache_dir, fields, lambda: spmr_tables(
            probe, disc, c, element, sub, half_window, virtual))
    L = _lib.load()
    hw = int(half_window)
    while True:
        s, keep = _spec(probe, disc, c, element, sub, hw, virtual)
        info = _lib.SpmrInfo()
        rc = L.msot_spmr_query(C.byref(s), C.byref(info))
        if rc == -2 and b"widen" in (L.msot_last_error() or b"") and hw < 4096:
            hw *= 2
            continue
        _lib.check(rc)
        break
    sir = np.empty((info.n_sir, info.sir_len), dtype=np.float64)
    se = np.empty((info.n_sir, 2), dtype=np.int32)
    idx = np.empty((probe.n_det, disc.nx * disc.nz), dtype=np.int32)
    _lib.check(L.msot_spmr_tables(C.byref(s), sir.ctypes.data_as(_lib._dp),
                                  se.ctypes.data_as(_lib._ip), idx.ctypes.data_as(_lib._ip)))
    meta = dict(d_min=info.d_min, d_step=info.d_step, a_step_deg=info.a_step_deg,
                n_dist=info.n_dist, n_angle=info.n_angle, half_window=hw)
    return sir, se, idx, meta


def virtual_sources(probe, disc, c_below: float):
    """(virt_x, virt_z) [n_det][nx*nz]: the virtual source of every pixel for
    every detector with two speeds of sound (MSOTmodel.m:585-594), from
    msot_travel_times_dual with the probe's membrane and coupling speed."""
    from .model import travel_times_dual
    _, _, vx, vz = travel_times_dual(probe, disc, c_below, probe.coupling_speed_of_sound,
                                     probe.membrane, virtual=True)
    return vx, vz
