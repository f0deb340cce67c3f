"""On-disk cache of the model's geometry tables, the role of the reference's
acoustic_file_<hash>.mat / polarSPMR_*.mat files (MSOTmodel.m:289-318,
350-382, 482-548).

The key of a travel-time table hashes the fields of
hash_to_load_and_save_acoustic_data (MSOTmodel.m:289-308): coupling and
medium speed of sound, detector positions, the pixel region, the single /
dual speed-of-sound flag and the membrane sampled at the pixel columns (Inf
for a single speed of sound), plus the sampling rate, delay and crop the
stored indices include.  The reference hashes with DataHash (MD5 of MATLAB's
serialisation); here SHA-256 of the little-endian FP64 bytes of the same
fields, so the files are not interchangeable with the reference's.  As in
the reference a file whose stored fields differ from the model's is a hash
collision and raises.  SPMR tables are keyed by every field of their
specification and reused only on an exact match (the reference also reuses
a coarser-request-covering table; not provided).
"""
from __future__ import annotations

import hashlib
import os

import numpy as np


def _fields_acoustic(probe, disc, c, n_crop, single_sos: bool):
    xd, zd = probe.detector_positions()
    X = np.asarray(disc.x, dtype=np.float64)
    if single_sos:
        c_coupling = float(c)
        membrane = np.full(X.size, np.inf)
    else:
        c_coupling = float(probe.coupling_speed_of_sound)
        membrane = np.polynomial.polynomial.polyval(X, np.asarray(probe.membrane, dtype=np.float64))
    return {
        "coupling_speed_of_sound": np.array([c_coupling]),
        "detector_x": np.asarray(xd, dtype=np.float64),
        "detector_z": np.asarray(zd, dtype=np.float64),
        "medium_speed_of_sound": np.array([float(c)]),
        "region_x": X,
        "region_z": np.asarray(disc.z, dtype=np.float64),
        "use_single_sos": np.array([1.0 if single_sos else 0.0]),
        "membrane": membrane,
        "dac": np.array([float(probe.fs), float(probe.delay), float(n_crop)]),
    }


def _digest(fields: dict) -> str:
    h = hashlib.sha256()
    for k in sorted(fields):
        h.update(k.encode())
        h.update(np.ascontiguousarray(fields[k], dtype="<f8").tobytes())
    return h.hexdigest()[:32]


def _check(path, stored: dict, fields: dict):
    for k, v in fields.items():
        if k not in stored or not np.array_equal(stored[k], v):
            raise RuntimeError(f"hash collision: {path} was written for another model "
                               f"(field {k}); delete the outdated table file")


def acoustic_tables(cache_dir, probe, disc, c, n_crop, single_sos, compute):
    """Travel-time indices (and membrane intersections, None for a single
    speed of sound) from cache_dir/acoustic_file_<key>.npz, or compute() ->
    (travel, x_mem) and store them."""
    fields = _fields_acoustic(probe, disc, c, n_crop, single_sos)
    path = os.path.join(cache_dir, f"acoustic_file_{_digest(fields)}.npz")
    if os.path.exists(path):
        with np.load(path) as z:
            stored = {k[6:]: z[k] for k in z.files if k.startswith("field_")}
            _check(path, stored, fields)
            travel = np.array(z["travel"])
            xm = np.array(z["x_membrane_intersections"]) if "x_membrane_intersections" in z.files \
                else None
        return travel, xm
    travel, xm = compute()
    os.makedirs(cache_dir, exist_ok=True)
    data = {f"field_{k}": v for k, v in fields.items()}
    data["travel"] = travel
    if xm is not None:
        data["x_membrane_intersections"] = xm
    tmp = path + ".tmp.npz"
    np.savez(tmp, **data)
    os.replace(tmp, path)
    return travel, xm


def spmr_tables(cache_dir, spec_fields: dict, compute):
    """(sir, start_end, sir_idx, meta) from cache_dir/polarSPMR_<key>.npz, or
    compute() and store."""
    fields = {k: np.atleast_1d(np.asarray(v, dtype=np.float64)) for k, v in spec_fields.items()}
    path = os.path.join(cache_dir, f"polarSPMR_{_digest(fields)}.npz")
    if os.path.exists(path):
        with np.load(path) as z:
            stored = {k[6:]: z[k] for k in z.files if k.startswith("field_")}
            _check(path, stored, fields)
            meta = {k[5:]: float(z[k][0]) if k != "meta_half_window" else int(z[k][0])
                    for k in z.files if k.startswith("meta_")}
            for k in ("n_dist", "n_angle"):
                if k in meta:
                    meta[k] = int(meta[k])
            return np.array(z["sir"]), np.array(z["start_end"]), np.array(z["sir_idx"]), meta
    sir, se, idx, meta = compute()
    os.makedirs(cache_dir, exist_ok=True)
    data = {f"field_{k}": v for k, v in fields.items()}
    data.update(sir=sir, start_end=se, sir_idx=idx)
    data.update({f"meta_{k}": np.array([v]) for k, v in meta.items()})
    tmp = path + ".tmp.npz"
    np.savez(tmp, **data)
    os.replace(tmp, path)
    return sir, se, idx, meta
