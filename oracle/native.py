"""ctypes bindings of the CPU oracle libraries.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg.  The product never imports this module.

Two libraries, same calling convention (column-major MATLAB layouts, FP64):
  * ``port``: oracle/build/libmsotoracle.so -- the project's C restatement of
    the four MEX operators (msot_oracle.c), portable to aarch64.
  * ``ref``:  oracle/_ref/libmsotref.so -- the reference's own MEX sources
    compiled unmodified (x86_64 only; absent on other hosts).

Array conventions (numpy C-order shapes that are memory-identical to the
MATLAB column-major arrays of the MEX contracts, forwardMex.cpp:18-27):
  image      (P, W)     == MATLAB W x P
  sinogram   (D, T, W)  == MATLAB W x T x D
  travel     (D, P)     == MATLAB P x D
  sir        (NS, S)    == MATLAB S x NS
  start_end  (NS, 2)    == MATLAB 2 x NS   (1-based, inclusive)
  sir_idx    (D, P)     == MATLAB P x D    (1-based)
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(HERE, "build", "libmsotoracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libmsotref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_port() -> None:
    """Compile the C restatement (gcc only; no reference sources needed)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


class OracleLib:
    """One of the two oracle libraries; ``prefix`` is "orc" or "ref"."""

    def __init__(self, path: str, prefix: str):
        self.path = path
        self.prefix = prefix
        lib = C.CDLL(path)
        self._lib = lib
        f = getattr(lib, f"{prefix}_forward_das")
        f.argtypes = [_dp, C.c_int, C.c_int, _dp, C.c_int, C.c_int, C.c_double, _dp]
        f.restype = C.c_int
        self._fwd_das = f
        f = getattr(lib, f"{prefix}_transpose_das")
        f.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp, C.c_int, C.c_double, _dp]
        f.restype = C.c_int
        self._adj_das = f
        f = getattr(lib, f"{prefix}_forward_sir")
        f.argtypes = [_dp, C.c_int, C.c_int, _ip, _dp, C.c_int, _dp, C.c_int, C.c_int, C.c_int,
                      _ip, C.c_double, _dp]
        f.restype = C.c_int
        self._fwd_sir = f
        f = getattr(lib, f"{prefix}_transpose_sir")
        f.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _ip, _dp, C.c_int, _dp, C.c_int, C.c_int,
                      _ip, C.c_double, _dp]
        f.restype = C.c_int
        self._adj_sir = f
        self._set_threads = getattr(lib, f"{prefix}_set_threads")
        self._set_threads.argtypes = [C.c_int]
        self._max_threads = getattr(lib, f"{prefix}_max_threads")
        self._max_threads.restype = C.c_int

    def set_threads(self, n: int) -> None:
        self._set_threads(int(n))

    def max_threads(self) -> int:
        return int(self._max_threads())

    @staticmethod
    def _c(a, dt=np.float64):
        return np.ascontiguousarray(a, dtype=dt)

    def forward_das(self, image_pw, travel_dp, n_t, radius):
        image_pw = self._c(image_pw)
        travel_dp = self._c(travel_dp)
        P, W = image_pw.shape
        D = travel_dp.shape[0]
        out = np.empty((D, n_t, W))
        rc = self._fwd_das(image_pw, W, P, travel_dp, D, n_t, float(radius), out)
        if rc:
            raise ValueError(f"{self.prefix}_forward_das rejected its inputs (rc={rc})")
        return out

    def transpose_das(self, sig_dtw, travel_dp, radius):
        sig_dtw = self._c(sig_dtw)
        travel_dp = self._c(travel_dp)
        D, T, W = sig_dtw.shape
        P = travel_dp.shape[1]
        out = np.empty((P, W))
        rc = self._adj_das(sig_dtw, W, T, D, travel_dp, P, float(radius), out)
        if rc:
            raise ValueError(f"{self.prefix}_transpose_das rejected its inputs (rc={rc})")
        return out

    def forward_sir(self, image_pw, sir_idx_dp, travel_dp, sir_ns, n_t, start_end_ns2, radius):
        image_pw = self._c(image_pw)
        travel_dp = self._c(travel_dp)
        sir_ns = self._c(sir_ns)
        sir_idx_dp = self._c(sir_idx_dp, np.int32)
        start_end_ns2 = self._c(start_end_ns2, np.int32)
        P, W = image_pw.shape
        D = travel_dp.shape[0]
        NS, S = sir_ns.shape
        out = np.empty((D, n_t, W))
        rc = self._fwd_sir(image_pw, W, P, sir_idx_dp, travel_dp, D, sir_ns, S, NS, n_t,
                           start_end_ns2, float(radius), out)
        if rc:
            raise ValueError(f"{self.prefix}_forward_sir rejected its inputs (rc={rc})")
        return out

    def transpose_sir(self, sig_dtw, sir_idx_dp, travel_dp, sir_ns, start_end_ns2, radius):
        sig_dtw = self._c(sig_dtw)
        travel_dp = self._c(travel_dp)
        sir_ns = self._c(sir_ns)
        sir_idx_dp = self._c(sir_idx_dp, np.int32)
        start_end_ns2 = self._c(start_end_ns2, np.int32)
        D, T, W = sig_dtw.shape
        P = travel_dp.shape[1]
        NS, S = sir_ns.shape
        out = np.empty((P, W))
        rc = self._adj_sir(sig_dtw, W, T, D, sir_idx_dp, travel_dp, P, sir_ns, S, NS,
                           start_end_ns2, float(radius), out)
        if rc:
            raise ValueError(f"{self.prefix}_transpose_sir rejected its inputs (rc={rc})")
        return out


_cache: dict = {}


def port() -> OracleLib:
    """The C restatement; built on first use if missing."""
    if "port" not in _cache:
        if not os.path.exists(PORT_PATH):
            build_port()
        _cache["port"] = OracleLib(PORT_PATH, "orc")
    return _cache["port"]


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref() -> OracleLib:
    """The reference's own MEX code (only where it was compiled: x86_64)."""
    if "ref" not in _cache:
        if not ref_available():
            raise FileNotFoundError(REF_PATH)
        _cache["ref"] = OracleLib(REF_PATH, "ref")
    return _cache["ref"]
