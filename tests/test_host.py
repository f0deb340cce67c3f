"""CPU tests of the product's host-side logic against the oracle, and of the
C-ABI library's exports (no device calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import model as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_discretization_taps_match_oracle():
    from msot_gb300 import Discretization
    for n in (128, 200, 101):
        d = Discretization([-0.0127, 0.0127], n)
        tx, tz = d.prefilter_taps()
        g = M.Grid(n, n, (-0.0127, 0.0127, -0.0127, 0.0127))
        ox = M.separable_prefilter_taps(n, g.spacing()[0], g.sigma())
        K = min(tx.size, ox.size) // 2
        cx, co = tx.size // 2, ox.size // 2
        assert np.allclose(tx[cx - K:cx + K + 1], ox[co - K:co + K + 1], rtol=0, atol=1e-15)


def test_impulse_response_and_travel_times_match_oracle():
    from msot_gb300 import Discretization, Probe
    from msot_gb300.model import model_impulse_response
    eir = M.gauss_pulse_eir()
    p = Probe(eir=eir)
    d = Discretization([-0.0127, 0.0127], 128)
    ir = model_impulse_response(p, d, 1500.0, 1e5, 12e6, False)
    op = M.config1_probe()
    og = M.config_grid(128)
    ref = M.impulse_response(op, og, 1500.0, 1e5, 12e6)
    assert np.allclose(ir, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    ir_sir = model_impulse_response(p, d, 1500.0, 1e5, 12e6, True)
    ref_sir = M.impulse_response(op, og, 1500.0, 1e5, 12e6, include_sir=True)
    assert np.allclose(ir_sir, ref_sir, rtol=0, atol=1e-12 * np.abs(ref_sir).max())
    xd, zd = p.detector_positions()
    oxd, ozd = op.positions()
    assert np.allclose(xd, oxd, atol=1e-15) and np.allclose(zd, ozd, atol=1e-15)


def declared_symbols():
    with open(os.path.join(ROOT, "include", "msot_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(msot_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from msot_gb300 import _build, _lib
    path = _lib.lib_path()
    if not os.path.exists(path):
        _build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 16
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # every declared symbol also has a Python binding
    assert set(syms) <= set(_lib.SIGNATURES), set(syms) - set(_lib.SIGNATURES)


def test_library_reports_errors_without_a_device():
    from msot_gb300 import _lib
    L = _lib.load(build_if_missing=True)
    assert L.msot_version() >= 1
    h = ctypes.c_void_p()
    rc = L.msot_plan_create(None, ctypes.byref(h))
    assert rc == -1 and b"plan" in L.msot_last_error()


@pytest.mark.parametrize("name", ["forwardDelayAndSumMex", "transposeDelayAndSumMex",
                                  "forwardMex", "transposeMex"])
def test_mex_gateways_compile_against_the_mex_api(name, tmp_path):
    """The MATLAB gateways of the C ABI compile against the MEX API (the
    project's stand-in header here, MATLAB's mex.h on a MATLAB host)."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("no g++")
    src = os.path.join(ROOT, "mb-rec-msot_gb300", "mex", name + ".cpp")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I",
                        os.path.join(ROOT, "oracle", "mex_shim"), "-I",
                        os.path.join(ROOT, "include"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("order,btype,wn,n,whole", [
    (8, "low", 2 * 12e6 / 4e7, 2030, True),      # filter_butter_zero_phase low-pass
    (2, "high", 2 * 1e5 / 4e7, 2030, True),      # and high-pass
    (2, "bandpass", (300 / 2030, 1830 / 2030), 2030, False),  # the sinogram window
    (4, "bandpass", (0.1, 0.45), 777, False),
    (3, "low", 0.2, 64, False),
])
def test_butterworth_design_matches_scipy(order, btype, wn, n, whole):
    # the library's own Butterworth design (host code, no GPU) against
    # scipy.signal's, evaluated on the same grid
    import scipy.signal as sps
    from msot_gb300 import _lib
    from msot_gb300.preprocess import butter_response
    _lib.load(build_if_missing=True)
    got = butter_response(order, btype, wn, n, whole)
    z, p, k = sps.butter(order, wn, btype, output="zpk")
    _, h = sps.freqz_zpk(z, p, k, worN=n, whole=whole)
    assert np.max(np.abs(got - np.abs(h))) <= 1e-10 * max(1.0, np.abs(h).max())


def test_butterworth_window_matches_oracle():
    from oracle import preprocess as Q
    from msot_gb300 import _lib
    from msot_gb300.preprocess import butter_response
    _lib.load(build_if_missing=True)
    T = 2030
    got = butter_response(2, "bandpass", (300 / T, (T - 200) / T), T)
    assert np.max(np.abs(got - Q.butter_window(T, 2, 300, T - 200))) <= 1e-10


def test_table_cache_round_trip_and_collision(tmp_path):
    # the acoustic-table cache (MSOTmodel.m:289-308, 350-379): stored on the
    # first call, loaded (without computing) on the second, a file written for
    # other fields is a hash collision
    from msot_gb300 import Discretization, Probe
    from msot_gb300 import cache
    probe = Probe(n_det=8)
    disc = Discretization([-0.003, 0.003], 6)
    calls = []

    def compute():
        calls.append(1)
        return np.arange(8 * 36, dtype=np.float64).reshape(8, 36), None

    t1, x1 = cache.acoustic_tables(str(tmp_path), probe, disc, 1500.0, 0, True, compute)
    t2, x2 = cache.acoustic_tables(str(tmp_path), probe, disc, 1500.0, 0, True, compute)
    assert len(calls) == 1 and np.array_equal(t1, t2) and x2 is None
    # a different speed of sound is another key (no collision, computed again)
    cache.acoustic_tables(str(tmp_path), probe, disc, 1510.0, 0, True, compute)
    assert len(calls) == 2
    # tamper with a stored field: loading reports the collision
    import glob
    f = sorted(glob.glob(str(tmp_path / "acoustic_file_*.npz")))[0]
    with np.load(f) as z:
        data = {k: z[k] for k in z.files}
    data["field_region_x"] = data["field_region_x"] + 1.0
    np.savez(f, **data)
    with pytest.raises(RuntimeError, match="collision"):
        for c in (1500.0, 1510.0):
            cache.acoustic_tables(str(tmp_path), probe, disc, c, 0, True, compute)
    # SPMR tables: exact-match reuse
    spec = dict(c=1500.0, sub=(8, 8))
    mk = lambda: (np.ones((3, 5)), np.ones((3, 2), np.int32), np.ones((8, 36), np.int32),
                  dict(d_min=0.01, d_step=1e-4, a_step_deg=0.1, n_dist=3, n_angle=1,
                       half_window=45))
    a = cache.spmr_tables(str(tmp_path), spec, mk)
    b = cache.spmr_tables(str(tmp_path), spec, lambda: 1 / 0)
    assert np.array_equal(a[0], b[0]) and b[3]["half_window"] == 45 and b[3]["n_dist"] == 3


def test_bp_kernel_matches_oracle():
    # the library's real-arithmetic form (K = M - M^T) against the oracle's
    # complex Hankel product (bp_kernel.m:1-12)
    from oracle import backprojection as B
    from msot_gb300.analytic import bp_kernel
    t = np.arange(1, 301) / 4e7
    K = bp_kernel(t)
    R = B.bp_kernel(t)
    assert np.max(np.abs(K - R)) <= 1e-9 * np.abs(R).max()
    assert np.max(np.abs(K + K.T)) <= 1e-12 * np.abs(K).max()


def test_new_entry_points_reject_bad_arguments_without_a_device():
    # argument checks run before any device work, so they hold on any host
    from msot_gb300 import _lib
    L = _lib.load(build_if_missing=True)
    D = ctypes.POINTER(ctypes.c_double)
    out = (ctypes.c_double * 16)()
    x = (ctypes.c_double * 4)(0.0, 1e-3, 2e-3, 3e-3)
    a = (ctypes.c_double * 9)(*([0.0] * 9))
    h = ctypes.c_void_p()
    cases = [
        # pre-processing: low >= high, cut-off above Nyquist, nothing left after the crop
        (lambda: L.msot_prep_create(100, 0, 2, 50.0, 40.0, 4e7, 0.0, 0.0, 4, ctypes.byref(h)),
         b"prep_create"),
        (lambda: L.msot_prep_create(100, 0, 0, 0.0, 0.0, 4e7, 0.0, 3e7, 4, ctypes.byref(h)),
         b"prep_create"),
        (lambda: L.msot_prep_create(10, 9, 0, 0.0, 0.0, 0.0, 0.0, 0.0, 4, ctypes.byref(h)),
         b"prep_create"),
        (lambda: L.msot_prep_apply(None, None, None, 1, None), b"prep_apply"),
        (lambda: L.msot_butter_response(8, 0, 1.5, 0.0, 16, 0, ctypes.cast(out, D)),
         b"butter_response"),
        # dual speed of sound: no or too many membrane coefficients, one of the
        # two virtual-source outputs
        (lambda: L.msot_travel_times_dual(4, 0.04, 135.0, x, 4, x, 4, 1500.0, 1480.0, a, 0,
                                          4e7, 0.0, 0.0, ctypes.cast(out, D), None, None, None),
         b"travel_times_dual"),
        (lambda: L.msot_travel_times_dual(4, 0.04, 135.0, x, 4, x, 4, 1500.0, 1480.0, a, 9,
                                          4e7, 0.0, 0.0, ctypes.cast(out, D), None, None, None),
         b"travel_times_dual"),
        (lambda: L.msot_travel_times_dual(4, 0.04, 135.0, x, 4, x, 4, 1500.0, 1480.0, a, 2,
                                          4e7, 0.0, 0.0, ctypes.cast(out, D), None,
                                          ctypes.cast(out, D), None),
         b"travel_times_dual"),
        (lambda: L.msot_rec_nn_with_L2_reg_2(None, None, None, 1, 1, 1e-2, 1e-2, None, 0, None,
                                             None, None, None), b"rec_nn_with_L2_reg_2"),
        (lambda: L.msot_laplacian_per_wavelength(None, None, 1, 4, 4, None),
         b"laplacian_per_wavelength"),
        (lambda: L.msot_autotune(None, 1, None, None), b"autotune"),
        (lambda: L.msot_l2_gather_probe(1024, ctypes.cast(out, D)), b"l2_gather_probe"),
        (lambda: L.msot_tune_set(b"no_such_knob", 1), b"tune_set"),
        (lambda: L.msot_tune_set(b"conv_min_blocks", 2), b"tune_set"),
        (lambda: L.msot_tune_set(b"fwd_ell", 2), b"tune_set"),
        (lambda: L.msot_tune_set(b"tv_prox_cluster", -2), b"tune_set"),
        # storage format outside 0 .. 2, no plan
        (lambda: L.msot_plan_set_storage(None, 3, 0), b"plan_set_storage"),
        (lambda: L.msot_plan_set_storage(None, 2, 0), b"plan_set_storage"),
        # the state-returning L2 solve: no plan / no v output / v0 without w0
        (lambda: L.msot_rec_nn_with_L2_reg_state(None, None, None, None, 1, 1, 1e-2, None,
                                                 None, 0, None, None, None),
         b"rec_nn_with_L2_reg_state"),
        # U-Net input channels 1 .. 8
        (lambda: L.msot_unet_create_ch(3, 8, 0, 32, 4, 0, ctypes.byref(h)), b"unet_create"),
        (lambda: L.msot_unet_create_ch(3, 8, 9, 32, 4, 0, ctypes.byref(h)), b"unet_create"),
    ]
    for call, where in cases:
        rc = call()
        assert rc == -1, where
        assert where in L.msot_last_error(), (where, L.msot_last_error())


def test_last_error_is_per_thread():
    """msot_last_error() reports the calling thread's own last failure: two
    threads that fail in different entry points at the same time each read
    their own message (argument checks only, no device work)."""
    import threading
    from msot_gb300 import _lib
    L = _lib.load(build_if_missing=True)
    start = threading.Barrier(2)
    seen = {}

    def worker(name, call, where):
        start.wait()
        msgs = []
        for _ in range(200):
            assert call() == -1
            msgs.append(L.msot_last_error())
        seen[name] = (where, msgs)

    h = ctypes.c_void_p()
    threads = [
        threading.Thread(target=worker, args=(
            "plan", lambda: L.msot_plan_create(None, ctypes.byref(h)), b"plan")),
        threading.Thread(target=worker, args=(
            "tune", lambda: L.msot_tune_set(b"no_such_knob", 1), b"tune_set")),
    ]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert set(seen) == {"plan", "tune"}
    for where, msgs in seen.values():
        assert all(where in m for m in msgs), (where, set(msgs))
    assert not any(b"tune_set" in m for m in seen["plan"][1])


def test_mex_gateways_raise_the_reference_error_ids(tmp_path):
    """Each gateway, given one input of the wrong class at a time, raises the
    error ID and message the reference's MEX raises for it
    (forwardMex.cpp:30-50, transposeMex.cpp:30-47,
    forwardDelayAndSumMex.cpp:27-38, transposeDelayAndSumMex.cpp:26-34).
    Where the reference's MEX code was compiled (x86 hosts) the harness calls
    it too and the two must agree line by line; elsewhere the gateways are
    checked against the expected IDs.  No device work: every call stops at
    the class check."""
    import shutil
    import subprocess
    from msot_gb300 import _build, _lib
    from oracle import native
    if not shutil.which("g++"):
        pytest.skip("no g++")
    lib = _lib.lib_path()
    if not os.path.exists(lib):
        _build.build()
    shim = os.path.join(ROOT, "oracle", "mex_shim")
    inc = os.path.join(ROOT, "include")
    objs = []
    for name in ("forwardDelayAndSumMex", "transposeDelayAndSumMex", "forwardMex",
                 "transposeMex"):
        o = str(tmp_path / f"{name}.o")
        src = os.path.join(ROOT, "mb-rec-msot_gb300", "mex", name + ".cpp")
        subprocess.run(["g++", "-std=c++17", "-O1", "-fPIC", f"-DmexFunction=gw_{name}",
                        "-I", shim, "-I", inc, "-c", src, "-o", o], check=True)
        objs.append(o)
    with_ref = native.ref_available()
    exe = str(tmp_path / "harness")
    cmd = ["g++", "-std=c++17", "-O1", "-I", shim,
           os.path.join(ROOT, "tests", "mex_error_harness.cpp"), *objs, "-o", exe,
           "-L", os.path.dirname(lib), "-lmsotgpu", "-Wl,-rpath," + os.path.dirname(lib)]
    if with_ref:
        cmd[3:3] = ["-DWITH_REF"]
        cmd += [native.REF_PATH, "-Wl,-rpath," + os.path.dirname(native.REF_PATH), "-fopenmp"]
    subprocess.run(cmd, check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    rows = {}
    for line in out:
        who, name, k, rest = line.split(" ", 3)
        rows[(who, name, int(k))] = rest
    classes = {"forwardDelayAndSumMex": "ddid", "transposeDelayAndSumMex": "ddd",
               "forwardMex": "diddiid", "transposeMex": "diddid"}
    for name, cl in classes.items():
        for k, c in enumerate(cl):
            got = rows[("gw", name, k)]
            want_id = "forwardMex:notInt32" if c == "i" else "forwardMex:notDouble"
            assert got.startswith(want_id + "|"), (name, k, got)
            assert got.endswith(" must be type int32." if c == "i" else " must be type double.")
            if with_ref:
                assert got == rows[("ref", name, k)], (name, k, got, rows[("ref", name, k)])
        assert rows[("gw", name, -1)].startswith("forwardMex:nrhs|"), name


def test_sb_itv2_mirror_takes_the_reference_signature():
    """SB_ITV2(g, mu, B, Bt, BtB) as PsiForTVReg.m:6 calls it: the operators
    of DiffOper(n) are accepted (the kernel applies that operator itself) and
    operators of another size are refused before any device work; SB_ITV is
    the library's own two-argument entry point."""
    import inspect
    import msot_gb300 as m
    from oracle import solvers as S
    assert list(inspect.signature(m.SB_ITV2).parameters)[:5] == ["g", "mu", "B", "Bt", "BtB"]
    assert list(inspect.signature(m.SB_ITV).parameters)[:2] == ["g", "mu"]
    B, Bt, BtB = S.diff_oper(5)
    g = np.zeros((6, 6))
    for bad in ((B, None, None), (None, Bt, None), (None, None, BtB)):
        with pytest.raises(ValueError, match="DiffOper"):
            m.SB_ITV2(g, 0.1, *bad)
    with pytest.raises(ValueError, match="square"):
        m.SB_ITV2(np.zeros((6, 5)), 0.1)


def test_analytic_mirror_accepts_the_reference_meshgrids():
    """dmas_cf / backproject_waveeq receive region.xPositionsFov and
    zPositionsFov, Nz x Nx meshgrid matrices (reconstruct_dmas_cf.m:6-7);
    the mirror reads the same coordinate vectors from them as from plain
    vectors, and refuses a matrix that is not a meshgrid."""
    from msot_gb300 import analytic as A
    x = np.linspace(-1e-3, 1e-3, 7)
    z = np.linspace(-2e-3, 1e-3, 5)
    X, Z = np.meshgrid(x, z)  # Nz x Nx, as MATLAB's meshgrid
    assert np.array_equal(A._fov_axis(X, "x"), x)
    assert np.array_equal(A._fov_axis(Z, "z"), z)
    assert np.array_equal(A._fov_axis(x, "x"), x)
    assert np.array_equal(A._fov_axis(z[:, None], "z"), z)
    with pytest.raises(ValueError, match="meshgrid"):
        A._fov_axis(Z, "x")
    with pytest.raises(ValueError, match="meshgrid"):
        A._fov_axis(np.random.default_rng(0).random((5, 7)), "z")


def test_discretization_exposes_the_reference_region():
    """Discretization.region.xPositionsFov / zPositionsFov are MATLAB's
    meshgrid(x, z) (Discretization.m:34), Nz x Nx, and numberOfPixels /
    sizeOfPixelGrid follow the reference's names."""
    from msot_gb300 import Discretization
    from msot_gb300 import analytic as A
    d = Discretization([-0.005, 0.005, -0.004, 0.006], (9, 7))
    X, Z = d.region.xPositionsFov, d.region.zPositionsFov
    assert X.shape == (7, 9) and Z.shape == (7, 9)
    assert np.array_equal(X[0], d.x) and np.array_equal(Z[:, 0], d.z)
    assert d.numberOfPixels == 63 and d.sizeOfPixelGrid == (9, 7)
    assert np.array_equal(A._fov_axis(X, "x"), d.x)
    assert np.array_equal(A._fov_axis(Z, "z"), d.z)


class _FakeLib:
    """Records the C-ABI calls a Python wrapper makes (returns MSOT_OK)."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def call(*args):
            self.calls.append((name, args))
            return 0
        return call


def _host_only(monkeypatch):
    """Run the wrappers' host logic without a device: tensors stay on the
    CPU and the library is a recorder."""
    import torch
    from msot_gb300 import _lib, analytic, solvers
    fake = _FakeLib()
    monkeypatch.setattr(_lib, "load", lambda *a, **k: fake)
    monkeypatch.setattr(torch.Tensor, "cuda", lambda self, *a, **k: self)
    monkeypatch.setattr(analytic, "_stream_ptr", lambda stream=None: None)
    monkeypatch.setattr(solvers, "_stream_ptr", lambda stream=None: None)
    return fake


def test_analytic_wrappers_pass_the_grid_sizes(monkeypatch):
    """dmas_cf and backproject_waveeq hand the library the sinogram shape and
    the fov vector lengths, whether the fov comes as vectors or as the
    reference's meshgrids."""
    from msot_gb300 import analytic as A
    fake = _host_only(monkeypatch)
    x = np.linspace(-1e-3, 1e-3, 7)
    z = np.linspace(-2e-3, 1e-3, 5)
    X, Z = np.meshgrid(x, z)
    sig = np.zeros((3, 16, 40), dtype=np.float32)
    for fx, fz in ((x, z), (X, Z)):
        outs = A.dmas_cf(sig, fx, fz, 1500.0, 4e7, 0, 135.0, 0.04)
        name, args = fake.calls[-1]
        assert name == "msot_dmas_cf" and args[1:4] == (3, 16, 40)
        assert args[5] == 7 and args[7] == 5
        assert all(tuple(o.shape) == (3, 7, 5) for o in outs)
        out = A.backproject_waveeq(sig, fx, fz, 1500.0, 4e7, 0, 135.0, 0.04, np.ones((1, 1)),
                                   np.eye(40))
        name, args = fake.calls[-1]
        assert name == "msot_backproject_waveeq" and args[1:4] == (3, 16, 40)
        assert args[5] == 7 and args[7] == 5 and tuple(out.shape) == (3, 7, 5)


def test_sb_itv2_wrapper_passes_batch_and_size(monkeypatch):
    from msot_gb300 import solvers as S
    from oracle import solvers as OS
    fake = _host_only(monkeypatch)
    B, Bt, BtB = OS.diff_oper(6)
    u = S.SB_ITV2(np.zeros((4, 6, 6)), 0.05, B, Bt, BtB)
    name, args = fake.calls[-1]
    assert name == "msot_sb_itv2" and args[2:5] == (4, 6, 0.05)
    assert tuple(u.shape) == (4, 6, 6)
    assert tuple(S.SB_ITV(np.zeros((6, 6)), 0.05).shape) == (6, 6)


def test_model_and_solver_wrappers_marshal_the_plan(monkeypatch):
    """MSOTmodel's host logic without a device: the plan descriptor carries
    the grid, T = samples - crop, the interpolation radius of
    MSOTmodel.m:36-38 (dz / (c / fs)), an odd IR and the prefilter taps; the
    operators and rec_nn_with_L2_reg pass batch, iterations and lambda; the
    batch limit is enforced on the host."""
    from msot_gb300 import MSOTmodel, Discretization, Probe, rec_nn_with_L2_reg
    from msot_gb300 import model as Mo
    fake = _host_only(monkeypatch)
    monkeypatch.setattr(Mo, "_stream_ptr", lambda stream=None: None)
    probe = Probe(n_det=32, radius=0.02, angular_coverage=135.0, n_samples=900, eir_length=65)
    disc = Discretization([-0.003, 0.003, -0.002, 0.002], (24, 20))
    m = MSOTmodel(probe, disc, 1500.0, False, True, 10, 1e5, 12e6, 2.5, max_batch=4)
    creates = [a for n, a in fake.calls if n == "msot_plan_create"]
    d = creates[-1][0]._obj
    assert (d.nx, d.nz, d.n_det, d.n_t, d.max_batch) == (24, 20, 32, 890, 4)
    assert abs(d.radius - disc.dz / (1500.0 / probe.fs)) < 1e-12
    assert d.ir_len % 2 == 1 and d.pre_len_x % 2 == 1 and d.pre_len_z % 2 == 1
    assert d.norm == 2.5
    y = m.Funcs.applyForward(np.zeros((3, 24, 20), dtype=np.float32))
    name, args = fake.calls[-1]
    assert name == "msot_forward" and args[3] == 3 and tuple(y.shape) == (3, 32, 890)
    x = m.Funcs.applyTranspose(y)
    assert fake.calls[-1][0] == "msot_transpose" and tuple(x.shape) == (3, 24, 20)
    with pytest.raises(ValueError, match="max_batch"):
        m.Funcs.applyForward(np.zeros((5, 24, 20), dtype=np.float32))
    rec = rec_nn_with_L2_reg(m, np.zeros((2, 32, 890), dtype=np.float32), 7, 1e-2)[0]
    name, args = fake.calls[-1]
    assert name == "msot_rec_nn_with_L2_reg" and args[3:6] == (2, 7, 1e-2)
    assert tuple(rec.shape) == (2, 24, 20)


def test_preprocessor_splits_batches_into_max_cols(monkeypatch):
    """Preprocessor applies a batch of columns in chunks of at most max_cols
    (the scratch it was created for), covering every column once."""
    from msot_gb300 import preprocess as P
    fake = _host_only(monkeypatch)
    monkeypatch.setattr(P, "_stream_ptr", lambda stream=None: None)
    p = P.Preprocessor(100, 10, (2, 20.0, 70.0), 4e7, 1e5, 12e6, max_cols=7)
    name, args = [c for c in fake.calls if c[0] == "msot_prep_create"][-1]
    assert args[:3] == (100, 10, 2) and args[8] == 7
    x = np.zeros((3, 5, 100), dtype=np.float32)  # 15 columns
    out = p(x)
    applies = [a for n, a in fake.calls if n == "msot_prep_apply"]
    assert [a[3] for a in applies] == [7, 7, 1]
    assert tuple(out.shape) == (3, 5, 90)
    with pytest.raises(ValueError, match="samples"):
        p(np.zeros((2, 99), dtype=np.float32))


def test_model_struct_views_run_reference_style_code(monkeypatch):
    """Code written against the reference's model struct runs on the mirror:
    reconstruct_dmas_cf.m:4-12 reads the fov meshgrids, Medium, DAC,
    DataPreprocessing and detector fields; the views carry the mirror's
    values (host logic only, library calls recorded)."""
    from msot_gb300 import MSOTmodel, Discretization, Probe
    from msot_gb300 import analytic as A
    from msot_gb300 import model as Mo
    fake = _host_only(monkeypatch)
    monkeypatch.setattr(Mo, "_stream_ptr", lambda stream=None: None)
    probe = Probe(n_det=32, radius=0.02, angular_coverage=135.0, n_samples=900, delay=3.0,
                  eir_length=65)
    model = MSOTmodel(probe, Discretization([-0.003, 0.003], 24), 1480.0, False, True, 10, 1e5,
                      12e6, 1.0)
    assert model.Probe.detector.numOfTransducers == 32 and model.Probe.eirLength == 65
    assert model.Probe.DAC.frequency == probe.fs and model.Probe.DAC.delayBeforeRecording == 3.0
    assert model.Medium.speedOfSound == 1480.0
    assert model.DataPreprocessing.numCroppedSamplesAtSinogramStart == 10
    assert model.Data.numTimeSamplesPerTransducer == 890
    assert model.Data.circularInterpolationRadiusInSamples == model.radius
    assert model.useSingleSpeedOfSound and not model.includeSir
    sinogram = np.zeros((1, 32, 890), dtype=np.float32)
    A.dmas_cf(sinogram,
              model.Discretization.region.xPositionsFov,
              model.Discretization.region.zPositionsFov,
              model.Medium.speedOfSound,
              model.Probe.DAC.frequency,
              model.DataPreprocessing.numCroppedSamplesAtSinogramStart
              + model.Probe.DAC.delayBeforeRecording,
              model.Probe.detector.angularCoverage,
              model.Probe.detector.radius)
    name, args = fake.calls[-1]
    assert name == "msot_dmas_cf" and args[5] == 24 and args[7] == 24
    assert args[8:13] == (1480.0, probe.fs, 13.0, 135.0, 0.02)
    A.reconstruct_dmas_cf(model, sinogram)
    assert fake.calls[-1][1][8:13] == args[8:13]


def test_storage_and_warm_start_wrappers(monkeypatch):
    """set_storage maps 'fp32' / 'bf16' / 'fp16' (and the booleans) to the
    library's formats 0 / 1 / 2 and rejects anything else; the trajectory
    input of the learned warm start needs 0 < m < input_iters, checked before
    any network is built."""
    from msot_gb300 import MSOTmodel, Discretization, Probe
    from msot_gb300.warmstart import LearnedWarmStart
    fake = _host_only(monkeypatch)
    probe = Probe(n_det=16, radius=0.02, angular_coverage=135.0, n_samples=400, eir_length=33)
    disc = Discretization([-0.002, 0.002], 16)
    m = MSOTmodel(probe, disc, 1500.0, False, True, 0, 1e5, 12e6, 2.5, max_batch=2)
    for arg, code in (("fp32", 0), (False, 0), ("bf16", 1), (True, 1), ("fp16", 2)):
        m.set_storage(arg, 3)
        name, args = fake.calls[-1]
        assert name == "msot_plan_set_storage" and args[1:] == (code, 3)
    with pytest.raises(ValueError):
        m.set_storage("fp8")
    for traj, iters in ((5, 5), (3, 0), (-1, 4)):
        with pytest.raises(ValueError, match="trajectory"):
            LearnedWarmStart(m, 1e-2, input_iters=iters, trajectory=traj)
