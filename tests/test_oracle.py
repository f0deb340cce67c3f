"""CPU tests of the oracle: the C restatement against the golden vectors made
by the reference's own MEX code, and the FP64 model/solver restatements."""
import numpy as np
import pytest

from oracle import model as M
from oracle import native
from oracle import solvers as S


@pytest.fixture(scope="module")
def port():
    return native.port()


@pytest.mark.parametrize("W", [1, 5])
def test_port_das_matches_reference_bitwise(port, golden, W):
    tau, r, T = golden["tau"], float(golden["radius"]), int(golden["T"])
    y = port.forward_das(golden[f"das_img_w{W}"], tau, T, r)
    assert np.array_equal(y, golden[f"das_fwd_w{W}"])
    x = port.transpose_das(golden[f"das_sig_w{W}"], tau, r)
    assert np.array_equal(x, golden[f"das_adj_w{W}"])


@pytest.mark.parametrize("W", [1, 3])
def test_port_sir_matches_reference_bitwise(port, golden, W):
    g = golden
    r, T = float(g["radius"]), int(g["sir_T"])
    y = port.forward_sir(g[f"sir_img_w{W}"], g["sir_idx"], g["sir_tau"], g["sir"], T,
                         g["sir_se"], r)
    assert np.array_equal(y, g[f"sir_fwd_w{W}"])
    x = port.transpose_sir(g[f"sir_sig_w{W}"], g["sir_idx"], g["sir_tau"], g["sir"], g["sir_se"], r)
    assert np.array_equal(x, g[f"sir_adj_w{W}"])


@pytest.mark.skipif(not native.ref_available(), reason="reference MEX not compiled on this host")
def test_reference_library_reproduces_golden(golden):
    ref = native.ref()
    tau, r, T = golden["tau"], float(golden["radius"]), int(golden["T"])
    assert np.array_equal(ref.forward_das(golden["das_img_w5"], tau, T, r), golden["das_fwd_w5"])


@pytest.mark.skipif(not native.ref_available(), reason="reference MEX not compiled on this host")
@pytest.mark.parametrize("seed", range(12))
def test_port_matches_reference_on_random_geometries(port, seed):
    """Beyond the committed golden vectors: the C restatement against the
    reference MEX code itself on seeded random arcs, grids, interpolation
    radii (1 to 8 samples), batch sizes and thread counts, bit for bit, for
    all four operators."""
    from tests.golden.make_golden import small_geometry
    ref = native.ref()
    rng = np.random.default_rng(1000 + seed)
    nx, nz = int(rng.integers(3, 30)), int(rng.integers(3, 30))
    n_det = int(rng.integers(2, 40))
    pitch = float(rng.uniform(0.04e-3, 0.3e-3))
    tau, r = small_geometry(nx, nz, n_det, R=float(rng.uniform(0.006, 0.03)),
                            cov=float(rng.uniform(60, 270)), pitch=pitch)
    D, P = tau.shape
    W = int(rng.choice([1, 2, 4, 7]))
    T = int(np.ceil(tau.max() + r)) + int(rng.integers(2, 30))
    threads = int(rng.choice([1, 3, 8]))
    for lib in (port, ref):
        lib.set_threads(threads)
    img = rng.random((P, W))
    sig = rng.standard_normal((D, T, W))
    assert np.array_equal(port.forward_das(img, tau, T, r), ref.forward_das(img, tau, T, r))
    assert np.array_equal(port.transpose_das(sig, tau, r), ref.transpose_das(sig, tau, r))
    S, NS = int(rng.integers(5, 60)), int(rng.integers(1, 20))
    sir = rng.standard_normal((NS, S))
    se = np.zeros((NS, 2), dtype=np.int32)
    for k in range(NS):
        a = int(rng.integers(1, S + 1))
        se[k] = (a, int(rng.integers(a, S + 1)))
    idx = rng.integers(1, NS + 1, size=(D, P)).astype(np.int32)
    tau_s = tau - (tau.min() - 3.0)
    Ts = int(np.ceil(tau_s.max())) + int(rng.integers(1, 20))
    sig_s = rng.standard_normal((D, Ts, W))
    assert np.array_equal(port.forward_sir(img, idx, tau_s, sir, Ts, se, r),
                          ref.forward_sir(img, idx, tau_s, sir, Ts, se, r))
    assert np.array_equal(port.transpose_sir(sig_s, idx, tau_s, sir, se, r),
                          ref.transpose_sir(sig_s, idx, tau_s, sir, se, r))


def test_port_rejects_out_of_range_taps(port, golden):
    tau, r, T = golden["tau"], float(golden["radius"]), int(golden["T"])
    bad = tau.copy()
    bad[3, 7] = T - 1.0  # taps past the end of the sinogram
    with pytest.raises(ValueError):
        port.forward_das(golden["das_img_w1"], bad, T, r)
    bad[3, 7] = np.nan
    with pytest.raises(ValueError):
        port.transpose_das(golden["das_sig_w1"], bad, r)


def test_port_adjoint_config1_geometry(port):
    probe, grid = M.config1_probe(eir=False), M.config_grid(128)
    tau = M.travel_time_indices(probe, grid, 1500.0)
    r = M.interpolation_radius(grid, probe, 1500.0)
    rng = np.random.default_rng(0)
    x = rng.random((grid.n_pix, 2))
    y = rng.standard_normal((probe.n_det, probe.n_samples, 2))
    Ax = port.forward_das(x, tau, probe.n_samples, r)
    Aty = port.transpose_das(y, tau, r)
    err = abs(np.vdot(Ax, y) - np.vdot(x, Aty)) / (np.linalg.norm(Ax) * np.linalg.norm(y))
    assert err < 1e-13


@pytest.mark.parametrize("n", [128, 101, 40])
def test_separable_prefilter_equals_2d_fft_prefilter(n):
    grid = M.Grid(n, n, (-0.0127, 0.0127, -0.0127, 0.0127))
    pre = M.prefilter(grid)
    rng = np.random.default_rng(n)
    img = rng.random((1, n, n))
    ref = M.project(img, pre)[0]
    dx, dz = grid.spacing()
    hx = M.separable_prefilter_taps(n, dx, grid.sigma())
    hz = M.separable_prefilter_taps(n, dz, grid.sigma())
    Kx, Kz = hx.size // 2, hz.size // 2
    m = img[0]  # (nx, nz)
    out = np.zeros_like(m)
    for k in range(-Kz, Kz + 1):
        out += hz[k + Kz] * np.roll(m, k, axis=1)
    out2 = np.zeros_like(m)
    for k in range(-Kx, Kx + 1):
        out2 += hx[k + Kx] * np.roll(out, k, axis=0)
    assert np.max(np.abs(out2 - ref)) < 1e-11 * np.max(np.abs(ref))


def test_oracle_model_is_adjoint():
    probe = M.ArcProbe(n_det=32, radius=0.02, coverage_deg=135, n_samples=800,
                       eir=M.gauss_pulse_eir(n_taps=64), eir_length=65)
    grid = M.Grid(24, 20, (-0.003, 0.003, -0.0025, 0.0025))
    m = M.Model(probe, grid, c=1500.0)
    rng = np.random.default_rng(1)
    x = rng.random((2, 24, 20))
    y = rng.standard_normal((2, 32, 800))
    Ax, Aty = m.forward(x), m.transpose(y)
    err = abs(np.vdot(Ax, y) - np.vdot(x, Aty)) / (np.linalg.norm(Ax) * np.linalg.norm(y))
    assert err < 1e-12


def test_convolve_ir_matches_direct_fir():
    rng = np.random.default_rng(2)
    ir = rng.standard_normal(9)
    s = rng.standard_normal((3, 40))
    y = M.convolve_ir(s, ir)
    h = ir.size // 2
    direct = np.zeros_like(s)
    for t in range(40):
        for k in range(ir.size):
            u = t + h - k
            if 0 <= u < 40:
                direct[:, t] += ir[k] * s[:, u]
    assert np.allclose(y, direct, rtol=0, atol=1e-12)


@pytest.mark.parametrize("fmin,fmax", [(1e5, 12e6), (0.0, 12e6), (5e5, 0.0)])
def test_fft_zero_phase_filter_equals_forward_backward_iir(fmin, fmax):
    """filter_butter_zero_phase.m:26-48 (use_fft = true) multiplies the
    spectrum by |H|^2 on the whole circle.  For a pulse whose filtered tails
    stay inside the record that equals running the Butterworth sections
    forward and then backward in the time domain (after the mean removal the
    reference applies with a high-pass)."""
    import scipy.signal as sps
    fs, n = 4e7, 8192
    t = np.arange(n)
    x = np.exp(-0.5 * ((t - n / 2) / 6.0) ** 2) * np.sin(2 * np.pi * 5e6 * t / fs)
    y = M.filter_butter_zero_phase(x[:, None], fs, fmin, fmax)[:, 0]
    xs = x - x.mean() if fmin > 0 else x
    secs = []
    if fmax > 0:
        secs.append(sps.butter(8, fmax * 2 / fs, "low", output="sos"))
    if fmin > 0:
        secs.append(sps.butter(2, fmin * 2 / fs, "high", output="sos"))
    sos = np.vstack(secs)
    ff = sps.sosfilt(sos, sps.sosfilt(sos, xs)[::-1])[::-1]
    assert np.abs(y - ff).max() <= 1e-12 * np.abs(y).max()


def test_sigma_max_estimate_matches_svd():
    """The power iteration standing in for svds(A, 1) (MSOTmodel.m:277-278)
    against the largest singular value of a dense matrix with a clear gap."""
    rng = np.random.default_rng(9)
    U, _ = np.linalg.qr(rng.standard_normal((50, 20)))
    V, _ = np.linalg.qr(rng.standard_normal((20, 20)))
    s = np.linspace(0.1, 1.0, 20)
    s[-1] = 2.0
    A = (U * s) @ V.T
    est = M.estimate_sigma_max(lambda v: A @ v, lambda u: A.T @ u, (20,), iters=60)
    assert abs(est - np.linalg.svd(A, compute_uv=False)[0]) <= 1e-12 * 2.0


def test_lsqr_restatement_matches_scipy():
    from scipy.sparse.linalg import lsqr as sp_lsqr
    rng = np.random.default_rng(3)
    A = rng.standard_normal((40, 15))
    b = rng.standard_normal(40)
    x0 = rng.standard_normal(15)
    for k in range(1, 13):
        ours = S.lsqr(lambda v: A @ v, lambda u: A.T @ u, b, 1e-12, k, x0)
        ref = sp_lsqr(A, b, atol=0, btol=0, iter_lim=k, x0=x0)[0]
        assert np.allclose(ours, ref, rtol=1e-10, atol=1e-12), k


def test_cgs_restatement_solves_spd_system():
    rng = np.random.default_rng(4)
    B = rng.standard_normal((20, 20))
    A = B @ B.T + 20 * np.eye(20)
    b = rng.standard_normal(20)
    x = S.cgs(lambda v: A @ v, b, 1e-12, 200)
    assert np.linalg.norm(A @ x - b) < 1e-9 * np.linalg.norm(b)
    # not converged after 2 steps: returns the iterate of smallest residual
    x2 = S.cgs(lambda v: A @ v, b, 1e-12, 2)
    assert np.linalg.norm(A @ x2 - b) <= np.linalg.norm(b)


def test_cgs_iterates_match_scipy():
    """Each CGS step against scipy's independent implementation of the same
    algorithm (Templates form, x0 = 0) on a non-symmetric system whose
    residual is not monotone: after k steps the restatement returns scipy's
    iterate of smallest residual among its first k."""
    from scipy.sparse.linalg import cgs as sp_cgs
    rng = np.random.default_rng(7)
    n = 30
    A = 4 * np.eye(n) + 0.5 * rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    its = []
    sp_cgs(A, b, x0=np.zeros(n), rtol=1e-14, atol=0, maxiter=12,
           callback=lambda x: its.append(x.copy()))
    assert len(its) == 12
    res = [np.linalg.norm(b - A @ x) for x in its]
    assert any(res[k + 1] > res[k] for k in range(11))  # non-monotone case
    for k in range(1, 13):
        ours = S.cgs(lambda v: A @ v, b, 1e-14, k)
        j = int(np.argmin(res[:k]))
        assert np.abs(ours - its[j]).max() < 1e-11


def test_l2_nnls_oracle_is_nonnegative_and_fits():
    rng = np.random.default_rng(5)
    A = rng.random((60, 30))
    xt = np.maximum(rng.standard_normal(30), 0)
    b = A @ xt
    rec, e_img, e_reg = S.rec_nn_with_L2_reg(lambda v: A @ v, lambda u: A.T @ u, b, 30, 200, 1e-4)
    assert rec.min() >= 0
    assert e_img < 0.1 * np.linalg.norm(b) ** 2


def test_l2_nnls_oracle_converges_to_scipy_nnls():
    """The splitting of nnls_L2_less.m:51-72 (beta = 1e-3, two LSQR steps
    per iteration) approaches the minimiser of |A x - b|^2 + lambda |x|^2,
    x >= 0, that scipy's active-set NNLS (Lawson & Hanson) finds on the
    augmented system; A has unit norm as the normalised model does."""
    from scipy.optimize import nnls
    rng = np.random.default_rng(0)
    A = rng.standard_normal((60, 30))
    A /= np.linalg.norm(A, 2)
    lam = 1e-2
    xt = np.maximum(rng.standard_normal(30), 0)
    b = A @ xt + 0.05 * rng.standard_normal(60)
    xa, _ = nnls(np.vstack([A, np.sqrt(lam) * np.eye(30)]), np.concatenate([b, np.zeros(30)]))
    assert (xa == 0).sum() >= 3  # active constraints present
    errs = []
    for it in (50, 200, 1000):
        rec, _, _ = S.rec_nn_with_L2_reg(lambda v: A @ v, lambda u: A.T @ u, b, 30, it, lam)
        errs.append(np.linalg.norm(rec - xa) / np.linalg.norm(xa))
    assert errs[0] > errs[1] > errs[2] and errs[2] < 2e-4


def test_l1_nnls_oracle_minimises_nonnegative_lasso():
    """nnls_L1_eye_matrix_less.m:38-54 is split Bregman for
    min 1/2 |A u - b|^2 + eta sum(u), u >= 0.  With an accurate inner solve
    (30 CGS steps) it reaches the minimiser that projected FISTA finds.  The
    reference's own setting (2 CGS steps from zero per iteration) stalls about
    1 % away from it on this problem: the inexact inner solve moves the fixed
    point, a property of the reference's algorithm that the GPU solver
    reproduces."""
    rng = np.random.default_rng(0)
    A = rng.standard_normal((60, 30))
    A /= np.linalg.norm(A, 2)
    xt = np.maximum(rng.standard_normal(30), 0)
    b = A @ xt + 0.05 * rng.standard_normal(60)
    eta = 1e-2
    x, z, t = np.zeros(30), np.zeros(30), 1.0
    for _ in range(20000):  # step 1/L with L = |A|^2 = 1
        xn = np.maximum(z - (A.T @ (A @ z - b) + eta), 0.0)
        tn = (1 + np.sqrt(1 + 4 * t * t)) / 2
        z, x, t = xn + (t - 1) / tn * (xn - x), xn, tn
    assert (x == 0).sum() >= 3
    fwd, adj = (lambda v: A @ v), (lambda u: A.T @ u)
    rec = S.nnls_L1_eye_matrix_less(fwd, adj, b, A.T @ b, eta, 1.0, 1000, 30)
    assert np.linalg.norm(rec - x) <= 1e-6 * np.linalg.norm(x)
    rec2 = S.rec_nn_with_L1_eye_reg(fwd, adj, b, 1000, eta)[0]
    assert 1e-3 < np.linalg.norm(rec2 - x) / np.linalg.norm(x) < 5e-2


def test_sb_itv2_reduces_tv():
    rng = np.random.default_rng(6)
    n = 12
    B, Bt, BtB = S.diff_oper(n)
    g = np.zeros((n, n))
    g[3:8, 4:9] = 1.0
    g += 0.1 * rng.standard_normal((n, n))
    u = S.sb_itv2(g, 0.05, B, Bt, BtB).reshape(n, n, order="F")
    assert S.itv(u) < S.itv(g)


def test_sb_itv2_minimises_isotropic_tv_objective():
    """Split Bregman with lambda = 1 (SB_ITV2.m:20-40) minimises
    E(u) = mu * sum_i |(B u)_i|_2 + 1/2 |u - g|^2 over the DiffOper
    gradient B.  An independent solver of the same objective (the
    Chambolle-Pock primal-dual iteration, dual constraint |p_i| <= mu) gives
    the reference minimum."""
    rng = np.random.default_rng(6)
    n = 12
    N = n * n
    B, Bt, BtB = S.diff_oper(n)
    g = np.zeros((n, n))
    g[3:8, 4:9] = 1.0
    g += 0.1 * rng.standard_normal((n, n))
    gf = g.ravel(order="F")
    mu = 0.05

    def energy(u):
        Bu = B @ u
        return mu * np.sum(np.hypot(Bu[:N], Bu[N:])) + 0.5 * np.sum((u - gf) ** 2)

    u, ub, p = gf.copy(), gf.copy(), np.zeros(2 * N)
    tau = sig = 0.34  # tau * sigma * |B|^2 < 1 with |B|^2 <= 8
    for _ in range(20000):
        p = p + sig * (B @ ub)
        f = np.maximum(1.0, np.hypot(p[:N], p[N:]) / mu)
        p = p / np.concatenate([f, f])
        un = (u - tau * (Bt @ p) + tau * gf) / (1 + tau)
        ub, u = 2 * un - u, un
    e_ref = energy(u)
    us = S.sb_itv2(g, mu, B, Bt, BtB, tol=1e-6, max_outer=2000)
    assert abs(energy(us) - e_ref) <= 1e-5 * e_ref
    assert np.linalg.norm(us - u) <= 1e-4 * np.linalg.norm(u)
    # the reference's own stopping tolerance (1e-3) stays within 1e-3 of it
    assert energy(S.sb_itv2(g, mu, B, Bt, BtB)) <= (1 + 1e-3) * e_ref


def test_sparsa_reaches_the_lasso_minimiser():
    """The SpaRSA restatement (Barzilai-Borwein prox-gradient) with the
    soft-threshold prox converges to the minimiser of
    1/2 |y - A x|^2 + tau |x|_1 that an independent method (FISTA, Beck &
    Teboulle 2009) finds."""
    rng = np.random.default_rng(8)
    m, n = 60, 40
    A = rng.standard_normal((m, n)) / np.sqrt(m)
    xt = np.zeros(n)
    xt[rng.choice(n, 6, replace=False)] = rng.standard_normal(6)
    y = A @ xt + 0.01 * rng.standard_normal(m)
    tau = 0.02

    def soft(v, t):
        return np.sign(v) * np.maximum(np.abs(v) - t, 0.0)

    def objective(x):
        return 0.5 * np.sum((y - A @ x) ** 2) + tau * np.abs(x).sum()

    L = np.linalg.norm(A, 2) ** 2
    x, z, t = np.zeros(n), np.zeros(n), 1.0
    for _ in range(20000):
        xn = soft(z - (A.T @ (A @ z - y)) / L, tau / L)
        tn = (1 + np.sqrt(1 + 4 * t * t)) / 2
        z, x, t = xn + (t - 1) / tn * (xn - x), xn, tn
    xs = S.sparsa(y, lambda v: A @ v, lambda u: A.T @ u, tau, soft, lambda v: np.abs(v).sum(),
                  np.zeros(n), 200, tol=1e-14)
    assert abs(objective(xs) - objective(x)) <= 1e-12 * objective(x)
    assert np.linalg.norm(xs - x) <= 1e-7 * np.linalg.norm(x)


def test_bp_kernel_is_antisymmetric_and_dmas_identity():
    from oracle import backprojection as B
    t = np.arange(1, 41) / 4e7
    K = B.bp_kernel(t)
    assert np.allclose(K, -K.T, atol=1e-12 * np.abs(K).max())
    rng = np.random.default_rng(9)
    sig = rng.standard_normal((1, 16, 400))
    x = np.linspace(-0.002, 0.002, 6)
    z = np.linspace(-0.002, 0.002, 5)
    dmcf, dm, cf, das = B.dmas_cf(sig, x, z, 1500.0, 4e7, 0.0, 135.0, 0.008)
    assert np.allclose(dmcf, dm * cf)
    assert (cf >= 0).all() and (cf <= 1.0 + 1e-9).all()


def test_analytic_reconstructors_locate_a_point_source():
    """Sinograms of one point source, made from the arc geometry alone
    (detector p at angle -(off + step p), pulse at |x_p - x_s| / c):
    DAS, DMAS and DMAS-CF peak on the source pixel; backproject_waveeq of the
    N-shaped pressure signal peaks on the source mirrored in x (its final
    fliplr, backproject_waveeq.m:49)."""
    from oracle import backprojection as BP
    n, R, c, fs, D, cov, T = 32, 0.04, 1500.0, 4e7, 64, 135.0, 1700
    x = np.linspace(-0.0127, 0.0127, n)
    z = x.copy()
    ang = BP.transducer_angles(D, cov)
    xd, zd = R * np.cos(ang), R * np.sin(ang)
    i0, j0 = 22, 9
    t = np.arange(1, T + 1) / fs
    u = (t[None, :] - np.hypot(xd - x[i0], zd - z[j0])[:, None] / c) * fs / 2.0
    pulse = np.exp(-0.5 * u ** 2)[None]
    for img in BP.dmas_cf(pulse, x, z, c, fs, 0, cov, R)[:4]:
        assert np.unravel_index(np.argmax(img[0]), img[0].shape) == (i0, j0)
    K = BP.bp_kernel(t)
    bw = BP.backproject_waveeq(-u * pulse, x, z, c, fs, 0, cov, R, np.ones((1, 1)), K)[0]
    assert np.unravel_index(np.argmax(bw), bw.shape) == (n - 1 - i0, j0)
    assert bw.max() > 4 * abs(bw.min())


def test_model_and_analytic_geometries_agree():
    """The model-based forward of one pixel (MSOTmodel restatement, N-shaped
    pixel response) seen by the analytic reconstructors and by the model's
    own transpose: A^T A e_s peaks on the source; backproject_waveeq peaks
    on the x-mirrored source; DAS / DMAS / DMAS-CF land within one pixel of
    it (the N-shape crosses zero at the arrival time)."""
    from oracle import backprojection as BP
    n = 32
    probe = M.ArcProbe(n_det=64, n_samples=1700)
    grid = M.Grid(n, n)
    om = M.Model(probe, grid, c=1500.0)
    x, z = grid.vectors()
    i0, j0 = 22, 9
    img = np.zeros((1, n, n))
    img[0, i0, j0] = 1.0
    sino = om.forward(img)
    back = om.transpose(sino)[0]
    assert np.unravel_index(np.argmax(back), back.shape) == (i0, j0)
    geo = (1500.0, probe.fs, 0, probe.coverage_deg, probe.radius)
    K = BP.bp_kernel(np.arange(1, probe.n_samples + 1) / probe.fs)
    bw = BP.backproject_waveeq(sino, x, z, *geo, np.ones((1, 1)), K)[0]
    assert np.unravel_index(np.argmax(bw), bw.shape) == (n - 1 - i0, j0)
    for im in BP.dmas_cf(sino, x, z, *geo):
        i, j = np.unravel_index(np.argmax(np.abs(im[0])), im[0].shape)
        assert abs(i - i0) <= 1 and abs(j - j0) <= 1


def test_spmr_antialias_response_matches_butterworth_design():
    """calculate_polarSPMR.m:50-54,73: |freqz|^2 of butter(8, fs_dac / f_field,
    'low') on the whole circle; the restatement writes it in closed form
    (bilinear Butterworth), checked here against scipy's design."""
    import scipy.signal as sps
    from oracle import sir as O
    fs, n = 4e7, 1 << 16
    f = np.arange(n) / n
    with np.errstate(divide="ignore", over="ignore"):
        ratio = np.tan(np.pi * f) / np.tan(np.pi * (fs / 2.0) / O.FSF)
        h2 = 1.0 / (1.0 + ratio ** 16)
    h2[n // 2] = 0.0
    _, h = sps.sosfreqz(sps.butter(8, fs / O.FSF, "low", output="sos"), worN=n, whole=True)
    assert np.abs(np.abs(h) ** 2 - h2).max() < 1e-10
    # and nshape_filtered applies exactly this response to the N-shape
    sigma, c = 1e-5, 1500.0  # decays within the default 200 field samples
    g, M = O.nshape_filtered(sigma, c, fs)
    m = np.arange(-M, M + 2)
    circ = np.zeros(O.NF)
    circ[m % O.NF] = g
    j = np.arange(-200, 201)
    t = j / O.FSF
    q = np.zeros(O.NF)
    q[j % O.NF] = np.exp(-(c * t) ** 2 / (2 * sigma ** 2)) * (-t)
    ref = np.real(np.fft.ifft(np.fft.fft(q) * h2))
    assert np.abs(circ - ref).max() <= 1e-9 * np.abs(ref).max()


def test_spmr_oracle_tables_are_consistent():
    # SPMR generator restatement (parity with the reference's Field II tables
    # is unpinned): every column peaks near its travel time, start <= end
    # inside the window, and every (pixel, detector) maps into the table.
    from oracle import sir as Q
    g = M.config_grid(24)
    x, z = g.vectors()
    tab, se, idx, info = Q.spmr_tables(24, 0.040, 135.0, x, z, 1500.0, 4e7, 0.5e-3, 0.25e-3,
                                       10e-3, 0.040, 4, 4, half_window=60)
    NS, S = tab.shape
    assert NS == info["n_dist"] * info["n_angle"]
    assert np.all(se[:, 0] >= 1) and np.all(se[:, 0] <= se[:, 1]) and np.all(se[:, 1] <= S)
    h = S // 2
    assert np.all(np.abs(np.abs(tab).argmax(axis=1) - h) <= h)
    assert idx.min() >= 1 and idx.max() <= NS


def test_dual_sos_travel_times_against_bounded_brent_and_snell():
    # the oracle's vectorised golden-section Fermat search against scipy's
    # bounded Brent minimiser on sampled pixel-detector pairs, and Snell's law
    # at the intersection of a flat membrane
    from scipy.optimize import minimize_scalar
    probe = M.ArcProbe(n_det=16, radius=0.040, coverage_deg=135.0, n_samples=2030)
    grid = M.Grid(12, 12, (-0.006, 0.006, -0.006, 0.006))
    cb, ca, z0 = 1560.0, 1480.0, -0.012
    tau, xm = M.travel_time_indices_dual(probe, grid, cb, ca, [z0])
    xd, zd = probe.positions()
    X, Z = grid.pixel_xz()
    rng = np.random.default_rng(0)
    for _ in range(40):
        d, p = int(rng.integers(16)), int(rng.integers(X.size))
        f = lambda x: np.hypot(X[p] - x, Z[p] - z0) / cb + np.hypot(x - xd[d], z0 - zd[d]) / ca
        r = minimize_scalar(f, bounds=(-0.04, 0.04), method="bounded",
                            options={"xatol": 1e-14})
        assert abs(tau[d, p] - r.fun * probe.fs) <= 1e-6
        # Snell: sin(theta_below) / c_below = sin(theta_above) / c_above
        s1 = (xm[d, p] - X[p]) / np.hypot(xm[d, p] - X[p], z0 - Z[p])
        s2 = (xd[d] - xm[d, p]) / np.hypot(xd[d] - xm[d, p], zd[d] - z0)
        assert abs(s1 / cb - s2 / ca) <= 1e-9


def test_del2_restatement_properties():
    # MATLAB del2(U, 1) of x^2 + y^2 is 1 everywhere (the end values come from
    # linear extrapolation, exact for quadratics), of a linear field 0; lines
    # of 3 copy the centre, shorter lines give 0
    from oracle import solvers as S
    X, Y = np.meshgrid(np.arange(7.0), np.arange(5.0), indexing="ij")
    assert np.allclose(S.del2(X ** 2 + Y ** 2), 1.0)
    assert np.allclose(S.del2(3.0 * X - 2.0 * Y + 1.0), 0.0)
    u = np.random.default_rng(1).standard_normal((3, 2))
    d = S.del2(u)
    col = (u[2] - 2 * u[1] + u[0]) / 4.0  # the n = 3 axis, copied to its ends; n = 2 axis: 0
    assert np.allclose(d, np.broadcast_to(col, (3, 2)))


def test_virtual_sources_restatement():
    # the virtual source lies at distance t c_coupling from its detector, and
    # is the pixel itself when the path does not cross the membrane
    probe = M.ArcProbe(n_det=12, radius=0.040, coverage_deg=135.0, n_samples=2030)
    grid = M.Grid(10, 10, (-0.006, 0.006, -0.006, 0.006))
    mem = (-0.004, 0.1)  # cuts the grid: some pixels lie on the detector side
    tau, xm = M.travel_time_indices_dual(probe, grid, 1560.0, 1480.0, mem)
    vx, vz = M.virtual_sources(probe, grid, 1560.0, 1480.0, mem)
    xd, zd = probe.positions()
    d = np.hypot(vx - xd[:, None], vz - zd[:, None])
    assert np.allclose(d, tau / probe.fs * 1480.0, rtol=0, atol=1e-12)
    X, Z = grid.pixel_xz()
    direct = np.isnan(xm)
    assert direct.any() and (~direct).any()
    assert np.array_equal(vx[direct], np.broadcast_to(X, vx.shape)[direct])


def test_spmr_with_pixels_as_virtual_sources_is_unchanged():
    from oracle import sir as Q
    x = np.linspace(-0.002, 0.002, 8)
    z = np.linspace(-0.002, 0.002, 8)
    args = (8, 0.040, 135.0, x, z, 1500.0, 4e7, 0.00029, 0.25e-3, 10e-3, 0.0, 2, 2)
    a = Q.spmr_tables(*args, half_window=60)
    X, Z = np.meshgrid(x, z, indexing="ij")
    virt = (np.broadcast_to(X.ravel(), (8, 64)), np.broadcast_to(Z.ravel(), (8, 64)))
    b = Q.spmr_tables(*args, half_window=60, virtual=virt)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
