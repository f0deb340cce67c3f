"""FP64 restatement of the reference's non-negative solvers.

TEST INFRASTRUCTURE ONLY ("the oracle"): imported by tests/ and bench.py's
CPU-baseline leg, never by the product.

MATLAB's ``lsqr`` and ``cgs`` and the SpaRSA package are closed or absent
(MATLAB built-ins; SpaRSA 2.0 is not vendored, reference .gitignore:8), so they
are restated here from their published algorithms:
  * LSQR  -- Paige & Saunders, ACM TOMS 8(1), 1982, in the form MATLAB's
    lsqr uses (x0 given, residual estimate |s| * normr, return the iterate
    with the smallest residual estimate when maxit is reached);
  * CGS   -- Sonneveld, SIAM J. Sci. Stat. Comput. 10(1), 1989, started from
    x0 = 0 as MATLAB's cgs is called here, with the recursively updated
    residual, returning the iterate with the smallest residual norm when
    maxit is reached;
  * SpaRSA -- Wright, Nowak & Figueiredo, IEEE TSP 57(7), 2009: x+ =
    Psi(x - grad/alpha, tau/alpha) with Barzilai-Borwein alpha, non-monotone,
    no continuation, no debiasing, StopCriterion 1 (relative change of the
    objective below ToleranceA).
Parity against MATLAB for these is therefore unpinned; the GPU solvers are
pinned against these restatements.  The LSQR and CGS restatements are
checked step by step against scipy.sparse.linalg's lsqr and cgs, independent
implementations of the same published algorithms (tests/test_oracle.py);
SpaRSA has no such second implementation here.

Solver sources restated:
  rec_nn_with_L2_reg.m:1-66, nnls_L2_less.m:27-77 (aug operator :79-101),
  incorporate_l2_reg_into_model_functions.m:1-23,
  combine_forward_and_transpose_with_reg.m:1-10,
  rec_nn_with_L1_eye_reg.m:1-49, nnls_L1_eye_matrix_less.m:26-65,
  rec_nn_with_TV_reg.m:1-55, nnls_sparsa_based_reg_matrix_less.m:31-86,
  PsiForTVReg.m, PhiForTVReg.m, SplitBregmanTVdenoising/SB_ITV2.m:20-40,
  DiffOper.m:1-7, ITV.m:5-6.

Vectors are flat float64 numpy arrays.  ``fwd(x)``/``adj(y)`` act on the flat
image (W*P) and sinogram (W*D*T) vectors of one solve.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


# ----------------------------------------------------------------------------
# Krylov solvers
# ----------------------------------------------------------------------------
def lsqr(A, At, b, tol, maxit, x0):
    """LSQR with initial guess x0; returns x after at most ``maxit`` steps."""
    x = np.array(x0, dtype=np.float64, copy=True)
    u = b - A(x)
    beta = np.linalg.norm(u)
    normr = beta
    normb = np.linalg.norm(b)
    if beta != 0:
        u = u / beta
    c, s = 1.0, 0.0
    phibar = beta
    v = At(u)
    alpha = np.linalg.norm(v)
    if alpha != 0:
        v = v / alpha
    if alpha * beta == 0:
        return x
    d = np.zeros_like(x)
    xmin, normrmin = x.copy(), normr
    for _ in range(maxit):
        z = v
        u = A(z) - alpha * u
        beta = np.linalg.norm(u)
        u = u / beta
        thet = -s * alpha
        rhot = c * alpha
        rho = np.sqrt(rhot * rhot + beta * beta)
        c = rhot / rho
        s = -beta / rho
        phi = c * phibar
        phibar = s * phibar
        d = (z - thet * d) / rho
        x = x + phi * d
        normr = abs(s) * normr
        if normr <= tol * normb:
            return x
        if normr < normrmin:
            normrmin, xmin = normr, x.copy()
        vt = At(u)
        v = vt - beta * v
        alpha = np.linalg.norm(v)
        v = v / alpha
    return xmin


def cgs(Aop, b, tol, maxit):
    """CGS from x0 = 0.  Returns the iterate of smallest ||b - A x||."""
    n2b = np.linalg.norm(b)
    x = np.zeros_like(b)
    if n2b == 0:
        return x
    r = b.copy()
    rt = r.copy()
    normr = n2b
    xmin, normrmin = x.copy(), normr
    rho = 1.0
    u = q = p = None
    for i in range(maxit):
        rho1 = rho
        rho = float(np.dot(rt, r))
        if rho == 0 or not np.isfinite(rho):
            break
        if i == 0:
            u = r.copy()
            p = u.copy()
        else:
            beta = rho / rho1
            u = r + beta * q
            p = u + beta * (q + beta * p)
        vh = Aop(p)
        rtvh = float(np.dot(rt, vh))
        if rtvh == 0:
            break
        alpha = rho / rtvh
        q = u - alpha * vh
        uh = u + q
        x = x + alpha * uh
        r = r - alpha * Aop(uh)
        normr = np.linalg.norm(r)
        if normr <= tol * n2b:
            return x
        if normr < normrmin:
            normrmin, xmin = normr, x.copy()
    return xmin


# ----------------------------------------------------------------------------
# L2-regularised NNLS
# ----------------------------------------------------------------------------
def nnls_L2_less(Aaug, Aaug_t, target, n_img, lam, beta, n_iter, n_inner, w0=None):
    """nnls_L2_less.m:27-72 (loop :51-72).  ``Aaug`` is the operator [A; sqrt(lamL2) I]
    (combine_forward_and_transpose_with_reg.m), target = [b; 0].  w0 seeds the
    iterate (the reference starts from zero, nnls_L2_less.m:28-29)."""
    w = np.zeros(n_img) if w0 is None else np.array(w0, dtype=np.float64)
    v = np.zeros(n_img)
    m = target.size
    sl, sb = np.sqrt(lam), np.sqrt(beta)

    def A_nt(x):
        return np.concatenate([sl * Aaug(x), sb * x])

    def A_t(y):
        return sl * Aaug_t(y[:m]) + sb * y[m:]

    for _ in range(n_iter):
        rhs = np.concatenate([sl * target, sb * (w + v)])
        u = lsqr(A_nt, A_t, rhs, 1e-8, n_inner, w)
        w = np.maximum(u - v, 0.0)
        v = v + w - u
    return w


def _second_diff(u, axis):
    """Second differences along one axis with the end values extrapolated
    linearly from the interior (n > 3), copied (n == 3), or zero (n < 3):
    the per-dimension term of MATLAB's del2."""
    u = np.moveaxis(np.asarray(u, dtype=np.float64), axis, 0)
    n = u.shape[0]
    g = np.zeros_like(u)
    if n >= 3:
        g[1:-1] = u[2:] - 2.0 * u[1:-1] + u[:-2]
        if n > 3:
            g[0] = 2.0 * g[1] - g[2]
            g[-1] = 2.0 * g[-2] - g[-3]
        else:
            g[0] = g[1]
            g[-1] = g[1]
    return np.moveaxis(g, 0, axis)


def del2(u):
    """MATLAB del2(U, 1) of a 2-D array: (sum of the second differences of
    both dimensions) / 4."""
    return (_second_diff(u, 0) + _second_diff(u, 1)) / 4.0


def laplacian_per_wavelength(x, nx, nz):
    """laplacian_per_wavelength.m:4-8 on images stacked (W, nx, nz)."""
    x = np.asarray(x, dtype=np.float64).reshape(-1, nx, nz)
    return np.stack([del2(xi) for xi in x]).ravel()


def rec_nn_with_L2_reg(fwd, adj, b, n_img, num_iter, lambdaL2, w0=None, lambdaL2_2=0.0,
                       shape=None):
    """rec_nn_with_L2_reg.m:24-63 with RegL2 = identity (or none if
    lambdaL2 <= 0) and, when lambdaL2_2 > 0 as well, the second term
    RegL2_2 = RegL2T_2 = laplacian_per_wavelength on images of ``shape``
    (nx, nz) (incorporate_l2_reg_into_model_functions.m:8-12,
    combine_forward_and_transpose_with_two_regs.m:8-14; the reference passes
    the Laplacian as its own transpose).  Returns (rec, lCurveErrImg,
    lCurveErrReg[, lCurveErrReg_2])."""
    two = bool(lambdaL2 and lambdaL2 > 0 and lambdaL2_2 and lambdaL2_2 > 0)
    if two:
        sq, sq2 = np.sqrt(lambdaL2), np.sqrt(lambdaL2_2)
        nb = b.size
        lap = lambda x: laplacian_per_wavelength(x, *shape)

        def Aaug(x):
            return np.concatenate([fwd(x), sq * x, sq2 * lap(x)])

        def Aaug_t(y):
            return adj(y[:nb]) + sq * y[nb:nb + n_img] + sq2 * lap(y[nb + n_img:])

        target = np.concatenate([b, np.zeros(2 * n_img)])
        rec = nnls_L2_less(Aaug, Aaug_t, target, n_img, 1.0, 1e-3, num_iter, 2, w0)
        err_img = float(np.linalg.norm(fwd(rec) - b) ** 2)
        return (rec, err_img, float(np.linalg.norm(rec) ** 2),
                float(np.linalg.norm(lap(rec)) ** 2))
    if lambdaL2 and lambdaL2 > 0:
        sq = np.sqrt(lambdaL2)
        nb = b.size

        def Aaug(x):
            return np.concatenate([fwd(x), sq * x])

        def Aaug_t(y):
            return adj(y[:nb]) + sq * y[nb:]

        target = np.concatenate([b, np.zeros(n_img)])
    else:
        Aaug, Aaug_t, target = fwd, adj, b
    rec = nnls_L2_less(Aaug, Aaug_t, target, n_img, 1.0, 1e-3, num_iter, 2, w0)
    err_img = float(np.linalg.norm(fwd(rec) - b) ** 2)
    err_reg = float(np.linalg.norm(rec) ** 2) if (lambdaL2 and lambdaL2 > 0) else 0.0
    return rec, err_img, err_reg


# ----------------------------------------------------------------------------
# L1 (identity) NNLS by split Bregman
# ----------------------------------------------------------------------------
def nnls_L1_eye_matrix_less(fwd, adj, b, u0, eta, lam, n_iter, cg_iter):
    """nnls_L1_eye_matrix_less.m:26-57 (loop :38-54): d = P(u - bp);
    rhs = P(d) + bp + lam A^T b - lam eta; u = cgs(lam A^T A + I, rhs, 1e-8, 2);
    bp += P(d) - u."""
    bp = np.zeros_like(u0)
    u = np.array(u0, dtype=np.float64)

    def op(x):
        return lam * adj(fwd(x)) + x

    for _ in range(n_iter):
        d = np.maximum(u - bp, 0.0)
        rhs = np.maximum(d, 0.0) + bp + lam * adj(b) - lam * eta
        u = cgs(op, rhs, 1e-8, cg_iter)
        bp = bp + np.maximum(d, 0.0) - u
    return u


def rec_nn_with_L1_eye_reg(fwd, adj, b, num_iter, reg):
    """rec_nn_with_L1_eye_reg.m:21-47; the start value is A^T b (:33)."""
    u0 = adj(b)
    rec = nnls_L1_eye_matrix_less(fwd, adj, b, u0, reg, 1.0, num_iter, 2)
    err_img = float(np.linalg.norm(fwd(rec) - b) ** 2)
    return rec, err_img, float(np.abs(rec).sum())


# ----------------------------------------------------------------------------
# TV NNLS: SpaRSA + split-Bregman isotropic TV prox
# ----------------------------------------------------------------------------
def diff_oper(n):
    """DiffOper.m:1-7: forward differences with a zero first row, on an
    n x n image (column-major vectorisation)."""
    Dm = sp.diags([-np.ones(n), np.ones(n)], [0, 1], shape=(n, n + 1)).tolil()
    Dm = Dm[:, 1:]
    Dm[0, 0] = 0
    Dm = sp.csr_matrix(Dm)
    I = sp.identity(n, format="csr")
    B = sp.vstack([sp.kron(I, Dm), sp.kron(Dm, I)]).tocsr()
    return B, B.T.tocsr(), (B.T @ B).tocsr()


def sb_itv2(g, mu, B, Bt, BtB, tol=1e-3, max_outer=200):
    """SB_ITV2.m:20-40 (inner solve: cgs(I + BtB, ., 1e-5, 100))."""
    g = np.asarray(g, dtype=np.float64).ravel(order="F")
    n = g.size
    b = np.zeros(2 * n)
    d = np.zeros(2 * n)
    u = g.copy()
    M = sp.identity(n, format="csr") + BtB
    lam = 1.0
    for _ in range(max_outer):
        up = u
        u = cgs(lambda x: M @ x, g - lam * (Bt @ (b - d)), 1e-5, 100)
        Bub = B @ u + b
        s = np.sqrt(Bub[:n] ** 2 + Bub[n:] ** 2)
        shrink = np.maximum(s - mu / lam, 0.0)
        with np.errstate(invalid="ignore", divide="ignore"):
            f = np.where(s > 0, shrink / s, 0.0)
        d = np.concatenate([f * Bub[:n], f * Bub[n:]])
        b = Bub - d
        nu = np.linalg.norm(u)
        err = np.linalg.norm(up - u) / nu if nu > 0 else 0.0
        if err <= tol:
            break
    return u


def itv(x):
    """ITV.m:5-6 with MATLAB gradient (central differences inside,
    one-sided at the borders)."""
    dz, dx = np.gradient(x)  # x is (nz, nx): axis 0 -> dy(rows), axis 1 -> dx
    return float(np.sum(np.sqrt(dx ** 2 + dz ** 2)))


def sparsa(y, A, At, tau, psi, phi, x0, maxiter, tol=1e-8, alpha_min=1e-30, alpha_max=1e30):
    """SpaRSA (Wright-Nowak-Figueiredo 2009), basic non-monotone BB variant
    with the stopping rule on relative objective change, at most ``maxiter``
    iterations (MaxiterA)."""
    x = np.array(x0, dtype=np.float64)
    resid = y - A(x)
    grad = -At(resid)
    alpha = 1.0
    f = 0.5 * float(resid @ resid) + tau * phi(x)
    for _ in range(maxiter):
        prev_f = f
        xn = psi(x - grad / alpha, tau / alpha)
        dx = xn - x
        Adx = A(dx)
        resid = resid - Adx
        x = xn
        f = 0.5 * float(resid @ resid) + tau * phi(x)
        dd = float(dx @ dx)
        if dd == 0:
            break
        alpha = min(alpha_max, max(alpha_min, float(Adx @ Adx) / dd))
        grad = -At(resid)
        if abs(f - prev_f) / max(abs(prev_f), 1e-300) <= tol:
            break
    return x


def rec_nn_with_TV_reg(fwd, adj, b, nx, nz, n_wl, num_iter, reg, sparsa_iter=2):
    """rec_nn_with_TV_reg.m:20-54 + nnls_sparsa_based_reg_matrix_less.m:31-85
    (SpaRSA's MaxiterA = sparsa_iter, 2 in the reference, :64)."""
    if nx != nz:
        raise ValueError("This TV implementation works only with square images!")
    B, Bt, BtB = diff_oper(nx)
    npix = nx * nz

    def Psi(x, t):
        out = np.empty_like(x)
        for k in range(n_wl):
            img = x[k * npix:(k + 1) * npix]
            out[k * npix:(k + 1) * npix] = sb_itv2(img.reshape(nz, nx, order="F"), t, B, Bt, BtB)
        return out

    def Phi(x):
        return sum(itv(x[k * npix:(k + 1) * npix].reshape(nz, nx, order="F")) for k in range(n_wl))

    lam, beta = 1.0, 1e-3
    w = np.zeros(npix * n_wl)
    v = np.zeros_like(w)
    m = b.size
    sl, sb = np.sqrt(lam), np.sqrt(beta)

    def Aaug(x):
        return np.concatenate([sl * fwd(x), sb * x])

    def Aaug_t(y):
        return sl * adj(y[:m]) + sb * y[m:]

    for _ in range(num_iter):
        rhs = np.concatenate([sl * b, sb * (w + v)])
        u = sparsa(rhs, Aaug, Aaug_t, reg, Psi, Phi, w, sparsa_iter)
        w = np.maximum(u - v, 0.0)
        v = v + w - u
    err_img = float(np.linalg.norm(fwd(w) - b) ** 2)
    return w, err_img, Phi(w)


def relative_error(x, ref):
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = np.asarray(ref, dtype=np.float64).ravel()
    return float(np.linalg.norm(x - ref) / max(np.linalg.norm(ref), 1e-300))
