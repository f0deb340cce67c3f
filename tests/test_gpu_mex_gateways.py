"""The MATLAB-level drop-in on the GPU, driven through the MEX API (the
project's stand-in header): a GPU model created by
msot_model_mex('create', model, ...) from the members of a reference model
object (travel-time table, IRHat, prefilter -- built here by the FP64
oracle model the same way MSOTmodel.m:31-47 and Discretization.m:47-51
build them), its applyForward / applyTranspose, and the solver gateways
with the reference's signatures, each against the FP64 oracle.
Bars: operators 1e-5, solves 1e-3 (relative)."""
import ctypes as C

import numpy as np
import pytest

import mexdrv
from oracle import model as M
from oracle import solvers as S
from pairs import rel

pytestmark = pytest.mark.gpu

N, D, T = 64, 128, 1200


@pytest.fixture(scope="module")
def env(cuda, tmp_path_factory):
    drv = mexdrv.build(str(tmp_path_factory.mktemp("mexdrv")))
    eir = M.gauss_pulse_eir()
    op = M.ArcProbe(n_det=D, radius=0.02, coverage_deg=135.0, n_samples=T, eir=eir,
                    eir_length=eir.size)
    om = M.Model(op, M.Grid(N, N, (-0.0063, 0.0063, -0.0063, 0.0063)))
    om.normalize(60)
    fields = dict(travel=np.ascontiguousarray(om.travel, dtype=np.float64),
                  ir_hat=np.ascontiguousarray(np.fft.fft(om.ir, T + om.ir.size - 1)),
                  pre=np.ascontiguousarray(om.pre.T))  # MATLAB nz x nx, column-major
    yield drv, om, fields


def _create(drv, om, fields, norm, max_batch=2):
    h = C.c_uint64()
    msg = C.create_string_buffer(512)
    rc = drv.drv_create(N, N, D, T, om.radius, mexdrv.dptr(fields["travel"]),
                        mexdrv.dptr(fields["ir_hat"].view(np.float64)), fields["ir_hat"].size,
                        om.ir.size, mexdrv.dptr(fields["pre"].view(np.float64)), norm, max_batch,
                        C.byref(h), msg, 512)
    assert rc == 0, msg.value
    return h.value


def _data(om, W, seed):
    rng = np.random.default_rng(seed)
    return np.stack([M.noisy_sinogram(om, M.phantom(om.grid, rng), rng) for _ in range(W)])


@pytest.fixture(scope="module")
def model(env):
    drv, om, fields = env
    h = _create(drv, om, fields, om.norm)
    yield h
    msg = C.create_string_buffer(512)
    assert drv.drv_model(b"destroy", h, None, 0, None, 0, msg, 512) == 0, msg.value


def test_apply_forward_and_transpose_match_the_oracle(env, model):
    drv, om, _ = env
    msg = C.create_string_buffer(512)
    rng = np.random.default_rng(1)
    x = rng.random((2, N, N))  # Nz x Nx x W in MATLAB's memory order
    y = np.empty(2 * D * T)
    assert drv.drv_model(b"applyForward", model, mexdrv.dptr(x), x.size, mexdrv.dptr(y),
                         y.size, msg, 512) == 0, msg.value
    assert rel(y, om.forward(x)) <= 1e-5
    s = rng.standard_normal((2, D, T))
    xa = np.empty(2 * N * N)
    assert drv.drv_model(b"applyTranspose", model, mexdrv.dptr(s), s.size, mexdrv.dptr(xa),
                         xa.size, msg, 512) == 0, msg.value
    assert rel(xa, om.transpose(s)) <= 1e-5


def test_normalisation_estimated_when_not_given(env):
    # [] for the factor: sigma_max by the library's power iteration (100
    # steps), as MSOTmodel(..., None) of the Python mirror estimates it on
    # the same geometry
    from pairs import make_pair
    drv, om, fields = env
    h = _create(drv, om, fields, 0.0, 1)
    out = np.zeros(1)
    msg = C.create_string_buffer(512)
    assert drv.drv_model(b"normalizationFactor", h, None, 0, mexdrv.dptr(out), 1, msg, 512) == 0
    assert drv.drv_model(b"destroy", h, None, 0, None, 0, msg, 512) == 0
    pm, _ = make_pair(n=N, n_det=D, n_samples=T, radius=0.02, fov_half=0.0063, norm=1.0,
                      max_batch=1)
    ref = pm.estimate_sigma_max(100)
    assert abs(out[0] - ref) / ref < 1e-4
    # power iteration approaches sigma_max from below: within a few per cent
    # of the oracle's own (shorter) estimate
    assert abs(out[0] - om.norm) / om.norm < 3e-2


def _ops(om, W):
    fwd = lambda v: om.forward(v.reshape(W, N, N)).ravel()
    adj = lambda y: om.transpose(y.reshape(W, D, T)).ravel()
    return fwd, adj


@pytest.mark.parametrize("W", [1, 2])
def test_rec_nn_with_L2_reg_gateway(env, model, W):
    # W = 2: one reference call on a two-wavelength stack (coupled)
    drv, om, _ = env
    b = _data(om, W, 40 + W)
    rec = np.empty(W * N * N)
    outs = np.zeros(5)
    msg = C.create_string_buffer(512)
    assert drv.drv_l2(model, mexdrv.dptr(b), b.size, 20, 1e-2, b"fh:@(x) x", -1.0, None,
                      mexdrv.dptr(rec), rec.size, mexdrv.dptr(outs), msg, 512) == 0, msg.value
    fwd, adj = _ops(om, W)
    ref, r_img, r_reg = S.rec_nn_with_L2_reg(fwd, adj, b.ravel(), W * N * N, 20, 1e-2)
    assert rel(rec, ref) <= 1e-3
    assert abs(outs[0] - r_img) / r_img < 1e-3
    assert abs(outs[1] - r_reg) / r_reg < 1e-3
    assert outs[2] == 0.0 and outs[3] == 20 and outs[4] > 0


def test_rec_nn_with_L2_reg_gateway_two_regularisers(env, model):
    # the overview script's RegL2 = @(x) x and RegL2_2 = a handle calling
    # laplacian_per_wavelength
    drv, om, _ = env
    b = _data(om, 1, 43)
    rec = np.empty(N * N)
    outs = np.zeros(5)
    msg = C.create_string_buffer(512)
    lap = (b"fh:@(x) laplacian_per_wavelength(reshape(x, model.Discretization."
           b"sizeOfPixelGrid(2), model.Discretization.sizeOfPixelGrid(1), []))")
    assert drv.drv_l2(model, mexdrv.dptr(b), b.size, 15, 5e-4, b"fh:@(x)x", 5e-3, lap,
                      mexdrv.dptr(rec), rec.size, mexdrv.dptr(outs), msg, 512) == 0, msg.value
    fwd, adj = _ops(om, 1)
    ref, r_img, r_reg, r_reg2 = S.rec_nn_with_L2_reg(fwd, adj, b.ravel(), N * N, 15, 5e-4,
                                                     lambdaL2_2=5e-3, shape=(N, N))
    assert rel(rec, ref) <= 1e-3
    assert abs(outs[0] - r_img) / r_img < 1e-3
    assert abs(outs[2] - r_reg2) / r_reg2 < 1e-3


def test_rec_nn_with_L2_reg_gateway_rejects_other_regularisers(env, model):
    drv, om, _ = env
    b = np.zeros(D * T)
    rec = np.empty(N * N)
    outs = np.zeros(5)
    msg = C.create_string_buffer(512)
    assert drv.drv_l2(model, mexdrv.dptr(b), b.size, 5, 1e-2, b"fh:@(x) 2*x", -1.0, None,
                      mexdrv.dptr(rec), rec.size, mexdrv.dptr(outs), msg, 512) == 1
    assert msg.value.decode().startswith("rec_nn_with_L2_reg:regularizer|")


@pytest.mark.parametrize("which", [1, 2])
def test_rec_nn_with_L1_and_TV_gateways(env, model, which):
    drv, om, _ = env
    b = _data(om, 1, 50 + which)
    rec = np.empty(N * N)
    outs = np.zeros(3)
    msg = C.create_string_buffer(512)
    iters, reg = (15, 1e-3) if which == 1 else (4, 5e-3)
    assert drv.drv_l1_tv(which, model, mexdrv.dptr(b), b.size, iters, reg, mexdrv.dptr(rec),
                         rec.size, mexdrv.dptr(outs), msg, 512) == 0, msg.value
    fwd, adj = _ops(om, 1)
    if which == 1:
        ref, r_img, r_reg = S.rec_nn_with_L1_eye_reg(fwd, adj, b.ravel(), iters, reg)
    else:
        ref = S.rec_nn_with_TV_reg(fwd, adj, b.ravel(), N, N, 1, iters, reg)[0]
    assert rel(rec, ref) <= 1e-3
    assert outs[2] == iters


def test_destroyed_model_is_rejected(env):
    drv, om, fields = env
    h = _create(drv, om, fields, om.norm, 1)
    msg = C.create_string_buffer(512)
    assert drv.drv_model(b"destroy", h, None, 0, None, 0, msg, 512) == 0
    b = np.zeros(D * T)
    rec = np.empty(N * N)
    outs = np.zeros(3)
    assert drv.drv_l1_tv(1, h, mexdrv.dptr(b), b.size, 2, 1e-3, mexdrv.dptr(rec), rec.size,
                         mexdrv.dptr(outs), msg, 512) == 1
    assert msg.value.decode().startswith("rec_nn_with_L1_eye_reg:model|")
