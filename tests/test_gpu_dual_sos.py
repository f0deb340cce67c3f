"""Dual speed of sound on the GPU (Fermat refraction at a polynomial
membrane) against the FP64 oracle: travel-time indices within 1e-7 samples,
membrane intersections within 1e-7 m, and the dual-SoS operator A / A^T
within 1e-5 relative (the operator bar)."""
import numpy as np
import pytest

from oracle import model as M
from pairs import rel

pytestmark = pytest.mark.gpu

CB, CA = 1560.0, 1480.0  # medium, coupling


def _geom(n, n_det, fov_half, membrane):
    from msot_gb300 import Discretization, Probe
    from msot_gb300.synthetic import gauss_pulse_eir
    eir = gauss_pulse_eir()
    p = Probe(n_det=n_det, radius=0.040, angular_coverage=135.0, n_samples=2030, eir=eir,
              eir_length=eir.size, membrane=tuple(membrane), coupling_speed_of_sound=CA)
    op = M.ArcProbe(n_det=n_det, radius=0.040, coverage_deg=135.0, n_samples=2030, eir=eir,
                    eir_length=eir.size)
    return p, Discretization([-fov_half, fov_half], n), op, M.Grid(n, n, (-fov_half, fov_half,
                                                                           -fov_half, fov_half))


# flat membrane between FOV and array; a curved one; one cutting the FOV
# (pixels above it travel straight at the coupling speed)
@pytest.mark.parametrize("membrane", [(-0.014,), (-0.014, 0.0, 3.0), (-0.004, 0.05)])
def test_dual_travel_times_match_oracle(cuda, membrane):
    from msot_gb300.model import travel_times_dual
    p, d, op, og = _geom(40, 48, 0.0127, membrane)
    tau, xm = travel_times_dual(p, d, CB, CA, membrane, n_crop=2)
    rt, rx = M.travel_time_indices_dual(op, og, CB, CA, membrane, n_crop=2)
    assert np.max(np.abs(tau - rt)) <= 1e-7
    assert np.array_equal(np.isnan(xm), np.isnan(rx))
    ok = ~np.isnan(rx)
    if ok.any():
        assert np.max(np.abs(xm[ok] - rx[ok])) <= 1e-7


def test_dual_equal_speeds_is_the_straight_ray(cuda):
    from msot_gb300.model import travel_times, travel_times_dual
    p, d, _, _ = _geom(32, 32, 0.0127, (-0.014, 0.0, 3.0))
    tau, _ = travel_times_dual(p, d, 1500.0, 1500.0, p.membrane)
    assert np.max(np.abs(tau - travel_times(p, d, 1500.0))) <= 1e-7


def test_dual_sos_operator_matches_oracle(cuda):
    import torch
    from msot_gb300 import MSOTmodel
    mem = (-0.014, 0.0, 3.0)
    p, d, op, og = _geom(48, 64, 0.0063, mem)
    pm = MSOTmodel(p, d, CB, False, False, 0, 1e5, 12e6, 1.0, max_batch=2)
    om = M.Model(op, og, c=CB, norm=1.0, membrane=mem, c_coupling=CA)
    assert np.max(np.abs(pm.travel - om.travel)) <= 1e-7
    rng = np.random.default_rng(4)
    x = rng.random((2, 48, 48))
    y = pm.forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < 1e-5
    s = rng.standard_normal((2, 64, 2030))
    assert rel(pm.transpose(torch.tensor(s, dtype=torch.float32)).cpu().numpy(),
               om.transpose(s)) < 1e-5


def test_dual_sos_needs_membrane_and_coupling_speed(cuda):
    from msot_gb300 import Discretization, MSOTmodel, Probe
    with pytest.raises(ValueError):
        MSOTmodel(Probe(n_det=16), Discretization([-0.003, 0.003], 16), CB, False, False)


def test_virtual_sources_match_oracle(cuda):
    from msot_gb300.model import travel_times_dual
    mem = (-0.014, 0.0, 3.0)
    p, d, op, og = _geom(24, 32, 0.0127, mem)
    tau, xm, vx, vz = travel_times_dual(p, d, CB, CA, mem, virtual=True)
    rx, rz = M.virtual_sources(op, og, CB, CA, mem)
    # the travel time is stationary in x_m, so two searches agree on x_m (and
    # the ray direction through it) only to ~1e-9 m: bar 1e-8 m
    assert np.max(np.abs(vx - rx)) <= 1e-8 and np.max(np.abs(vz - rz)) <= 1e-8
    # the virtual source lies at distance t * c_coupling from its detector
    xd, zd = op.positions()
    dist = np.hypot(vx - xd[:, None], vz - zd[:, None])
    assert np.max(np.abs(dist - tau / p.fs * CA)) <= 1e-12


def test_dual_sos_with_sir_matches_oracle(cuda):
    # SPMR tables from the virtual sources (MSOTmodel.m:579-596) with the
    # coupling speed, then the SIR operator on the Fermat travel times
    import torch
    from oracle import sir as Q
    from msot_gb300 import MSOTmodel
    from msot_gb300.sir import spmr_tables, virtual_sources
    mem = (-0.014, 0.0, 3.0)
    n, D = 24, 32
    p, d, op, og = _geom(n, D, 0.004, mem)
    virt = virtual_sources(p, d, CB)
    sir, se, idx, meta = spmr_tables(p, d, CA, element=(0.25e-3, 10e-3, 0.0), sub=(4, 4),
                                     half_window=60, virtual=virt)
    rsir, rse, ridx, info = Q.spmr_tables(D, 0.040, 135.0, d.x, d.z, CA, p.fs, d.sigma, 0.25e-3,
                                          10e-3, 0.0, 4, 4, half_window=meta["half_window"],
                                          virtual=M.virtual_sources(op, og, CB, CA, mem))
    assert rel(sir, rsir) <= 1e-9
    assert np.array_equal(se, rse) and np.array_equal(idx, ridx)
    pm = MSOTmodel(p, d, CB, True, False, 0, 1e5, 12e6, 1.0, sir_tables=(sir, se, idx),
                   max_batch=2)
    om = M.Model(op, og, c=CB, norm=1.0, include_sir=True, membrane=mem, c_coupling=CA)
    om.sir_tables = (sir, se, idx)
    rng = np.random.default_rng(6)
    x = rng.random((2, n, n))
    y = pm.forward(torch.tensor(x, dtype=torch.float32)).cpu().numpy()
    assert rel(y, om.forward(x)) < 1e-5
    s = rng.standard_normal((2, D, 2030))
    assert rel(pm.transpose(torch.tensor(s, dtype=torch.float32)).cpu().numpy(),
               om.transpose(s)) < 1e-5
