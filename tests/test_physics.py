"""Analytic known answers (the oracle on the CPU; the GPU solvers in FP64 and
FP32):

- Rabi flopping: a resonant sech pulse of area pi on an undamped 2-level
  system at one point inverts it (inversion -1 -> +1), area 2 pi returns
  it to the ground state (the pulse area theorem; counter-rotating terms
  at Rabi/carrier ~ 0.02 leave errors of ~1e-3);
- vacuum propagation (Maxwell only): a Gaussian pulse travels at c between
  two probes and keeps its energy (1-D Yee scheme at Courant 0.5, ~200
  points per wavelength);
- Cayley form: the populations of a 3-level Lambda medium sum to 1 along
  the run (unitary propagation, trace-preserving dissipation; FP32 with
  the once-per-launch FP64 trace renormalisation).
"""
import math

import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups

BETA = 2.0 * math.acosh(2.0) / 100e-15   # 100 fs FWHM
F0 = 2e14
D_M = 6.24e-11                            # dipole / e in metres


def _rabi(area):
    qm = mb.qm_desc_2lvl(1e24, 2 * math.pi * F0, D_M, 0.0, 0.0, -1.0)
    ar = setups._material("AR_Rabi", qm)
    dev = mb.device("rabi")
    dev.add_region(mb.region("Active region (single point)", ar, 0, 0))
    phase = 12.0
    t_end = 2 * phase / BETA
    sce = mb.scenario("rabi", 1, t_end,
                      mb.ic_density_const(mb.qm_operator([1, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0), 40000)
    ampl = area * mb.HBAR * BETA / (math.pi * mb.E0 * D_M)
    sce.add_source(mb.sech_pulse("sech", 0.0, mb.source.hard_source, ampl,
                                 F0, phase, BETA))
    sce.add_record(mb.record("inv12", 0.0))
    return dev, sce


def _vacuum():
    vac = setups._material("Vacuum")
    dev = mb.device("vacuum")
    # 60 um: the reflection from the far boundary reaches the probes only
    # after the window
    dev.add_region(mb.region("Vacuum", vac, 0, 60e-6))
    sce = mb.scenario("vacuum", 8192, 250e-15, mb.ic_density_const(
        mb.qm_operator([1, 0])), mb.ic_field_const(0.0),
        mb.ic_field_const(0.0))
    sce.add_source(mb.gaussian_pulse("g", 0.0, mb.source.hard_source, 1e9,
                                     F0, 60e-15, 20e-15))
    sce.add_record(mb.record("e1", mb.record.electric, 0, 0, 0.0, 5e-6))
    sce.add_record(mb.record("e2", mb.record.electric, 0, 0, 0.0, 25e-6))
    return dev, sce


def _lambda():
    dev, sce = setups.lambda_3lvl(num_gridpoints=4096, num_timesteps=60000,
                                  probe=2e-6)
    for i in (1, 2, 3):
        sce.add_record(mb.record("d%d%d" % (i, i), mb.record.density, i, i,
                                 0.0, 2e-6))
    return dev, sce


def _check_rabi(area, inv):
    want = 1.0 if abs(area - math.pi) < 1e-9 else -1.0
    assert inv[0] == pytest.approx(-1.0, abs=1e-12)
    assert abs(inv[-1] - want) < 1e-2, (area, inv[-1])
    if want > 0:
        assert inv.max() > 0.99


def _check_vacuum(e1, e2, dt):
    t = np.arange(len(e1)) * dt
    c1 = np.sum(t * e1 ** 2) / np.sum(e1 ** 2)
    c2 = np.sum(t * e2 ** 2) / np.sum(e2 ** 2)
    c0 = 1.0 / math.sqrt(mb.MU0 * mb.EPS0)
    assert (c2 - c1) == pytest.approx(20e-6 / c0, rel=5e-3)
    assert np.sum(e2 ** 2) == pytest.approx(np.sum(e1 ** 2), rel=1e-2)


def _check_lambda(pops, tol):
    s = pops[0] + pops[1] + pops[2]
    assert np.abs(s - 1.0).max() < tol, np.abs(s - 1.0).max()
    assert pops[1].max() > 1e-3    # the pulses did move population


@pytest.mark.parametrize("area", [math.pi, 2 * math.pi])
def test_oracle_rabi_flopping(area):
    from oracle import oracle as O
    mb.material.clear_library()
    dev, sce = _rabi(area)
    o = O.OracleRun("cvr-rodr", 2, mb.to_pod(dev, sce))
    o.run(threads=1)
    _check_rabi(area, o.results()[0][0][:, 0])


def test_oracle_vacuum_propagation():
    from oracle import oracle as O
    mb.material.clear_library()
    dev, sce = _vacuum()
    o = O.OracleRun("noop", 0, mb.to_pod(dev, sce))
    o.run()
    r = o.results()
    _check_vacuum(r[0][0][:, 0], r[1][0][:, 0], o.grid().timestep_size)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("area", [math.pi, 2 * math.pi])
def test_gpu_rabi_flopping(native, prec, area):
    from mbsolve_gb300 import solvergpu
    mb.material.clear_library()
    dev, sce = _rabi(area)
    s = solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-2lvl-cvr-rodr-" + prec)
    s.run()
    _check_rabi(area, s.get_results()[0].as_array()[:, 0])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_vacuum_propagation(native, prec):
    from mbsolve_gb300 import solvergpu
    mb.material.clear_library()
    dev, sce = _vacuum()
    s = solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-noop-" + prec)
    s.run()
    r = s.get_results()
    _check_vacuum(r[0].as_array()[:, 0], r[1].as_array()[:, 0],
                  sce.get_timestep_size())


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_gpu_cayley_keeps_trace(native, prec, tol):
    from mbsolve_gb300 import solvergpu
    mb.material.clear_library()
    dev, sce = _lambda()
    s = solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-3lvl-reg-cayley-" + prec)
    s.run()
    r = s.get_results()
    _check_lambda([r[k].as_array()[:, 0] for k in (1, 2, 3)], tol)
