"""Semi-transparent mirror boundaries (MBG_BC_MIRROR; lib.bc_field_mirror).

The reference stores bc_field_reflectivity and applies H = 0 beyond both
ends in every solver (device.hpp:50-79, solver_cpu_fdtd.tpp:263-275); the
mirror boundary is built beside it and is off unless asked for:

- the reference's own bc_field_reflectivity (any values) and a mirror of
  reflectivity 1 give the PMC results bit for bit (oracle);
- a vacuum pulse meets each end and comes back with the stated fraction
  of its energy (oracle; the known answer of the boundary, not of the
  oracle's code);
- the GPU solvers equal the oracle with mirrors (FP64 1e-9, FP32 1e-5),
  in vacuum and in a 2-level medium, whatever the tile shape (bit for
  bit), and runs with different boundaries share one ensemble.
"""
import math

import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

C0 = 1.0 / math.sqrt(mb.MU0 * mb.EPS0)
F0 = 2e14
TAU = 20e-15
T0 = 60e-15
LENGTH = 120e-6


def _vacuum(bc=None, n=8192):
    """Soft Gaussian source in the middle of 120 um of vacuum: one pulse
    runs to each end. Probes at a quarter of the length from each end
    see the outgoing pulse first and its reflection L/(2c) later."""
    mb.material.clear_library()
    vac = setups._material("Vacuum")
    dev = mb.device("mirror", bc)
    dev.add_region(mb.region("Vacuum", vac, 0, LENGTH))
    t_end = T0 + 0.75 * LENGTH / C0 + 4 * TAU
    sce = mb.scenario("mirror", n, t_end, mb.ic_density_const(
        mb.qm_operator([1, 0])), mb.ic_field_const(0.0),
        mb.ic_field_const(0.0))
    sce.add_source(mb.gaussian_pulse("g", LENGTH / 2, mb.source.soft_source,
                                     1e7, F0, T0, TAU))
    sce.add_record(mb.record("eL", mb.record.electric, 0, 0, 0.0,
                             LENGTH / 4))
    sce.add_record(mb.record("eR", mb.record.electric, 0, 0, 0.0,
                             3 * LENGTH / 4))
    return dev, sce


def _medium(bc, n=1203, steps=4000, clear=True):
    """2-level medium (the plain workload's material) with a soft sech
    source in the middle, probes at both ends."""
    if clear:
        mb.material.clear_library()
    dev, sce0 = setups.sit_2lvl(num_gridpoints=n, num_timesteps=steps)
    dev.set_bc_field(bc)
    length = dev.get_length()
    sce = mb.scenario("mirror-medium", n, sce0.get_endtime(),
                      mb.ic_density_const(mb.qm_operator([1, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0))
    sce.add_source(mb.sech_pulse("sech", length / 2, mb.source.soft_source,
                                 setups.sech_area_amplitude(math.pi), 2e14,
                                 15.0, setups.BETA))
    sce.add_record(mb.record("e0", mb.record.electric, 0, 0, 0.0, 0.0))
    sce.add_record(mb.record("e1", mb.record.electric, 0, 0, 0.0, length))
    sce.add_record(mb.record("inv12", 0.0, length / 3))
    return dev, sce


def _energies(e, dt):
    """Energy of the outgoing pulse and of its reflection at a probe a
    quarter length from its end."""
    t = np.arange(len(e)) * dt
    t_out = T0 + 0.25 * LENGTH / C0
    t_back = T0 + 0.75 * LENGTH / C0
    w = 3.5 * TAU
    out = np.sum(e[np.abs(t - t_out) < w] ** 2)
    back = np.sum(e[np.abs(t - t_back) < w] ** 2)
    return out, back


@pytest.mark.parametrize("rl,rr", [(0.64, 0.25), (0.0, 1.0), (0.9, 0.5)])
def test_oracle_mirror_reflects_power(rl, rr):
    dev, sce = _vacuum(mb.bc_field_mirror(rl, rr))
    grid, (eL, eR) = helpers.oracle_results("noop", 0, dev, sce, threads=4)
    dt = grid.timestep_size
    for e, want in ((eL[:, 0], rl), (eR[:, 0], rr)):
        out, back = _energies(e, dt)
        assert out > 0
        # 1-D Yee at Courant 0.5, ~100 points per wavelength: within 2e-4
        assert back / out == pytest.approx(want, abs=2e-3), (want, back / out)


def test_oracle_reference_bc_is_ignored_and_unit_mirror_is_pmc():
    _, base = helpers.oracle_results("noop", 0, *_vacuum(), threads=4)
    for bc in (mb.bc_field_reflectivity(0.3, 0.5), mb.bc_field_mirror(1, 1)):
        _, got = helpers.oracle_results("noop", 0, *_vacuum(bc), threads=4)
        for a, b in zip(got, base):
            assert np.array_equal(a, b)
    # a mirror of reflectivity 1 also leaves the medium runs unchanged
    _, pmc = helpers.oracle_results(
        "cvr-rodr", 2, *_medium(mb.bc_field_reflectivity(0.2, 0.2)))
    _, unit = helpers.oracle_results(
        "cvr-rodr", 2, *_medium(mb.bc_field_mirror(1.0, 1.0)))
    for a, b in zip(unit, pmc):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_mirror_reflectivity_out_of_range_is_rejected(native):
    from mbsolve_gb300 import solvergpu
    dev, sce = _vacuum(mb.bc_field_mirror(1.2, 0.5), n=256)
    with pytest.raises(RuntimeError, match="reflectivity"):
        solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-noop-fp64")


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-5)])
def test_gpu_mirror_matches_oracle(native, prec, tol):
    bc = mb.bc_field_mirror(0.64, 0.25)
    _, ref = helpers.oracle_results("noop", 0, *_vacuum(bc), threads=4)
    _, got = helpers.gpu_results("gpu-fdtd-noop-" + prec, *_vacuum(bc))
    for a, b in zip(got, ref):
        assert helpers.rel_err(a, b) <= tol
    bc = mb.bc_field_mirror(0.3, 0.7)
    _, ref = helpers.oracle_results("cvr-rodr", 2, *_medium(bc), threads=4)
    _, got = helpers.gpu_results("gpu-fdtd-2lvl-cvr-rodr-" + prec,
                                 *_medium(bc))
    for k, (a, b) in enumerate(zip(got, ref)):
        assert helpers.rel_err(a, b) <= tol, (k, helpers.rel_err(a, b))
    # the reflection from the right wall reached the right probe
    _, pmc = helpers.oracle_results(
        "cvr-rodr", 2, *_medium(mb.bc_field_reflectivity()), threads=4)
    assert helpers.rel_err(ref[1], pmc[1]) > 1e-2


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1203, 1200, 1025])
def test_gpu_mirror_tuning_does_not_change_results(native, n):
    """The run's last point sits at every position inside a thread's
    points (n mod C varies): the wall is applied wherever it lands."""
    bc = mb.bc_field_mirror(0.3, 0.7)
    out = []
    for c_, nt, d, g in [(1, 128, 1, 2), (2, 128, 8, 4), (4, 256, 16, 8),
                         (8, 256, 32, 2), (4, 128, 24, 2)]:
        t = helpers.tuning(c_, nt, d, g)
        _, res = helpers.gpu_results("gpu-fdtd-2lvl-cvr-rodr-fp32",
                                     *_medium(bc, n=n, steps=2500), tuning=t)
        out.append(res)
    for res in out[1:]:
        for a, b in zip(res, out[0]):
            assert np.array_equal(a, b)


@pytest.mark.gpu
def test_gpu_mirror_runs_share_an_ensemble(native):
    from mbsolve_gb300 import ensemble
    bcs = [mb.bc_field_mirror(0.3, 0.7), mb.bc_field_reflectivity(),
           mb.bc_field_mirror(0.0, 0.0), mb.bc_field_mirror(1.0, 0.5)]
    mb.material.clear_library()
    pairs = [_medium(bc, n=900 + 101 * i, steps=2000, clear=False)
             for i, bc in enumerate(bcs)]
    ens = ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-fp64", pairs)
    ens.run()
    assert ens.status() == 0
    for i, bc in enumerate(bcs):
        _, single = helpers.gpu_results("gpu-fdtd-2lvl-cvr-rodr-fp64",
                                        *_medium(bc, n=900 + 101 * i,
                                                 steps=2000))
        got = [r.as_array() for r in ens.results(i)]
        for a, b in zip(got, single):
            assert np.array_equal(a, b)
