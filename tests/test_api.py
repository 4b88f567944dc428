"""Host-side behaviour without a GPU: the C-ABI library exports every
symbol the header declares, the Python mirror of mbsolve.lib keeps the
reference's semantics, configuration errors are reported as the reference
reports them."""
import ctypes as C
import os
import re

import pytest

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "mbsolve_gb300.h")).read() + \
        open(os.path.join(ROOT, "include", "mbsolve_fno.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mbg_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(native):
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(native, n), n


def test_solver_names_follow_reference_scheme(native):
    from mbsolve_gb300 import _native
    names = _native.solver_names()
    assert "gpu-fdtd-2lvl-cvr-rodr-fp32" in names
    assert "gpu-fdtd-6lvl-reg-cayley-fp64" in names
    assert "gpu-fdtd-noop-fp64" in names
    assert len(names) == 22


def test_registration_in_factory(native):
    from mbsolve_gb300 import solvergpu  # noqa: F401  (registers)
    avail = mb.solver.get_avail_solvers()
    assert "gpu-fdtd-3lvl-reg-cayley-fp32" in avail
    with pytest.raises(RuntimeError, match="Unknown solver"):
        mb.solver.create_instance("cpu-fdtd-9lvl", None, None)
    with pytest.raises(RuntimeError, match="already registered"):
        mb.solver.register_bootstrap("gpu-fdtd-noop-fp32", lambda d, s: None)


def test_unknown_solver_name_is_invalid_argument(native):
    dev, sce = setups.sit_2lvl(64, 10)
    b = mb.to_pod(dev, sce)
    h = C.c_void_p()
    rc = native.mbg_solver_create(b"gpu-fdtd-7lvl-cvr-rodr-fp32",
                                  C.byref(b.device), C.byref(b.scenario),
                                  None, C.byref(h))
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert native.mbg_last_error().startswith(b"Unknown solver")


def test_scenario_grid_matches_oracle(native):
    from mbsolve_gb300 import _native
    from oracle import oracle as O
    for dev, sce in (setups.ziolkowski1995(2048, 100e-15),
                     setups.song2005(), setups.sit_2lvl(16384, 100000)):
        b = mb.to_pod(dev, sce)
        g = T.mbg_grid()
        _native.check(native.mbg_scenario_grid(C.byref(b.device),
                                               C.byref(b.scenario),
                                               C.byref(g)))
        og = O.OracleRun("noop", 0, b).grid()
        assert (g.num_gridpoints, g.num_timesteps) == \
            (og.num_gridpoints, og.num_timesteps)
        assert g.timestep_size == og.timestep_size
        assert g.gridpoint_size == og.gridpoint_size
    # the plain 2-level workload: 16,384 points, 100,000 steps
    dev, sce = setups.sit_2lvl(16384, 100000)
    b = mb.to_pod(dev, sce)
    _native.check(native.mbg_scenario_grid(C.byref(b.device),
                                           C.byref(b.scenario), C.byref(g)))
    assert g.num_timesteps == 100000
    assert g.gridpoint_size == pytest.approx(150e-6 / 16383, rel=1e-12)


def test_configuration_errors(native):
    from mbsolve_gb300 import _native
    # no regions
    dev = mb.device("empty")
    sce = mb.scenario("s", 16, 1e-15, mb.qm_operator([1, 0]))
    b = mb.to_pod(dev, sce)
    g = T.mbg_grid()
    rc = native.mbg_scenario_grid(C.byref(b.device), C.byref(b.scenario),
                                  C.byref(g))
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert b"No regions in device!" == native.mbg_last_error()
    # 0-D with fewer than 2 steps
    mat = mb.material("m0")
    mb.material.add_to_library(mat)
    dev = mb.device("d")
    dev.add_region(mb.region("r", mat, 0, 0))
    sce = mb.scenario("s", 1, 1e-15, mb.qm_operator([1, 0]), 1)
    b = mb.to_pod(dev, sce)
    rc = native.mbg_scenario_grid(C.byref(b.device), C.byref(b.scenario),
                                  C.byref(g))
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert native.mbg_last_error() == b"Invalid scenario."


def test_lindblad_relaxation_constructor_semantics():
    r = mb.qm_lindblad_relaxation([[0, 2.0, 1.0], [3.0, 0, 0], [0, 5.0, 0]],
                                  [1.0, -2.0, 0.5])
    s = r.get_scattering_rates()
    # diagonal = -(sum of scattering out of the level) (qm_description.hpp:
    # 177-187)
    assert s[0][0] == -3.0 and s[1][1] == -7.0 and s[2][2] == -1.0
    d = r.get_dephasing_rates()
    assert d[0] == -1.0 - 0.5 * (3.0 + 7.0)
    assert d[1] == -2.0 - 0.5 * (3.0 + 1.0)
    assert d[2] == -0.5 - 0.5 * (7.0 + 1.0)


def test_qm_desc_2lvl_matches_reference_formulas():
    q = mb.qm_desc_2lvl(1e24, 2 * mb.PI * 2e14, 6.24e-11, 1e10, 2e10, -1.0)
    h = q.get_hamiltonian().get_main_diagonal()
    assert h[0] == -mb.HBAR * 2 * mb.PI * 2e14 / 2
    assert q.get_dipole_operator().get_off_diagonal()[0] == -mb.E0 * 6.24e-11
    r = q.get_relaxation_superop()
    assert r.get_dephasing_rates()[0] == -2e10


def test_record_name_parsing():
    assert mb.record("inv12", 1e-15).get_type() == mb.record.inversion
    assert mb.record("e0", 0.0, 1e-6).get_type() == mb.record.electric
    r = mb.record("d23", mb.record.density, 2, 3, 0.0, 0.0)
    assert (r.get_row(), r.get_col(), r.is_complex()) == (1, 2, True)
    with pytest.raises(RuntimeError, match="Unknown record type"):
        mb.record("x", 0.0)


def test_device_materials_sorted_like_std_set():
    a = mb.material("zz")
    b = mb.material("Aa")
    c = mb.material("m")
    dev = mb.device("d")
    for m in (a, b, c, a):
        dev.add_region(mb.region("r", m, 0, 1e-6))
    assert dev.get_used_materials() == ["Aa", "m", "zz"]
    assert dev.get_length() == pytest.approx(4e-6)
