"""Failure detection on the GPU without a GPU fault: a bounded device wait
that is made to run out (a progress value no tile reaches) ends the run
with an error the host reads, and the GPU stays usable; a NaN injected on
the host (a source table entry) is reported by the run instead of passing
silently. The reference has no device waits; its error pattern for device
failures is common_cuda.hpp:60-66 (std::runtime_error("CUDA: ..."))."""
import ctypes as C
import math

import numpy as np
import pytest

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

pytestmark = pytest.mark.gpu


def _persistent_run(tuning):
    from mbsolve_gb300 import solvergpu
    mb.material.clear_library()
    dev, sce = setups.sit_2lvl(num_gridpoints=3000, num_timesteps=400)
    s = solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-2lvl-cvr-rodr-fp32",
                                  tuning)
    return s


def test_persistent_wait_runs_out_and_gpu_recovers(native, monkeypatch):
    t = helpers.tuning(4, 256, 16, 0, persistent=1)
    # a short bound on every poll loop, and waits that cannot be met
    monkeypatch.setenv("MBG_WAIT_LIMIT", "2000")
    monkeypatch.setenv("MBG_TEST_STALL_PERSIST", "1")
    s = _persistent_run(t)
    with pytest.raises(RuntimeError,
                       match="persistent-kernel wait for neighbour tiles "
                             "ran out"):
        s.run()
    del s
    # the context is intact: the same case runs and equals the
    # launch-per-level kernel bit for bit
    monkeypatch.delenv("MBG_TEST_STALL_PERSIST")
    monkeypatch.delenv("MBG_WAIT_LIMIT")
    s = _persistent_run(t)
    s.run()
    got = s.get_results()[0].as_array()
    s2 = _persistent_run(helpers.tuning(4, 256, 16, 0, persistent=2))
    s2.run()
    assert np.array_equal(got, s2.get_results()[0].as_array())
    assert np.isfinite(got).all()


class _nan_after(mb.source):
    """A source whose value table turns NaN from time t0 on (evaluated on
    the host, like every table source)."""

    def __init__(self, t0):
        super().__init__("nan", 0.0, mb.source.hard_source, 1.0, 0.0)
        self._t0 = t0

    def get_value(self, t, current_value=0.0):
        return math.nan if t >= self._t0 else 0.0


def _add_nan_source(native, dev, sce, step):
    """A hard source at x = 0 that turns NaN at time index `step`, its
    table computed on the scenario's grid."""
    from mbsolve_gb300 import _native
    g = T.mbg_grid()
    b = mb.to_pod(dev, sce)
    _native.check(native.mbg_scenario_grid(C.byref(b.device),
                                           C.byref(b.scenario), C.byref(g)))
    src = _nan_after(step * g.timestep_size)
    mb.tabulate(src, g.num_timesteps, g.timestep_size)
    sce.add_source(src)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_nonfinite_record_is_reported(native, prec):
    from mbsolve_gb300 import solvergpu
    dev, sce = setups.sit_2lvl(num_gridpoints=256, num_timesteps=300)
    sce.add_record(mb.record("e0", mb.record.electric, 1, 1, 0.0, 0.0))
    _add_nan_source(native, dev, sce, 100)
    s = solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-2lvl-cvr-rodr-" + prec)
    with pytest.raises(RuntimeError, match="non-finite value"):
        s.run()
    # the results stay readable; the NaN appears where the source set it
    e0 = s.get_results()[1].as_array().ravel()
    assert np.isfinite(e0[:90]).all()
    assert np.isnan(e0[-1])


def test_nonfinite_in_ensemble_run_is_reported(native):
    from mbsolve_gb300 import ensemble
    runs = []
    for k in range(3):
        dev, sce = setups.sit_2lvl(num_gridpoints=256 + 64 * k,
                                   num_timesteps=300)
        if k == 1:
            sce.add_record(mb.record("e0", mb.record.electric, 1, 1, 0.0,
                                     0.0))
            _add_nan_source(native, dev, sce, 150)
        runs.append((dev, sce))
    e = ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-fp32", runs)
    with pytest.raises(RuntimeError, match="non-finite value"):
        e.run()
    assert e.status() & 1
