"""GPU solvers for the mbsolve-style Python API.

Importing this module registers the solvers of the CUDA engine in
:class:`mbsolve_gb300.lib.solver`'s factory, as ``import mbsolve.solvercpu``
registers the reference's CPU solvers (solver-cpu/swig/solvercpu.i:6-9).
Names: ``gpu-fdtd-{N}lvl-{cvr-rodr|reg-cayley}-{fp32|fp64}`` and
``gpu-fdtd-noop-{fp32|fp64}``; the results match the reference's
``cpu-fdtd-{N}lvl-...`` solvers (solver_cpu_fdtd.tpp).
"""
import ctypes as C

import numpy as np

from . import capi_types as T
from . import lib as mb
from . import _native


class solver_gpu_fdtd(mb.solver):
    """One scenario on the GPU. The constructor does the reference's set-up
    (and, like it, writes the grid back into the scenario); run() advances
    num_timesteps steps; get_results() returns one result per record."""

    def __init__(self, dev, scen, name, tuning=None):
        super().__init__(name, dev, scen)
        L = _native.load()
        self._L = L
        self._bundle = mb.to_pod(dev, scen)
        h = C.c_void_p()
        tp = C.byref(tuning) if tuning is not None else None
        _native.check(L.mbg_solver_create(
            name.encode(), C.byref(self._bundle.device),
            C.byref(self._bundle.scenario), tp, C.byref(h)))
        self._h = h
        g = T.mbg_grid()
        _native.check(L.mbg_solver_grid(h, C.byref(g)))
        # init_fdtd_simulation mutates the scenario (common_fdtd.hpp:52-123)
        scen.set_gridpoint_size(g.gridpoint_size)
        scen.set_timestep_size(g.timestep_size)
        scen.set_num_timesteps(g.num_timesteps)
        self._grid = g
        self._results = []
        for k, rec in enumerate(scen.get_records()):
            r, c, z = C.c_uint32(), C.c_uint32(), C.c_int32()
            _native.check(L.mbg_solver_result_shape(h, k, C.byref(r),
                                                    C.byref(c), C.byref(z)))
            self._results.append(mb.result(rec.get_name(), c.value, r.value,
                                           bool(z.value)))

    def run(self):
        rc = self._L.mbg_solver_run(self._h)
        if rc != T.MBG_OK:
            # keep the error text: the copies below overwrite it
            err = _native.MbgError(rc, self._L.mbg_last_error().decode())
        for k, res in enumerate(self._results):
            re = np.zeros(res.get_count())
            im = np.zeros(res.get_count())
            crc = self._L.mbg_solver_copy_result(
                self._h, k, re.ctypes.data_as(T.PD), im.ctypes.data_as(T.PD))
            if crc != T.MBG_OK:
                if rc == T.MBG_OK:
                    _native.check(crc)
                break
            res._real = re
            res._imag = im
        # a run that diverged (NaN/Inf) or whose device wait ran out raises
        # after its results are in place, so that they can be inspected
        if rc != T.MBG_OK:
            raise err

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.mbg_solver_destroy(h)
            self._h = None


def _register():
    for name in _native.solver_names():
        if name not in mb.solver._bootstraps:
            mb.solver.register_bootstrap(
                name, (lambda n: (lambda dev, scen:
                                  solver_gpu_fdtd(dev, scen, n)))(name))


class solver_gpu_loader:
    """Mirror of solver_cpu_loader (solver-cpu/src/solver_cpu_loader.cpp:
    32-89): constructing it registers the GPU solvers."""

    def __init__(self):
        _register()


_register()
