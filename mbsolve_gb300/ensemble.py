"""Batched ensembles: many independent Maxwell-Bloch runs in one launch.

No reference counterpart: the reference runs one scenario per solver
object (solver.hpp:42-142). An ensemble packs all runs' grid points into
one ragged layout in HBM and advances them in lock-step with one kernel
launch per temporal block; runs may differ in length, materials, sources
and records. Per-run results have the same layout as the single-run
solver's.
"""
import ctypes as C

import numpy as np

from . import capi_types as T
from . import lib as mb
from . import _native


class ensemble:
    def __init__(self, name, runs, tuning=None):
        """runs: list of (device, scenario) pairs."""
        L = _native.load()
        self._L = L
        self._name = name
        self._bundles = [mb.to_pod(d, s) for d, s in runs]
        n = len(self._bundles)
        devs = (C.POINTER(T.mbg_device) * n)()
        scens = (C.POINTER(T.mbg_scenario) * n)()
        for i, b in enumerate(self._bundles):
            devs[i] = C.pointer(b.device)
            scens[i] = C.pointer(b.scenario)
        h = C.c_void_p()
        tp = C.byref(tuning) if tuning is not None else None
        _native.check(L.mbg_ensemble_create(name.encode(), n, devs, scens, tp,
                                            C.byref(h)))
        self._h = h
        self._n = n
        self._scens = [s for _, s in runs]
        for i, s in enumerate(self._scens):
            g = self.grid(i)
            s.set_gridpoint_size(g.gridpoint_size)
            s.set_timestep_size(g.timestep_size)
            s.set_num_timesteps(g.num_timesteps)

    def __len__(self):
        return self._n

    def grid(self, run):
        g = T.mbg_grid()
        _native.check(self._L.mbg_ensemble_grid(self._h, run, C.byref(g)))
        return g

    def advance(self, steps):
        _native.check(self._L.mbg_ensemble_advance(self._h, int(steps)))

    def run(self):
        _native.check(self._L.mbg_ensemble_run(self._h))

    def progress(self):
        d, t = C.c_uint64(), C.c_uint64()
        _native.check(self._L.mbg_ensemble_progress(self._h, C.byref(d),
                                                    C.byref(t)))
        return d.value, t.value

    def info(self):
        cells, tiles = C.c_uint64(), C.c_uint32()
        t = T.mbg_tuning()
        _native.check(self._L.mbg_ensemble_info(self._h, C.byref(cells),
                                                C.byref(tiles), C.byref(t)))
        return dict(cells=cells.value, tiles=tiles.value,
                    cells_per_thread=t.cells_per_thread, threads=t.threads,
                    depth=t.depth, launches_per_graph=t.launches_per_graph,
                    staging=t.staging, persistent=t.persistent)

    def results(self, run):
        out = []
        for k, rec in enumerate(self._scens[run].get_records()):
            r, c, z = C.c_uint32(), C.c_uint32(), C.c_int32()
            _native.check(self._L.mbg_ensemble_result_shape(
                self._h, run, k, C.byref(r), C.byref(c), C.byref(z)))
            re = np.zeros(r.value * c.value)
            im = np.zeros(r.value * c.value)
            _native.check(self._L.mbg_ensemble_copy_result(
                self._h, run, k, re.ctypes.data_as(T.PD),
                im.ctypes.data_as(T.PD)))
            out.append(mb.result(rec.get_name(), c.value, r.value,
                                 bool(z.value), re, im))
        return out

    def probe_rows(self, k, row0, nrows):
        """Rows [row0, row0+nrows) of single-point record k of every run,
        as a [runs, nrows] FP64 array."""
        out = np.zeros((self._n, nrows))
        _native.check(self._L.mbg_ensemble_copy_probe_rows(
            self._h, k, row0, nrows, out.ctypes.data_as(T.PD)))
        return out

    def set_timing(self, on=True):
        _native.check(self._L.mbg_ensemble_set_timing(self._h, int(on)))

    def kernel_time(self, reset=False):
        """(launches, milliseconds) of the time-step kernel since reset."""
        n, ms = C.c_uint64(), C.c_double()
        _native.check(self._L.mbg_ensemble_kernel_time(
            self._h, C.byref(n), C.byref(ms), int(reset)))
        return n.value, ms.value

    def region_begin(self):
        """Start a CUDA-event timed region on the ensemble's stream."""
        _native.check(self._L.mbg_ensemble_stream_time(self._h, 1, None))

    def region_end(self):
        """End the region; returns its device time in milliseconds."""
        ms = C.c_double()
        _native.check(self._L.mbg_ensemble_stream_time(self._h, 0,
                                                       C.byref(ms)))
        return ms.value

    def launches(self):
        """Kernel launches issued so far on this ensemble's stream."""
        n = C.c_uint64()
        _native.check(self._L.mbg_ensemble_launches(self._h, C.byref(n)))
        return n.value

    def pod_bytes(self):
        """Bytes of host description data handed to the engine."""
        return sum(C.sizeof(o) for b in self._bundles for o in b.keep)

    def status(self):
        f = C.c_uint32()
        _native.check(self._L.mbg_ensemble_status(self._h, C.byref(f)))
        return f.value

    def save_state(self):
        """Checkpoint: the full time-loop state as a numpy uint8 array."""
        n = C.c_uint64()
        _native.check(self._L.mbg_ensemble_state_size(self._h, C.byref(n)))
        buf = np.empty(n.value, dtype=np.uint8)
        _native.check(self._L.mbg_ensemble_save_state(
            self._h, buf.ctypes.data_as(C.c_void_p), n.value))
        return buf

    def load_state(self, buf):
        """Resume from save_state() of an ensemble of the same runs."""
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        _native.check(self._L.mbg_ensemble_load_state(
            self._h, buf.ctypes.data_as(C.c_void_p), buf.size))

    def save(self, path):
        with open(path, "wb") as f:
            f.write(self.save_state().tobytes())

    def load(self, path):
        with open(path, "rb") as f:
            self.load_state(np.frombuffer(f.read(), dtype=np.uint8))

    def close(self):
        if getattr(self, "_h", None):
            self._L.mbg_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def tuning(cells_per_thread=0, threads=0, depth=0, launches_per_graph=0,
           staging=0, persistent=0):
    """Launch shape (0 = autotuned); staging 1 = bulk-copy (TMA) staging of
    the tile state (2-level FP32); persistent 1 = one persistent kernel per
    advance where the launch shape has one, 2 = one launch per level, 0 =
    automatic (persistent when a launch has few waves of tiles)."""
    t = T.mbg_tuning()
    t.staging = staging
    t.persistent = persistent
    t.cells_per_thread = cells_per_thread
    t.threads = threads
    t.depth = depth
    t.launches_per_graph = launches_per_graph
    return t
