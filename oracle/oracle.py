"""ORACLE — test infrastructure only.

ctypes front end of the FP64 CPU oracle (mb_oracle.cpp) and of the
reference's own time loop built from its sources (oracle/_ref). Used by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; never by
the product.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build
from mbsolve_gb300 import capi_types as T

_lib = None
_base = None
_ref = {}


def lib():
    global _lib
    if _lib is None:
        _lib = _bind(C.CDLL(_build.build_oracle()))
    return _lib


def baseline_lib():
    """The same restatement built with the reference's own solver-cpu
    flags (oracle/build.py build_baseline): the timed CPU baseline."""
    global _base
    if _base is None:
        _base = _bind(C.CDLL(_build.build_baseline()))
    return _base


def _bind(L):
    L.mbo_last_error.restype = C.c_char_p
    L.mbo_create.argtypes = [C.c_char_p, C.c_uint32,
                             C.POINTER(T.mbg_device),
                             C.POINTER(T.mbg_scenario),
                             C.POINTER(C.c_void_p)]
    L.mbo_grid.argtypes = [C.c_void_p, C.POINTER(T.mbg_grid)]
    L.mbo_run.argtypes = [C.c_void_p, C.c_int, C.c_uint32]
    L.mbo_run_red.argtypes = [C.c_void_p, C.c_int, C.c_uint32, C.c_int]
    L.mbo_num_results.argtypes = [C.c_void_p, C.POINTER(C.c_uint32)]
    L.mbo_result_shape.argtypes = [C.c_void_p, C.c_uint32,
                                   C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_uint32),
                                   C.POINTER(C.c_int32)]
    L.mbo_copy_result.argtypes = [C.c_void_p, C.c_uint32, T.PD, T.PD]
    L.mbo_state.argtypes = [C.c_void_p, T.PD, T.PD, T.PD, T.PD]
    L.mbo_destroy.argtypes = [C.c_void_p]
    L.mbo_expm.argtypes = [C.c_int, T.PD, T.PD]
    L.mbo_rodr_constants.argtypes = [C.POINTER(T.mbg_qm), C.c_double,
                                     C.c_double] + [T.PD] * 9
    return L


def ref_lib(baseline=False):
    """The reference-built library, or None when the reference tree is
    absent (the GPU machines have only the oracle restatement); baseline:
    the build with the CPU baseline's flags."""
    if baseline not in _ref:
        path = _build.build_reference(baseline=baseline)
        if path is None:
            return None
        L = C.CDLL(path)
        L.mbr_last_error.restype = C.c_char_p
        L.mbr_create.argtypes = [C.c_char_p, C.POINTER(T.mbg_device),
                                 C.POINTER(T.mbg_scenario),
                                 C.POINTER(C.c_void_p)]
        L.mbr_grid.argtypes = [C.c_void_p, C.POINTER(T.mbg_grid)]
        L.mbr_run.argtypes = [C.c_void_p]
        L.mbr_result_shape.argtypes = [C.c_void_p, C.c_uint32,
                                       C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_uint32),
                                       C.POINTER(C.c_int32)]
        L.mbr_copy_result.argtypes = [C.c_void_p, C.c_uint32, T.PD, T.PD]
        L.mbr_destroy.argtypes = [C.c_void_p]
        _ref[baseline] = L
    return _ref[baseline]


def _ptr(a):
    return a.ctypes.data_as(T.PD)


class OracleError(RuntimeError):
    pass


class OracleRun:
    """One oracle solver: create, run (optionally a bounded number of
    steps), read grid and results."""

    def __init__(self, algo, num_levels, bundle, baseline=False):
        L = baseline_lib() if baseline else lib()
        self._L = L
        self._bundle = bundle
        h = C.c_void_p()
        rc = L.mbo_create(algo.encode(), num_levels, C.byref(bundle.device),
                          C.byref(bundle.scenario), C.byref(h))
        if rc != 0:
            raise OracleError(L.mbo_last_error().decode())
        self._h = h

    def grid(self):
        g = T.mbg_grid()
        self._L.mbo_grid(self._h, C.byref(g))
        return g

    def run(self, threads=None, max_steps=0, red=0):
        """solver_cpu_fdtd's loop, or with red > 0 the temporally blocked
        loop of solver_cpu_fdtd_red with an overlap of `red` steps (the
        same results bit for bit)."""
        if threads is None:
            threads = os.cpu_count() or 1
        if red:
            rc = self._L.mbo_run_red(self._h, int(threads), int(max_steps),
                                     int(red))
        else:
            rc = self._L.mbo_run(self._h, int(threads), int(max_steps))
        if rc != 0:
            raise OracleError(self._L.mbo_last_error().decode())

    def results(self):
        n = C.c_uint32()
        self._L.mbo_num_results(self._h, C.byref(n))
        out = []
        for k in range(n.value):
            r, c, z = C.c_uint32(), C.c_uint32(), C.c_int32()
            self._L.mbo_result_shape(self._h, k, C.byref(r), C.byref(c),
                                     C.byref(z))
            re = np.zeros(r.value * c.value)
            im = np.zeros(r.value * c.value)
            self._L.mbo_copy_result(self._h, k, _ptr(re), _ptr(im))
            out.append((re.reshape(r.value, c.value),
                        im.reshape(r.value, c.value) if z.value else None))
        return out

    def state(self, n_x, dens_len):
        e = np.zeros(n_x)
        h = np.zeros(n_x + 1)
        p = np.zeros(n_x)
        d = np.zeros(max(1, n_x * dens_len))
        self._L.mbo_state(self._h, _ptr(e), _ptr(h), _ptr(p), _ptr(d))
        return e, h, p, d

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.mbo_destroy(self._h)
            self._h = None


class ReferenceRun:
    """The reference's own solver (e.g. "cpu-fdtd-2lvl-cvr-rodr")."""

    def __init__(self, name, bundle, baseline=False):
        L = ref_lib(baseline)
        if L is None:
            raise OracleError("reference tree not available")
        self._L = L
        self._bundle = bundle
        h = C.c_void_p()
        rc = L.mbr_create(name.encode(), C.byref(bundle.device),
                          C.byref(bundle.scenario), C.byref(h))
        if rc != 0:
            raise OracleError(L.mbr_last_error().decode())
        self._h = h

    def grid(self):
        g = T.mbg_grid()
        self._L.mbr_grid(self._h, C.byref(g))
        return g

    def run(self):
        rc = self._L.mbr_run(self._h)
        if rc != 0:
            raise OracleError(self._L.mbr_last_error().decode())

    def results(self, n):
        out = []
        for k in range(n):
            r, c, z = C.c_uint32(), C.c_uint32(), C.c_int32()
            self._L.mbr_result_shape(self._h, k, C.byref(r), C.byref(c),
                                     C.byref(z))
            re = np.zeros(r.value * c.value)
            im = np.zeros(r.value * c.value)
            self._L.mbr_copy_result(self._h, k, _ptr(re), _ptr(im))
            out.append((re.reshape(r.value, c.value),
                        im.reshape(r.value, c.value) if z.value else None))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            self._L.mbr_destroy(self._h)
            self._h = None


def expm(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    out = np.zeros_like(a)
    rc = lib().mbo_expm(a.shape[0], _ptr(a), _ptr(out))
    if rc != 0:
        raise OracleError(lib().mbo_last_error().decode())
    return out


def rodr_constants(qm_pod, dt, probe):
    """Rodrigues constants of one material (see mbo_rodr_constants)."""
    n = qm_pod.num_levels
    V = n * n - 1
    M, U, A1, A2 = (np.zeros((V, V)) for _ in range(4))
    theta = np.zeros(max(1, V // 2))
    v, deq, din = np.zeros(V), np.zeros(V), np.zeros(V)
    mcp = np.zeros(1)
    rc = lib().mbo_rodr_constants(C.byref(qm_pod), dt, probe, _ptr(M),
                                  _ptr(U), _ptr(A1), _ptr(theta), _ptr(v),
                                  _ptr(deq), _ptr(din), _ptr(mcp), _ptr(A2))
    if rc != 0:
        raise OracleError(lib().mbo_last_error().decode())
    return dict(M=M, U=U, A1=A1, theta=theta, v=v, d_eq=deq, d_in=din,
                M_CP=mcp[0], A2=A2)
