"""Shared test helpers: run a (device, scenario) on the oracle, on the
reference-built library and on the GPU engine, and compare results."""
import ctypes as C
import json
import os

import numpy as np

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def build_setup(spec):
    """(device, scenario) from a JSON-able spec {"setup": name, "kw": {}}."""
    fn = getattr(setups, spec["setup"])
    return fn(**spec.get("kw", {}))


def oracle_results(algo, num_levels, dev, sce, threads=2, max_steps=0):
    from oracle import oracle as O
    b = mb.to_pod(dev, sce)
    o = O.OracleRun(algo, num_levels, b)
    o.run(threads=threads, max_steps=max_steps)
    return o.grid(), [r for r, _ in o.results()]


def reference_results(name, dev, sce):
    from oracle import oracle as O
    b = mb.to_pod(dev, sce)
    r = O.ReferenceRun(name, b)
    r.run()
    return r.grid(), [x for x, _ in r.results(len(sce.get_records()))]


def gpu_results(name, dev, sce, tuning=None):
    from mbsolve_gb300 import solvergpu
    s = solvergpu.solver_gpu_fdtd(dev, sce, name, tuning)
    s.run()
    return s._grid, [r.as_array() for r in s.get_results()]


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b.ravel())
    num = np.linalg.norm((a - b).ravel())
    if den == 0.0:
        return num
    return num / den


def load_golden(case):
    d = np.load(os.path.join(GOLDEN, case + ".npz"))
    meta = json.loads(str(d["meta"]))
    recs = [d["rec%d" % k] for k in range(meta["num_records"])]
    return meta, recs


def golden_cases():
    if not os.path.isdir(GOLDEN):
        return []
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def plane_basis_step(c, L, d, e):
    """One step of the engine's plane-basis form (numpy, FP64) from a
    constant block `c` with layout `L`: returns (d', P) for coherence
    vector d and field e. The kernels keep v = u + (Bh u + kh), u = Q^T d
    (half a step ahead), rotate it and apply the full step Bd, k; d' comes
    back through u' = (I + Bh)^-1 (v' - kh)."""
    import math
    V = L["V"]
    Q = c[L["Q"]:L["Q"] + V * V].reshape(V, V)
    Bh = c[L["Bh"]:L["Bh"] + V * V].reshape(V, V)
    kh = c[L["kh"]:L["kh"] + V]
    Bd = c[L["Bd"]:L["Bd"] + V * V].reshape(V, V)
    k_ = c[L["k"]:L["k"] + V]
    g = c[L["g"]:L["g"] + V]
    th = c[L["thdt"]:L["thdt"] + V // 2]
    u = Q.T @ d
    v = u + (Bh @ u + kh)
    for k in range(V // 2):
        phi = th[k] * e
        a, b = v[2 * k], v[2 * k + 1]
        v[2 * k] = math.cos(phi) * a - math.sin(phi) * b
        v[2 * k + 1] = math.sin(phi) * a + math.cos(phi) * b
    v2 = v + (Bd @ v + k_)
    u2 = np.linalg.solve(np.eye(V) + Bh, v2 - kh)
    return Q @ u2, c[L["p0"]] + g @ v2


def tuning(C_=0, NT=0, depth=0, graph=0, persistent=0):
    t = T.mbg_tuning()
    t.persistent = persistent
    t.cells_per_thread = C_
    t.threads = NT
    t.depth = depth
    t.launches_per_graph = graph
    return t
