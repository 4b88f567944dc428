"""The benchmark configurations at their own step counts against the FP64
oracle (the reference's time loop restated), in FP64 and FP32:

- plain 2-level medium: 16,384 points, 100,000 steps (full size);
- 6-level random medium (seed 0), Rodrigues and Cayley: 128 points at the
  65,536-point workload's grid spacing, all 200,000 steps;
- 3-level Lambda medium, Cayley: 512 points at the 1,048,576-point
  workload's grid spacing, all 500,000 steps (between the PMC ends the two
  pulses cross the shortened device about 60 times).

Per case: relative L2 error of the probe E trace at the output facet, the
largest population error at the probe point (records every 100 steps) and
the drift of the population sum there. FP64 must match the oracle to
1e-9, FP32 to 1e-5 (probe, populations) and 1e-6 (trace). The oracle
runs on a host thread while the GPU runs (ctypes releases the GIL)."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

pytestmark = pytest.mark.gpu

TOL = {"fp64": (1e-9, 1e-9, 1e-12), "fp32": (1e-5, 1e-5, 1e-6)}


def _with_populations(dev, sce, N, x, every):
    for i in range(1, N + 1):
        sce.add_record(mb.record("d%d%d" % (i, i), mb.record.density, i, i,
                                 every, x))
    return dev, sce


def _c2(algo):
    n = 128
    length = 150e-6 * (n - 1) / 65535

    def build():
        dev, sce = setups.random_nlvl(N=6, num_gridpoints=n,
                                      num_timesteps=200000, seed=0,
                                      length=length)
        dt = sce.get_endtime() / 200000
        return _with_populations(dev, sce, 6, length, 100 * dt)
    return (algo, 6, build, "gpu-fdtd-6lvl-%s-" % algo)


def _c4():
    n = 512
    length = 150e-6 * (n - 1) / 16383

    def build():
        dev, sce = setups.lambda_3lvl(num_gridpoints=n, num_timesteps=500000,
                                      length=length)
        dt = sce.get_endtime() / 500000
        return _with_populations(dev, sce, 3, length, 100 * dt)
    return ("reg-cayley", 3, build, "gpu-fdtd-3lvl-reg-cayley-")


def _c1():
    return ("cvr-rodr", 2, lambda: setups.sit_2lvl(16384, 100000),
            "gpu-fdtd-2lvl-cvr-rodr-")


CASES = {"plain_2lvl_full": _c1(), "6lvl_rodr_200k": _c2("cvr-rodr"),
         "6lvl_cayley_200k": _c2("reg-cayley"),
         "3lvl_lambda_cayley_500k": _c4()}


@pytest.fixture(scope="module")
def oracle_runs():
    """Every case's oracle result, computed on one host thread in the
    background while the GPU tests run. The scenarios are flattened here,
    on the calling thread (the material library is process-global)."""
    from oracle import oracle as O
    bundles = {}
    for key, (algo, N, build, _) in CASES.items():
        mb.material.clear_library()
        dev, sce = build()
        bundles[key] = (algo, N, mb.to_pod(dev, sce))
    mb.material.clear_library()
    threads = max(1, (os.cpu_count() or 2) - 2)

    def run(key):
        algo, N, b = bundles[key]
        o = O.OracleRun(algo, N, b)
        o.run(threads=threads)
        return [r for r, _ in o.results()]
    ex = cf.ThreadPoolExecutor(1)
    futs = {k: ex.submit(run, k) for k in CASES}
    yield futs
    ex.shutdown(wait=True)


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("key", list(CASES))
def test_config_at_full_step_count(native, oracle_runs, key, prec):
    algo, N, build, prefix = CASES[key]
    mb.material.clear_library()
    dev, sce = build()
    _, got = helpers.gpu_results(prefix + prec, dev, sce)
    ref = oracle_runs[key].result()
    tol_e, tol_pop, tol_tr = TOL[prec]
    e_err = helpers.rel_err(got[0], ref[0])
    line = "%s %s: probe E rel L2 %.2e" % (key, prec, e_err)
    if len(ref) > 1:
        pg = np.hstack([g.reshape(-1, 1) for g in got[1:]])
        pr = np.hstack([r.reshape(-1, 1) for r in ref[1:]])
        pop_err = float(np.abs(pg - pr).max())
        drift = float(np.abs(pg.sum(axis=1) - 1.0).max())
        line += ", populations max abs %.2e, trace drift %.2e" % (pop_err,
                                                                  drift)
        assert pop_err <= tol_pop, line
        assert drift <= tol_tr, line
    print(line)
    assert e_err <= tol_e, line
