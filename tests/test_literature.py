"""Known-answer tests against the literature traces the reference ships
(tools/reference-data, digitised from the papers; fixture built by
tests/golden/literature/make_traces.py). Plot-level tolerances: the traces are
digitised curves. The FP64 oracle (CPU) and the GPU solvers (FP64 and
FP32) must both reproduce them:

- Ziolkowski et al. 1995, fig. 2: population inversion along the device at
  187.5 fs (record row 75) of the self-induced-transparency preset;
- Song et al. 2005, fig. 3a: rho11 of the 0-D V-type 3-level system (the
  digitised time axis is shifted by < 1 fs; the comparison allows the best
  shift within +-1 fs);
- Marskar et al. 2011: rho55 and rho66 of the 6-level ladder at the source
  point (shortened device with the reference grid spacing; the records sit
  where the hard source fixes the field).
"""
import os

import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups

HERE = os.path.dirname(os.path.abspath(__file__))


def _fixture():
    return np.load(os.path.join(HERE, "golden", "literature", "traces.npz"))


def _err(t, y, ref, tscale, shifts=(0.0,)):
    """rms and max deviation of y(t) from the digitised trace, at the best
    of the given time shifts of the trace."""
    best = None
    for s in shifts:
        ct = (ref[:, 0] + s) * tscale
        m = (ct >= t[0]) & (ct <= t[-1])
        d = np.interp(ct[m], t, y) - ref[m, 1]
        r = (float(np.sqrt(np.mean(d * d))), float(np.abs(d).max()))
        if best is None or r[0] < best[0]:
            best = r
    return best


def _song():
    return setups.song2005()


def _marskar():
    return setups.marskar2011(N=6, num_gridpoints=16,
                              length=1e-3 * 15 / 8191)


def _check(kind, results, dt, dx):
    z = _fixture()
    if kind == "song":
        d11 = results[0][:, 0]
        t = np.arange(len(d11)) * dt
        rms, mx = _err(t, d11, z["song2005_d11"], 1e-15,
                       shifts=np.linspace(-1.0, 1.0, 41))
        assert rms < 0.05, (rms, mx)
    elif kind == "marskar":
        for k, key in ((4, "marskar2011_d55"), (5, "marskar2011_d66")):
            y = results[k][:, 0]
            t = np.arange(len(y)) * dt
            rms, mx = _err(t, y, z[key], 1e-12)
            assert rms < 0.01 and mx < 0.05, (key, rms, mx)
    else:
        inv = results[0][75]
        x = np.arange(len(inv)) * dx
        rms, mx = _err(x, inv, z["ziolkowski1995_inv12_row75"], 1e-6)
        assert rms < 0.03 and mx < 0.1, (rms, mx)


CASES = [("song", _song, 3), ("marskar", _marskar, 6),
         ("ziolkowski", setups.ziolkowski1995, 2)]


@pytest.mark.parametrize("kind,build,N", CASES)
def test_oracle_reproduces_literature(kind, build, N):
    from oracle import oracle as O
    mb.material.clear_library()
    dev, sce = build()
    o = O.OracleRun("cvr-rodr", N, mb.to_pod(dev, sce))
    o.run()
    g = o.grid()
    _check(kind, [r[0] for r in o.results()], g.timestep_size,
           g.gridpoint_size)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("kind,build,N", CASES)
def test_gpu_reproduces_literature(native, kind, build, N, prec):
    from mbsolve_gb300 import solvergpu
    mb.material.clear_library()
    dev, sce = build()
    s = solvergpu.solver_gpu_fdtd(dev, sce,
                                  "gpu-fdtd-%dlvl-cvr-rodr-%s" % (N, prec))
    s.run()
    _check(kind, [r.as_array() for r in s.get_results()],
           sce.get_timestep_size(), sce.get_gridpoint_size())
