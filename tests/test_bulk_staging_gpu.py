"""The 2-level FP32 kernels with bulk-copy (TMA) staging of the tile state
(tuning.staging = 1 or MBG_TILE_STAGING=bulk) compute the same numbers as
the default kernels that load the state into registers: results are
bit-identical over ragged ensembles and several launch shapes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(shape, staging):
    from mbsolve_gb300 import ensemble, lib as mb, setups
    mb.material.clear_library()
    runs, _ = setups.ensemble_2lvl(num_runs=12, num_timesteps=700, seed=5)
    c, nt, d = shape
    e = ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-fp32", runs,
                          ensemble.tuning(c, nt, d, staging=staging))
    e.run()
    out = [e.results(r)[0].as_array() for r in range(len(runs))]
    info, st = e.info(), e.status()
    e.close()
    return out, info, st


@pytest.mark.parametrize("shape", [(4, 256, 16), (2, 128, 8), (8, 256, 32),
                                   (1, 128, 1)])
def test_bulk_staging_is_bit_identical(native, shape):
    ref, info0, st0 = _run(shape, 0)
    got, info1, st1 = _run(shape, 1)
    assert info0["staging"] == 0 and info1["staging"] == 1
    assert st0 == 0 and st1 == 0
    for a, b in zip(got, ref):
        np.testing.assert_array_equal(a, b)


def test_environment_selects_bulk_staging(native, monkeypatch):
    monkeypatch.setenv("MBG_TILE_STAGING", "bulk")
    _, info, st = _run((4, 256, 16), 0)
    assert info["staging"] == 1 and st == 0
