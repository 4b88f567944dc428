"""The persistent time-step kernel (mbg_tuning.persistent = 1): resident
CTAs take the tiles of successive launches in order, each tile waiting for
its own and its neighbours' previous level. Same tiles, same arithmetic as
the launch-per-level kernels: results equal bit for bit, for ensembles of
uneven runs (short runs of one tile, runs that end at different steps,
mirror walls and coherence records on the non-uniform path), for the
tensor-core kernels, and across advances of any length."""
import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import ensemble, setups
from tests import helpers

pytestmark = pytest.mark.gpu


def _pairs():
    mb.material.clear_library()
    out = []
    for i, (n, steps) in enumerate([(5000, 1800), (700, 1500), (64, 900),
                                    (2300, 1711), (9000, 1800)]):
        dev, sce = setups.sit_2lvl(num_gridpoints=n, num_timesteps=steps,
                                   area=1.0 + 0.7 * i, detuning=0.01 * i)
        if i == 3:
            dev.set_bc_field(mb.bc_field_mirror(0.4, 0.6))
        sce.add_record(mb.coherence_record("d12", 1, 2, 0.0, -1.0))
        out.append((dev, sce))
    return out


def _run(name, pairs, t, chunks):
    ens = ensemble.ensemble(name, pairs, t)
    for c in chunks:
        ens.advance(c)
    ens.run()
    assert ens.status() == 0
    return ens, [[r.get_data_complex() for r in ens.results(i)]
                 for i in range(len(pairs))]


@pytest.mark.parametrize("depth", [16, 5])
def test_persistent_equals_launch_per_level(native, depth):
    name = "gpu-fdtd-2lvl-cvr-rodr-fp32"
    chunks = [1, 37, 300, 999]
    _, ref = _run(name, _pairs(), helpers.tuning(4, 256, depth, 8, 2), chunks)
    ens, got = _run(name, _pairs(), helpers.tuning(4, 256, depth, 8, 1),
                    chunks)
    assert ens.info()["persistent"] == 1
    for a, b in zip(got, ref):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("levels", [4, 6])
def test_persistent_tensor_core_equals_launch_per_level(native, levels):
    name = "gpu-fdtd-%dlvl-cvr-rodr-fp32" % levels

    def pairs():
        mb.material.clear_library()
        return [setups.random_nlvl(N=levels, num_gridpoints=n,
                                   num_timesteps=300, seed=s, e_seed=3e7)
                for n, s in ((6000, 1), (300, 2))]

    t0 = helpers.tuning(1, 128, 8, 8, 2)
    t1 = helpers.tuning(1, 128, 8, 8, 1)
    _, ref = _run(name, pairs(), t0, [77])
    ens, got = _run(name, pairs(), t1, [77])
    assert ens.info()["persistent"] == 1
    for a, b in zip(got, ref):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("levels", [4, 6])
def test_persistent_cayley_equals_launch_per_level(native, levels):
    name = "gpu-fdtd-%dlvl-reg-cayley-fp32" % levels

    def pairs():
        mb.material.clear_library()
        return [setups.random_nlvl(N=levels, num_gridpoints=n,
                                   num_timesteps=300, seed=s, e_seed=3e7)
                for n, s in ((6000, 3), (300, 4))]

    _, ref = _run(name, pairs(), helpers.tuning(1, 128, 8, 8, 2), [77])
    ens, got = _run(name, pairs(), helpers.tuning(1, 128, 8, 8, 1), [77])
    assert ens.info()["persistent"] == 1
    for a, b in zip(got, ref):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))


def test_persistent_is_chosen_for_few_tiles(native):
    """Automatic choice: a short single run (a few tiles per launch) takes
    the persistent kernel, a wide ensemble the launch per level."""
    mb.material.clear_library()
    few = ensemble.ensemble("gpu-fdtd-6lvl-cvr-rodr-fp32",
                            [setups.random_nlvl(N=6, num_gridpoints=4096,
                                                num_timesteps=50)],
                            helpers.tuning(1, 128, 8, 8))
    assert few.info()["persistent"] == 1
    few.close()
    mb.material.clear_library()
    many = ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-fp32",
                             [setups.sit_2lvl(num_gridpoints=30000,
                                              num_timesteps=50)
                              for _ in range(64)],
                             helpers.tuning(4, 256, 16, 8))
    assert many.info()["persistent"] == 0
    many.close()


def test_persistent_single_solver_matches_oracle(native, monkeypatch):
    """MBG_PERSISTENT=1 through the reference-facing solver."""
    monkeypatch.setenv("MBG_PERSISTENT", "1")
    mb.material.clear_library()
    dev, sce = setups.sit_2lvl(num_gridpoints=3000, num_timesteps=2000)
    _, got = helpers.gpu_results("gpu-fdtd-2lvl-cvr-rodr-fp32", dev, sce,
                                 helpers.tuning(4, 256, 16, 8))
    mb.material.clear_library()
    dev, sce = setups.sit_2lvl(num_gridpoints=3000, num_timesteps=2000)
    _, ref = helpers.oracle_results("cvr-rodr", 2, dev, sce)
    for a, b in zip(got, ref):
        assert helpers.rel_err(a, b) <= 1e-5
