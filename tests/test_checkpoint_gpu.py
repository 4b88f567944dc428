"""Checkpoint and resume of an ensemble (mbg_ensemble_save_state /
load_state): a run interrupted, saved, restored into a fresh ensemble of
the same descriptions and continued gives bit-identical results to the
uninterrupted run; a checkpoint of another ensemble is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ens(prec, n, seed=7):
    from mbsolve_gb300 import ensemble, lib as mb, setups
    mb.material.clear_library()
    runs, _ = setups.ensemble_2lvl(num_runs=n, num_timesteps=4000, seed=seed)
    return ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-" + prec, runs,
                             ensemble.tuning(2, 128, 8))


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_resume_is_bit_identical(native, prec, tmp_path):
    a = _ens(prec, 6)
    a.run()
    want = [a.results(r)[0].as_array() for r in range(6)]
    a.close()
    b = _ens(prec, 6)
    b.advance(1237)
    path = str(tmp_path / "ck.bin")
    b.save(path)
    b.close()
    c = _ens(prec, 6)
    c.load(path)
    c.run()
    for r in range(6):
        np.testing.assert_array_equal(c.results(r)[0].as_array(), want[r])
    c.close()


def test_foreign_checkpoint_is_refused(native):
    from mbsolve_gb300 import _native
    a = _ens("fp32", 6)
    a.advance(100)
    buf = a.save_state()
    a.close()
    b = _ens("fp32", 5)
    with pytest.raises(_native.MbgError):
        b.load_state(buf)
    with pytest.raises(_native.MbgError):
        b.load_state(buf[:10])
    b.close()


def test_same_size_other_physics_is_refused(native):
    """A checkpoint of an ensemble with the same sizes (runs, points,
    steps, records) but another material is refused: its state would
    continue under the wrong physics."""
    from mbsolve_gb300 import _native, ensemble, lib as mb, setups

    def ens(t2):
        mb.material.clear_library()
        runs = [setups.sit_2lvl(num_gridpoints=700, num_timesteps=900,
                                t2=t2) for _ in range(2)]
        return ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-fp32", runs,
                                 ensemble.tuning(2, 128, 8))
    a = ens(1e-12)
    a.advance(300)
    buf = a.save_state()
    a.close()
    b = ens(2e-12)
    with pytest.raises(_native.MbgError, match="other descriptions"):
        b.load_state(buf)
    b.close()
    c = ens(1e-12)
    c.load_state(buf)
    c.run()
    assert c.status() == 0
    c.close()

