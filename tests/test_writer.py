"""The result writer (mbsolve_gb300/writer.py): factory behaviour of
writer.hpp/writer.cpp and the HDF5 writer's layout (writer_hdf5.cpp:31-110)
in the npz archive, on results of the CPU oracle (no GPU needed)."""
import numpy as np
import pytest

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups, writer as W


def test_factory_like_reference():
    assert "npz" in W.writer.get_avail_writers()
    w = W.writer.create_instance("npz")
    assert w.get_name() == "npz" and w.get_extension() == "npz"
    with pytest.raises(ValueError, match="Unknown writer"):
        W.writer.create_instance("matlab")
    with pytest.raises(ValueError, match="already registered"):
        W.writer.register_writer("npz", W.writer_npz)


def test_layout_round_trip(tmp_path):
    dev, sce = setups.song2005(num_timesteps=50)
    sce.set_timestep_size(1e-17)
    sce.set_gridpoint_size(1e13)
    rows, cols = 51, 1
    rng = np.random.default_rng(0)
    re, im = rng.normal(size=rows * cols), rng.normal(size=rows * cols)
    results = [mb.result("d11", cols, rows, False, re, np.zeros_like(re)),
               mb.result("d12", cols, rows, True, re, im)]
    f = tmp_path / "out.npz"
    W.writer.create_instance("npz").write(str(f), results, dev, sce)
    z = W.read_npz(str(f))
    assert z["timestep_size"] == 1e-17
    assert z["gridpoint_size"] == 1e13
    assert z["sim_endtime"] == sce.get_endtime()
    assert z["dev_length"] == dev.get_length()
    assert z["d11"]["is_complex"] is False and "imag" not in z["d11"]
    np.testing.assert_array_equal(z["d11"]["real"], re.reshape(rows, cols))
    assert z["d12"]["is_complex"] is True
    np.testing.assert_array_equal(z["d12"]["imag"], im.reshape(rows, cols))
