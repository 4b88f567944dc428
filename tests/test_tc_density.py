"""The tensor-core density products (4-6 levels, FP32, tcgen05 kind::tf32)
against the CUDA-core FP32 kernel and FP64 on the same runs: probe traces
agree to the FP32 kernels' accuracy and no tensor-core wait runs out."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5   # the FP32 kernels' probe-field target vs FP64


def _probe(name, tuning, N, seed):
    from mbsolve_gb300 import ensemble, lib as mb, setups
    mb.material.clear_library()
    runs = [setups.random_nlvl(N=N, num_gridpoints=3000, num_timesteps=800,
                               seed=seed + k) for k in range(3)]
    e = ensemble.ensemble(name, runs, tuning)
    e.run()
    out = [e.results(r)[0].as_array().ravel() for r in range(3)]
    st = e.status()
    info = e.info()
    e.close()
    return out, st, info


@pytest.mark.parametrize("N", [4, 5, 6])
def test_tensor_core_products_match_cuda_cores_and_fp64(native, N):
    from mbsolve_gb300 import ensemble
    ref, st, _ = _probe("gpu-fdtd-%dlvl-cvr-rodr-fp64" % N, None, N, 10 * N)
    assert st == 0
    tc, st_tc, info = _probe("gpu-fdtd-%dlvl-cvr-rodr-fp32" % N,
                             ensemble.tuning(1, 128, 8), N, 10 * N)
    assert st_tc == 0
    assert info["threads"] == 128
    cc, st_cc, _ = _probe("gpu-fdtd-%dlvl-cvr-rodr-fp32" % N,
                          ensemble.tuning(1, 256, 8), N, 10 * N)
    assert st_cc == 0
    for a, b, r in zip(tc, cc, ref):
        e_tc = np.linalg.norm(a - r) / np.linalg.norm(r)
        e_cc = np.linalg.norm(b - r) / np.linalg.norm(r)
        print("N=%d tensor cores %.2e, CUDA cores %.2e" % (N, e_tc, e_cc))
        assert e_cc < TOL, e_cc
        assert e_tc < TOL, e_tc


def _two_region(N, seed):
    """random_nlvl's medium behind a vacuum section: tiles at the boundary
    mix materials and take the tensor-core kernel's CUDA-core path."""
    from mbsolve_gb300 import lib as mb, setups
    dev0, sce = setups.random_nlvl(N=N, num_gridpoints=3000, num_timesteps=800,
                                   seed=seed)
    ar = dev0.get_regions()[0].get_material()
    length = dev0.get_length()
    vac = setups._material("Vacuum")
    dev = mb.device("mixed")
    dev.add_region(mb.region("Vacuum", vac, 0.0, 0.3 * length))
    dev.add_region(mb.region("Active", ar, 0.3 * length, length))
    return dev, sce


def _probe_one(name, tuning, N, seed):
    from mbsolve_gb300 import ensemble, lib as mb
    mb.material.clear_library()
    e = ensemble.ensemble(name, [_two_region(N, seed)], tuning)
    e.run()
    out = e.results(0)[0].as_array().ravel()
    st = e.status()
    e.close()
    return out, st


@pytest.mark.parametrize("N", [4, 6])
def test_mixed_tiles_in_tensor_core_kernel(native, N):
    from mbsolve_gb300 import ensemble
    ref, st = _probe_one("gpu-fdtd-%dlvl-cvr-rodr-fp64" % N, None, N, 3)
    assert st == 0
    name = "gpu-fdtd-%dlvl-cvr-rodr-fp32" % N
    tc8, st8 = _probe_one(name, ensemble.tuning(1, 128, 8), N, 3)
    tc4, st4 = _probe_one(name, ensemble.tuning(1, 128, 4), N, 3)
    cc, stc = _probe_one(name, ensemble.tuning(1, 256, 8), N, 3)
    assert st8 == st4 == stc == 0
    # the schedule does not change the arithmetic of a point
    np.testing.assert_array_equal(tc8, tc4)
    e_tc = np.linalg.norm(tc8 - ref) / np.linalg.norm(ref)
    e_cc = np.linalg.norm(cc - ref) / np.linalg.norm(ref)
    print("N=%d mixed: tensor cores %.2e, CUDA cores %.2e" % (N, e_tc, e_cc))
    assert e_tc < TOL and e_cc < TOL
