"""GPU parity through the C-ABI: every golden case (the reference's own
time loop) in FP64 and FP32, tuning invariance (temporal blocking depth,
tile shape) bit for bit, ensembles against single runs, error paths."""
import ctypes as C

import numpy as np
import pytest

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

pytestmark = pytest.mark.gpu

# relative L2 error per record against the reference's FP64 result. FP32
# keeps the density state (coherence vector or Cayley density matrix), and
# E and H in all but the 2-level kernel, as float pairs, with the
# field-free part of every step from the FP64 precompute.
TOL = {"fp64": 1e-9, "fp32": 1e-5}


def _gpu_name(cpu_name, prec):
    return cpu_name.replace("cpu-", "gpu-") + "-" + prec


def _check(a, b, tol, what):
    nb = np.linalg.norm(b)
    err = np.linalg.norm(a - b)
    if nb == 0.0:
        assert err <= 1e-300 or err <= tol * 1e-6, (what, err)
        return 0.0
    assert err <= tol * nb, (what, err / nb)
    return err / nb


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("case", helpers.golden_cases())
def test_gpu_matches_golden(native, case, prec):
    meta, recs = helpers.load_golden(case)
    dev, sce = helpers.build_setup(meta["spec"])
    grid, res = helpers.gpu_results(_gpu_name(meta["solver"], prec), dev, sce)
    assert grid.num_timesteps == meta["num_timesteps"]
    assert sce.get_timestep_size() == meta["timestep_size"]
    errs = []
    tol = TOL[prec]
    for k, (a, b) in enumerate(zip(res, recs)):
        assert a.shape == b.shape
        errs.append(_check(a, b, tol, (case, k)))
    print(case, prec, ["%.2e" % e for e in errs])


@pytest.mark.parametrize("name,setup,kw", [
    ("gpu-fdtd-2lvl-cvr-rodr-fp32", "sit_2lvl",
     dict(num_gridpoints=3000, num_timesteps=700)),
    ("gpu-fdtd-2lvl-cvr-rodr-fp64", "sit_2lvl",
     dict(num_gridpoints=3000, num_timesteps=700)),
    ("gpu-fdtd-3lvl-reg-cayley-fp32", "lambda_3lvl",
     dict(num_gridpoints=2000, num_timesteps=500)),
    ("gpu-fdtd-2lvl-cvr-rodr-fp32", "ziolkowski1995",
     dict(num_gridpoints=2500, endtime=40e-15)),
    # off-diagonal Hamiltonian and complex dipole: a dense 2-level block
    # (the pair path's general variant)
    ("gpu-fdtd-2lvl-cvr-rodr-fp32", "random_nlvl",
     dict(N=2, num_gridpoints=3000, num_timesteps=700, seed=2, e_seed=3e7)),
])
def test_tuning_does_not_change_results(native, name, setup, kw):
    """Temporal blocking depth and tile shape change only the schedule:
    results are bit-identical (a halo error would show here)."""
    shapes = [(1, 128, 1, 2), (2, 128, 8, 4), (4, 256, 16, 8),
              (8, 256, 32, 2), (1, 128, 24, 2), (2, 256, 5, 0)]
    out = []
    for c_, nt, d, g in shapes:
        mb.material.clear_library()
        dev, sce = helpers.build_setup({"setup": setup, "kw": kw})
        t = helpers.tuning(c_, nt, d, g)
        try:
            _, res = helpers.gpu_results(name, dev, sce, t)
        except Exception as e:  # shape not instantiated for this algo
            if "no kernel instantiated" in str(e):
                continue
            raise
        out.append(res)
    assert len(out) >= 3
    for res in out[1:]:
        for a, b in zip(res, out[0]):
            assert np.array_equal(a, b)


def _sit_split(n, steps, split):
    """The self-induced-transparency medium of setups.sit_2lvl over n points
    with whole-grid records of E, H, P and the inversion every 25 steps;
    split > 0 cuts it into regions of `split` points that alternate between
    two materials with the same parameters, so that every tile holds two
    materials."""
    L = setups.LENGTH_2LVL * (n - 1) / 16383.0
    qm = mb.qm_desc_2lvl(1e24, 2 * mb.PI * 2e14, setups.DIPOLE / mb.E0,
                         1e9, 1e12, -1.0)
    mats = [mb.material("split_%s_%d_%d" % (k, n, split), qm) for k in "ab"]
    for m in mats:
        mb.material.add_to_library(m)
    dev = mb.device("split")
    if split <= 0:
        dev.add_region(mb.region("all", mats[0], 0.0, L))
    else:
        dx = L / (n - 1)
        for k, x0 in enumerate(range(0, n, split)):
            x1 = min(x0 + split, n - 1)
            dev.add_region(mb.region("r%d" % k, mats[k % 2], x0 * dx,
                                     x1 * dx))
    sce = mb.scenario("split", n, setups._courant_endtime(n, L, steps),
                      mb.ic_density_const(mb.qm_operator([1, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0))
    sce.add_source(mb.sech_pulse("sech", 0.0, mb.source.hard_source,
                                 setups.sech_area_amplitude(2.5), 2e14,
                                 15.0, setups.BETA))
    dt = sce.get_endtime() / (steps - 1.5)
    for name in ("e", "h", "p", "inv12"):
        sce.add_record(mb.record(name, 25 * dt))
    sce.add_record(mb.record("e_probe", 0.0, L))
    return dev, sce


def test_pair_path_equals_scalar_path(native):
    """The 2-level FP32 kernel updates uniform tiles two points per
    instruction (packed FP32 pairs) and tiles of several materials one
    point at a time, each with the same roundings: the same medium as one
    material and as alternating copies of it gives equal results at every
    point, at every shape (C = 1 keeps the one-point loop on uniform tiles
    too)."""
    n, steps = 2900, 600
    ref = None
    for split in (37, 0):
        for c_, nt, d in ([(4, 128, 16)] if split else
                          [(1, 128, 8), (2, 128, 8), (4, 128, 16),
                           (4, 256, 32), (8, 128, 7)]):
            mb.material.clear_library()
            dev, sce = _sit_split(n, steps, split)
            _, res = helpers.gpu_results("gpu-fdtd-2lvl-cvr-rodr-fp32", dev,
                                         sce, helpers.tuning(c_, nt, d, 2))
            assert all(np.isfinite(r).all() for r in res)
            if ref is None:
                ref = res
                # the pulse has crossed part of the medium
                assert np.abs(ref[0]).max() > 0.0
                continue
            for k, (a, b) in enumerate(zip(res, ref)):
                assert np.array_equal(a, b), (split, c_, nt, d, k,
                                              np.abs(a - b).max())


def test_run_twice_continues_like_reference(native):
    from oracle import oracle as O
    dev, sce = setups.ziolkowski1995(1024, 30e-15)
    b = mb.to_pod(dev, sce)
    o = O.OracleRun("cvr-rodr", 2, b)
    o.run(threads=2)
    o.run(threads=2)
    ref = [r for r, _ in o.results()]
    mb.material.clear_library()
    dev, sce = setups.ziolkowski1995(1024, 30e-15)
    from mbsolve_gb300 import solvergpu
    s = solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-2lvl-cvr-rodr-fp64")
    s.run()
    s.run()
    for a, r in zip(s.get_results(), ref):
        _check(a.as_array(), r, 1e-9, "run twice")


def _ensemble_runs():
    runs = []
    for n, area, det, t2 in [(700, 2.0, 0.0, 1e-9), (2500, 6.0, 0.03, 1e-12),
                             (1201, 3.0, -0.04, 3e-13), (64, 9.0, 0.01, 1e-11)]:
        runs.append(("sit_2lvl", dict(num_gridpoints=n, num_timesteps=900,
                                      area=area, detuning=det, t2=t2)))
    runs.append(("ziolkowski1995", dict(num_gridpoints=1500, endtime=40e-15)))
    return runs


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_ensemble_equals_single_runs(native, prec):
    from mbsolve_gb300 import ensemble
    specs = _ensemble_runs()
    pairs = [helpers.build_setup({"setup": s, "kw": kw}) for s, kw in specs]
    ens = ensemble.ensemble("gpu-fdtd-2lvl-cvr-rodr-" + prec, pairs)
    ens.run()
    assert ens.status() == 0
    for i, (s, kw) in enumerate(specs):
        mb.material.clear_library()
        dev, sce = helpers.build_setup({"setup": s, "kw": kw})
        _, single = helpers.gpu_results("gpu-fdtd-2lvl-cvr-rodr-" + prec,
                                        dev, sce)
        got = [r.as_array() for r in ens.results(i)]
        for a, b in zip(got, single):
            assert np.array_equal(a, b)
        if prec == "fp64":
            mb.material.clear_library()
            dev, sce = helpers.build_setup({"setup": s, "kw": kw})
            _, orc = helpers.oracle_results("cvr-rodr", 2, dev, sce)
            for a, b in zip(got, orc):
                _check(a, b, 1e-9, ("ensemble", i))


def test_device_precompute_equals_host(native):
    from mbsolve_gb300 import _native
    for N in (2, 3, 6):
        dev, sce = setups.random_nlvl(N=N, num_gridpoints=16,
                                      num_timesteps=10, seed=N)
        b = mb.to_pod(dev, sce)
        mat = b.device.materials[0]
        n = C.c_size_t()
        _native.check(native.mbg_material_constants(
            b"cvr-rodr", C.byref(mat), 2e-17, 0, None, 0, C.byref(n)))
        host = np.zeros(n.value)
        devc = np.zeros(n.value)
        for arr, on in ((host, 0), (devc, 1)):
            _native.check(native.mbg_material_constants(
                b"cvr-rodr", C.byref(mat), 2e-17, on,
                arr.ctypes.data_as(T.PD), arr.size, C.byref(n)))
        L = _native.material_layout("cvr-rodr", N)
        # the plane basis is not unique (degenerate planes, null space), so
        # compare what it computes: one update from the same state
        rng = np.random.default_rng(N)
        for e in (0.0, 2e8, -7e8):
            d = rng.normal(size=L["V"]) * 0.3
            dh, ph = helpers.plane_basis_step(host, L, d, e)
            dd, pd = helpers.plane_basis_step(devc, L, d, e)
            np.testing.assert_allclose(dd, dh, rtol=0, atol=1e-12)
            # P ~ n mu omega ~ 1e10 A/m^2 for these media
            assert abs(pd - ph) <= 1e-8 * max(abs(ph), 1e10)


def test_errors_reported_like_reference(native):
    from mbsolve_gb300 import solvergpu
    # gap between regions: "region not found" (solver_cpu_fdtd.tpp:119-125)
    qm = mb.qm_desc_2lvl(1e24, 2 * mb.PI * 2e14, 6.24e-11, 1e10, 1e10)
    m = mb.material("gap", qm)
    mb.material.add_to_library(m)
    dev = mb.device("gap")
    dev.add_region(mb.region("a", m, 0, 1e-6))
    dev.add_region(mb.region("b", m, 2e-6, 3e-6))
    sce = mb.scenario("s", 64, 1e-15, mb.ic_density_const(
        mb.qm_operator([1, 0])), mb.ic_field_const(0.0))
    with pytest.raises(RuntimeError, match="region not found"):
        solvergpu.solver_gpu_fdtd(dev, sce, "gpu-fdtd-2lvl-cvr-rodr-fp32")
    # level count mismatch
    dev2, sce2 = setups.sit_2lvl(64, 10)
    with pytest.raises(RuntimeError, match="does not match"):
        solvergpu.solver_gpu_fdtd(dev2, sce2, "gpu-fdtd-3lvl-cvr-rodr-fp32")


def _mixed_3lvl():
    """A 0-D run, 1-D runs of very different lengths and step counts, and a
    two-point run, all 3-level."""
    return [("song2005", dict(num_timesteps=3000)),
            ("lambda_3lvl", dict(num_gridpoints=2000, num_timesteps=1500)),
            ("random_nlvl", dict(N=3, num_gridpoints=500, num_timesteps=800,
                                 seed=4)),
            ("random_nlvl", dict(N=3, num_gridpoints=2, num_timesteps=300,
                                 seed=5))]


@pytest.mark.parametrize("algo", ["cvr-rodr", "reg-cayley"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_mixed_ensemble_equals_single_runs(native, algo, prec):
    """Runs of every shape in one launch sequence give exactly the single
    runs' results (and, in FP64, the oracle's). Both sides run the same
    tuning: FP32 Cayley renormalises the trace once per launch, so its
    results follow the launch depth wherever the trace has drifted (the
    autotuner may pick different depths for the ensemble and a single
    run)."""
    from mbsolve_gb300 import ensemble
    name = "gpu-fdtd-3lvl-%s-%s" % (algo, prec)
    specs = _mixed_3lvl()
    t = helpers.tuning(1, 128, 8, 2)
    mb.material.clear_library()
    pairs = [helpers.build_setup({"setup": s, "kw": kw}) for s, kw in specs]
    ens = ensemble.ensemble(name, pairs, t)
    ens.run()
    assert ens.status() == 0
    for i, (s, kw) in enumerate(specs):
        mb.material.clear_library()
        dev, sce = helpers.build_setup({"setup": s, "kw": kw})
        _, single = helpers.gpu_results(name, dev, sce, t)
        got = [r.as_array() for r in ens.results(i)]
        for a, b in zip(got, single):
            assert np.array_equal(a, b), (s, i)
        if prec == "fp64":
            mb.material.clear_library()
            dev, sce = helpers.build_setup({"setup": s, "kw": kw})
            _, orc = helpers.oracle_results(algo, 3, dev, sce)
            for a, b in zip(got, orc):
                _check(a, b, 1e-9, ("mixed", s, i))
