"""Pins the FP64 oracle: against golden vectors made by the reference's own
time loop (tests/golden, generated by make_golden.py from oracle/_ref),
against the reference-built library live (when the reference tree is
present), and its algebra against independent numpy/scipy constructions.
CPU only."""
import math

import numpy as np
import pytest
import scipy.linalg

from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

ALGO = {"cvr-rodr": "cvr-rodr", "reg-cayley": "reg-cayley", "noop": "noop"}


def _algo_levels(solver):
    # cpu-fdtd-{N}lvl-{algo} | cpu-fdtd-noop
    rest = solver[len("cpu-fdtd-"):]
    if rest == "noop":
        return "noop", 0
    return rest[5:], int(rest[0])


@pytest.mark.parametrize("case", helpers.golden_cases())
def test_oracle_matches_golden(case):
    meta, recs = helpers.load_golden(case)
    dev, sce = helpers.build_setup(meta["spec"])
    algo, n = _algo_levels(meta["solver"])
    grid, res = helpers.oracle_results(algo, n, dev, sce, threads=2)
    assert grid.num_timesteps == meta["num_timesteps"]
    assert grid.timestep_size == meta["timestep_size"]
    assert grid.gridpoint_size == meta["gridpoint_size"]
    for k, (a, b) in enumerate(zip(res, recs)):
        assert a.shape == b.shape
        # the oracle restates the reference's loop operation by operation
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * max(1.0, np.abs(b).max()))


def _ref_available():
    from oracle import oracle as O
    try:
        return O.ref_lib() is not None
    except Exception:
        return False


@pytest.mark.skipif(not _ref_available(), reason="reference tree not present")
@pytest.mark.parametrize("solver,setup,kw", [
    ("cpu-fdtd-2lvl-cvr-rodr", "tzenov2018_cpml",
     dict(num_gridpoints=512, endtime=3e-12)),
    ("cpu-fdtd-2lvl-reg-cayley", "tzenov2018_cpml",
     dict(num_gridpoints=512, endtime=3e-12)),
    ("cpu-fdtd-3lvl-cvr-rodr", "random_nlvl",
     dict(N=3, num_gridpoints=128, num_timesteps=300)),
    ("cpu-fdtd-4lvl-reg-cayley", "random_nlvl",
     dict(N=4, num_gridpoints=128, num_timesteps=300)),
    ("cpu-fdtd-2lvl-reg-cayley", "random_nlvl",
     dict(N=2, num_gridpoints=96, num_timesteps=300, e_seed=3e7)),
    ("cpu-fdtd-3lvl-reg-cayley", "random_nlvl",
     dict(N=3, num_gridpoints=96, num_timesteps=300, e_seed=3e7)),
    ("cpu-fdtd-4lvl-cvr-rodr", "random_nlvl",
     dict(N=4, num_gridpoints=96, num_timesteps=300, e_seed=3e7)),
    ("cpu-fdtd-5lvl-cvr-rodr", "random_nlvl",
     dict(N=5, num_gridpoints=64, num_timesteps=200, e_seed=3e7)),
    ("cpu-fdtd-5lvl-reg-cayley", "random_nlvl",
     dict(N=5, num_gridpoints=64, num_timesteps=200, e_seed=3e7)),
    ("cpu-fdtd-6lvl-cvr-rodr", "random_nlvl",
     dict(N=6, num_gridpoints=64, num_timesteps=200, e_seed=3e7)),
    ("cpu-fdtd-6lvl-reg-cayley", "random_nlvl",
     dict(N=6, num_gridpoints=64, num_timesteps=200, e_seed=3e7)),
])
def test_oracle_matches_reference_live(solver, setup, kw):
    """Fresh setups (random E initial field, two materials, H record at an
    interior point) through the reference's own solver_cpu_fdtd."""
    import os
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    spec = {"setup": setup, "kw": kw}
    dev, sce = helpers.build_setup(spec)
    if setup == "tzenov2018_cpml":
        sce.set_ic_electric(mb.ic_field_random(seed=3))
    algo, n = _algo_levels(solver)
    g1, ref = helpers.reference_results(solver, dev, sce)
    mb.material.clear_library()
    dev, sce2 = helpers.build_setup(spec)
    if setup == "tzenov2018_cpml":
        sce2.set_ic_electric(mb.ic_field_random(seed=3))
    g2, res = helpers.oracle_results(algo, n, dev, sce2, threads=3)
    assert g1.num_timesteps == g2.num_timesteps
    for a, b in zip(res, ref):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * max(1.0, np.abs(b).max()))


@pytest.mark.skipif(not _ref_available(), reason="reference tree not present")
@pytest.mark.parametrize("algo", ["cvr-rodr", "reg-cayley"])
def test_reference_plain_and_red_loops_agree(algo):
    """The reference's two CPU time loops, solver_cpu_fdtd and the
    temporally blocked solver_cpu_fdtd_red, give the same probe E bit for
    bit (the oracle restates the plain one; the CPU baseline times it)."""
    out = []
    for name in ("cpu-fdtd-2lvl-" + algo, "cpu-fdtd-red-2lvl-" + algo):
        mb.material.clear_library()
        dev, sce = helpers.build_setup(
            {"setup": "sit_2lvl", "kw": dict(num_gridpoints=1024,
                                             num_timesteps=3000)})
        _, r = helpers.reference_results(name, dev, sce)
        out.append(r[0])
    assert np.abs(out[0]).max() > 1.0
    assert np.array_equal(out[0], out[1])


# ---------------------------------------------- algebra vs numpy / scipy

def test_expm_matches_scipy():
    from oracle import oracle as O
    rng = np.random.default_rng(1)
    for n, scale in [(3, 0.01), (8, 0.3), (15, 2.0), (35, 7.0)]:
        a = rng.normal(size=(n, n)) * scale / math.sqrt(n)
        np.testing.assert_allclose(O.expm(a), scipy.linalg.expm(a),
                                   rtol=1e-12, atol=1e-13)


def _generators(N):
    """su(N) basis in the reference's order, built independently."""
    g = []
    for k in range(N):
        for j in range(k):
            m = np.zeros((N, N), complex)
            m[j, k] = m[k, j] = 1
            g.append(m)
    for k in range(N):
        for j in range(k):
            m = np.zeros((N, N), complex)
            m[j, k] = -1j
            m[k, j] = 1j
            g.append(m)
    for l in range(N - 1):
        m = np.zeros((N, N), complex)
        for j in range(l + 1):
            m[j, j] = -1
        m[l + 1, l + 1] = l + 1
        g.append(m / math.sqrt((l + 1) * (l + 2) / 2))
    return g


def _full(op, N):
    m = np.diag(np.array(op.get_main_diagonal()[:N], dtype=complex))
    i = 0
    for k in range(1, N):
        for j in range(k):
            m[j, k] = op.get_off_diagonal()[i]
            m[k, j] = np.conj(op.get_off_diagonal()[i])
            i += 1
    return m


@pytest.mark.parametrize("N", [2, 3, 4, 6])
def test_cvr_constants_are_the_lindblad_generator(N):
    """M d + d_eq is the coherence vector of the Lindblad right-hand side of
    rho(d) = I/N + 1/2 sum d_j g_j (without the field), and U is the
    dipole term's generator: d/dt d = (M + E U) d + d_eq."""
    from oracle import oracle as O
    dev, sce = setups.random_nlvl(N=N, num_gridpoints=16, num_timesteps=10,
                                  seed=N)
    b = mb.to_pod(dev, sce)
    qpod = b.device.materials[0].qm.contents
    qm = mb.material.get_from_library(dev.get_used_materials()[0]).get_qm()
    c = O.rodr_constants(qpod, 1e-16, 1e-6)
    H = _full(qm.get_hamiltonian(), N)
    mu = _full(qm.get_dipole_operator(), N)
    relax = qm.get_relaxation_superop()
    S = np.array(relax.get_scattering_rates())
    D = relax.get_dephasing_rates()

    def R(rho):
        out = np.diag(S @ np.diag(rho).real).astype(complex)
        i = 0
        for k in range(1, N):
            for j in range(k):
                out[j, k] = rho[j, k] * D[i]
                out[k, j] = np.conj(out[j, k])
                i += 1
        return out

    g = _generators(N)
    V = N * N - 1
    HB = mb.HBAR
    for j in range(V):
        rho = 0.5 * g[j]
        rhs = -1j / HB * (H @ rho - rho @ H) + R(rho)
        dip = -1j / HB * (-(mu @ rho - rho @ mu))  # field term per unit E
        for i in range(V):
            assert abs(np.trace(g[i] @ rhs).real - c["M"][i, j]) <= \
                1e-9 * np.abs(c["M"]).max()
            assert abs(np.trace(g[i] @ dip).real - c["U"][i, j]) <= \
                1e-9 * np.abs(c["U"]).max() + 1e-300
    eq = R(np.eye(N) / N)
    for i in range(V):
        assert abs(np.trace(g[i] @ eq).real - c["d_eq"][i]) <= \
            1e-9 * max(1.0, np.abs(c["d_eq"]).max())
        assert abs(np.trace(mu @ g[i]).real - c["v"][i]) <= 1e-40
    # the Rodrigues sum over Schur planes is exp(probe U) exactly
    np.testing.assert_allclose(c["A2"], scipy.linalg.expm(1e-6 * c["U"]),
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(c["A1"], scipy.linalg.expm(c["M"] * 1e-16 / 2),
                               rtol=0, atol=1e-13)


# ----------------------------- grid derivation (tests_common_fdtd.cpp)

def _grid_cases():
    L = 1e-3
    return [
        # zero device length, zero end time (tests_common_fdtd.cpp:30-49)
        dict(length=0.0, n_x=1, t_e=0.0, n_t=2,
             expect=dict(n_t=1, dt=3.154e10, dx=1e13)),
        # zero device length, nonzero end time (:51-72)
        dict(length=0.0, n_x=1, t_e=1e-9, n_t=10000,
             expect=dict(n_t=10000, dt=1e-9 / 9999, dx=1e13)),
        # nonzero length, zero end time (:74-98)
        dict(length=L, n_x=32768, t_e=0.0, n_t=12345,
             expect=dict(n_t=1, dt=3.154e10, dx=L / 32767)),
    ]


def _grid_device(length, n_x, t_e, n_t):
    mat = mb.material("Vacuum")
    mb.material.add_to_library(mat)
    dev = mb.device("dut")
    if length > 0:
        dev.add_region(mb.region("rut", mat, 0, length))
    else:
        dev.add_region(mb.region("rut", mat, 0, 0))
    sce = mb.scenario("test", n_x, t_e, mb.qm_operator([1, 0]), n_t)
    sce.set_ic_electric(mb.ic_field_const(0.0))
    return dev, sce


@pytest.mark.parametrize("case", range(3))
def test_grid_derivation_reference_cases(case):
    from oracle import oracle as O
    c = _grid_cases()[case]
    dev, sce = _grid_device(c["length"], c["n_x"], c["t_e"], c["n_t"])
    o = O.OracleRun("noop", 0, mb.to_pod(dev, sce))
    g = o.grid()
    e = c["expect"]
    assert g.num_timesteps == e["n_t"]
    assert g.timestep_size == pytest.approx(e["dt"], rel=1e-12)
    assert g.gridpoint_size == pytest.approx(e["dx"], rel=1e-12)


def test_grid_derivation_nonzero_length_and_time():
    """tests_common_fdtd.cpp:100-126 at Courant 1 there; solvers use 0.5."""
    from oracle import oracle as O
    L, t_e, n_x = 1e-3, 1e-9, 32768
    dev, sce = _grid_device(L, n_x, t_e, 12345)
    g = O.OracleRun("noop", 0, mb.to_pod(dev, sce)).grid()
    d_x = L / (n_x - 1)
    d_t = 0.5 * d_x * math.sqrt(mb.MU0 * mb.EPS0)
    n_t = math.ceil(t_e / d_t) + 1
    assert g.num_timesteps == n_t
    assert g.timestep_size == pytest.approx(t_e / (n_t - 1), rel=1e-12)
    assert g.gridpoint_size == pytest.approx(d_x, rel=1e-12)


@pytest.mark.parametrize("spec,algo,N", [
    ({"setup": "sit_2lvl", "kw": dict(num_gridpoints=2000, num_timesteps=500)},
     "cvr-rodr", 2),
    ({"setup": "ziolkowski1995", "kw": dict(num_gridpoints=1024,
                                            endtime=40e-15)}, "cvr-rodr", 2),
    ({"setup": "ziolkowski1995", "kw": dict(num_gridpoints=1024,
                                            endtime=40e-15)}, "noop", 0),
    ({"setup": "lambda_3lvl", "kw": dict(num_gridpoints=600,
                                         num_timesteps=300)}, "reg-cayley", 3),
    ({"setup": "random_nlvl", "kw": dict(N=4, num_gridpoints=700,
                                         num_timesteps=203, e_seed=3e7)},
     "cvr-rodr", 4),
])
@pytest.mark.parametrize("threads", [1, 3])
def test_blocked_loop_equals_plain_loop(spec, algo, N, threads):
    """The oracle's restatement of solver_cpu_fdtd_red (thread-private
    ranges with 8-step overlaps) gives solver_cpu_fdtd's results bit for
    bit, sources, records and boundaries included, with any step count
    (not a multiple of the overlap) and any thread count."""
    from oracle import oracle as O
    out = []
    for red in (0, 8):
        mb.material.clear_library()
        dev, sce = helpers.build_setup(spec)
        if spec["setup"] == "ziolkowski1995":
            sce.add_record(mb.record("h", mb.record.magnetic, 0, 0, 0.0, -1.0))
        o = O.OracleRun(algo, N, mb.to_pod(dev, sce))
        o.run(threads=threads, red=red)
        o.run(threads=threads, max_steps=37, red=red)   # continues
        out.append([r for r, _ in o.results()])
    for a, b in zip(*out):
        assert np.array_equal(a, b)
