"""Coherence records (lib.coherence_record, mbg_record.coherence = 1): the
off-diagonal density matrix entry rho[row][col], real and imaginary part.

The reference leaves these records zero (solver_cpu_fdtd.tpp:314-318, and a
`d12` record of this package still does); they are built beside it:

- a plain density record of an off-diagonal entry stays zero (oracle);
- pinned without the oracle's own formula: an undamped 2-level point
  driven by a pulse stays a pure state, 4 |rho_12|^2 + w^2 = 1 (w the
  inversion), and the coherence-vector and Cayley oracles, two different
  state representations, record the same rho_jk; rho_kj is the conjugate;
- the engine's precomputed record rows give rho_jk from the kernels'
  state (CPU, host instantiation of the GPU precompute);
- the GPU solvers equal the oracle (FP64 1e-9, FP32 1e-5), 2 to 6
  levels, tensor-core path included.
"""
import ctypes as C
import math

import numpy as np
import pytest

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

F0 = 2e14
BETA = 2.0 * math.acosh(2.0) / 100e-15
D_M = 6.24e-11


def _rabi(area=0.5 * math.pi):
    """Undamped 2-level point, resonant sech pulse of the given area."""
    mb.material.clear_library()
    qm = mb.qm_desc_2lvl(1e24, 2 * math.pi * F0, D_M, 0.0, 0.0, -1.0)
    ar = setups._material("AR_coh", qm)
    dev = mb.device("coh")
    dev.add_region(mb.region("Active region (single point)", ar, 0, 0))
    phase = 12.0
    sce = mb.scenario("coh", 1, 2 * phase / BETA,
                      mb.ic_density_const(mb.qm_operator([1, 0])),
                      mb.ic_field_const(0.0), mb.ic_field_const(0.0), 20000)
    ampl = area * mb.HBAR * BETA / (math.pi * mb.E0 * D_M)
    sce.add_source(mb.sech_pulse("sech", 0.0, mb.source.hard_source, ampl,
                                 F0, phase, BETA))
    sce.add_record(mb.record("inv12", 0.0))
    sce.add_record(mb.coherence_record("d12", 1, 2, 0.0, 0.0))
    sce.add_record(mb.coherence_record("d21", 2, 1, 0.0, 0.0))
    sce.add_record(mb.record("d12", mb.record.density, 1, 2, 0.0, 0.0))
    return dev, sce


def _song(n_t=3000):
    mb.material.clear_library()
    dev, sce = setups.song2005(num_timesteps=n_t)
    for j, k in ((1, 2), (1, 3), (3, 2)):
        sce.add_record(mb.coherence_record("d%d%d" % (j, k), j, k, 0.0, 0.0))
    return dev, sce


def _complex(dev, sce, algo, N):
    from oracle import oracle as O
    o = O.OracleRun(algo, N, mb.to_pod(dev, sce))
    o.run(threads=2)
    return [r + 1j * i if i is not None else r + 0j for r, i in o.results()]


@pytest.mark.parametrize("algo", ["cvr-rodr", "reg-cayley"])
def test_oracle_coherence_of_a_pure_state(algo):
    dev, sce = _rabi()
    inv, d12, d21, plain = _complex(dev, sce, algo, 2)
    w = inv.real[:, 0]
    r = d12[:, 0]
    assert np.abs(plain).max() == 0.0                # the reference's record
    # the reference's Cayley form keeps the full matrix, whose Hermiticity
    # drifts at the rounding level (4.5e-15 over this run)
    assert np.abs(d21[:, 0] - np.conj(r)).max() < 1e-13
    assert np.abs(r).max() > 0.4                     # the pulse made coherence
    assert np.abs(4 * np.abs(r) ** 2 + w ** 2 - 1.0).max() < 1e-9


def test_oracle_coherence_vector_and_cayley_agree():
    """The two propagators differ at the discretisation level (second
    order in dt: 2.3e-3 apart with 3,000 steps over the 80 fs, 2e-5 with
    100,000); a wrong
    convention (index order, sign of the imaginary part) would be O(1)."""
    recs = {a: _complex(*_song(100000), a, 3)
            for a in ("cvr-rodr", "reg-cayley")}
    for k in range(len(recs["cvr-rodr"])):
        a, b = recs["cvr-rodr"][k], recs["reg-cayley"][k]
        assert np.abs(a).max() > 1e-3
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err < 1e-4, (k, err)


@pytest.mark.parametrize("N,seed", [(2, 0), (3, 1), (6, 4)])
def test_engine_coherence_rows(native, N, seed):
    """rho[j][k] = (d_u - i d_v)/2 (u_jk, v_jk the generators of
    coherence_vector_representation.hpp:52-93) from the record rows on the
    kernels' state v = (I + Bh) Q^T d + kh."""
    from mbsolve_gb300 import _native
    dev, sce = setups.random_nlvl(N=N, num_gridpoints=16, num_timesteps=10,
                                  seed=seed)
    mat = mb.to_pod(dev, sce).device.materials[0]
    L = _native.material_layout("cvr-rodr", N)
    n = C.c_size_t()
    _native.check(native.mbg_material_constants(
        b"cvr-rodr", C.byref(mat), 2.5e-17, 0, None, 0, C.byref(n)))
    c = np.zeros(n.value)
    _native.check(native.mbg_material_constants(
        b"cvr-rodr", C.byref(mat), 2.5e-17, 0, c.ctypes.data_as(T.PD),
        c.size, C.byref(n)))
    V = L["V"]
    P = N * (N - 1) // 2
    Q = c[L["Q"]:L["Q"] + V * V].reshape(V, V)
    Bh = c[L["Bh"]:L["Bh"] + V * V].reshape(V, V)
    kh = c[L["kh"]:L["kh"] + V]
    d = np.random.default_rng(seed).normal(size=V)
    v = (np.eye(V) + Bh) @ (Q.T @ d) + kh
    for k in range(1, N):
        for j in range(k):
            q = k * (k - 1) // 2 + j
            want = 0.5 * (d[q] - 1j * d[P + q])
            re = c[L["coh"] + 2 * q * V:L["coh"] + (2 * q + 1) * V] @ v \
                + c[L["coh_c"] + 2 * q]
            im = c[L["coh"] + (2 * q + 1) * V:L["coh"] + (2 * q + 2) * V] @ v \
                + c[L["coh_c"] + 2 * q + 1]
            assert abs(re + 1j * im - want) < 1e-12


def _gpu_complex(name, dev, sce):
    from mbsolve_gb300 import solvergpu
    s = solvergpu.solver_gpu_fdtd(dev, sce, name)
    s.run()
    return [np.asarray(r.get_data_complex()).reshape(r.get_rows(),
                                                     r.get_cols())
            for r in s.get_results()]


def _random_case(N, seed):
    mb.material.clear_library()
    dev, sce = setups.random_nlvl(N=N, num_gridpoints=512, num_timesteps=800,
                                  seed=seed, e_seed=3e7)
    L = dev.get_length()
    for j, k in ((1, 2), (2, 1), (1, N), (N - 1, N)):
        sce.add_record(mb.coherence_record("d%d%d" % (j, k), j, k, 0.0,
                                           L / 2))
    sce.add_record(mb.coherence_record("d12all", 1, 2, 8 * 1.5e-17, -1.0))
    return dev, sce


@pytest.mark.gpu
@pytest.mark.parametrize("algo,N", [("cvr-rodr", 2), ("cvr-rodr", 3),
                                    ("cvr-rodr", 6), ("reg-cayley", 3),
                                    ("reg-cayley", 5)])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_coherence_matches_oracle(native, algo, N, prec):
    tol = 1e-9 if prec == "fp64" else 1e-5
    ref = _complex(*_random_case(N, 10 + N), algo, N)
    got = _gpu_complex("gpu-fdtd-%dlvl-%s-%s" % (N, algo, prec),
                       *_random_case(N, 10 + N))
    assert len(got) == len(ref)
    for k, (a, b) in enumerate(zip(got, ref)):
        assert a.shape == b.shape
        if k >= 1:
            assert np.abs(b.imag).max() > 0, k       # complex entries
        assert helpers.rel_err(a.real, b.real) <= tol, (k, "re")
        if k >= 1:
            assert helpers.rel_err(a.imag, b.imag) <= tol, (k, "im")


@pytest.mark.gpu
def test_gpu_plain_offdiagonal_record_stays_zero(native):
    dev, sce = _rabi()
    got = _gpu_complex("gpu-fdtd-2lvl-cvr-rodr-fp64", dev, sce)
    assert np.abs(got[3]).max() == 0.0
    assert np.abs(got[1]).max() > 0.4


@pytest.mark.gpu
@pytest.mark.parametrize("algo,prec,tol", [
    ("cvr-rodr", "fp64", 1e-9), ("reg-cayley", "fp64", 1e-9),
    ("cvr-rodr", "fp32", 2e-5), ("reg-cayley", "fp32", 1e-4)])
def test_gpu_bloch_norm_drift(native, algo, prec, tol):
    """Bloch-norm drift of an undamped 2-level point over a pulse (20,000
    steps): |4 |rho_12|^2 + w^2 - 1|, zero for the exact pure state. The
    FP32 coherence vector is a float pair (measured below 2e-5); the FP32
    Cayley matrix is plain FP32, renormalised in trace only (measured
    2.9e-5)."""
    got = _gpu_complex("gpu-fdtd-2lvl-%s-%s" % (algo, prec), *_rabi())
    w = got[0].real[:, 0]
    r = got[1][:, 0]
    assert np.abs(r).max() > 0.4
    drift = np.abs(4 * np.abs(r) ** 2 + w ** 2 - 1.0).max()
    print(algo, prec, "Bloch-norm drift %.2e" % drift)
    assert drift < tol
