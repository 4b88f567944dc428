"""The engine's FP64 precompute (host instantiation of the code the GPU
runs) against the oracle: one step of the plane-basis update equals one
step of the reference's dense Rodrigues update; the Cayley constants are
the closed forms. CPU only."""
import ctypes as C
import math

import numpy as np
import pytest
import scipy.linalg

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers


def _constants(native, algo, mat, dt):
    from mbsolve_gb300 import _native
    n = C.c_size_t()
    _native.check(native.mbg_material_constants(algo.encode(), C.byref(mat),
                                                dt, 0, None, 0, C.byref(n)))
    out = np.zeros(n.value)
    _native.check(native.mbg_material_constants(
        algo.encode(), C.byref(mat), dt, 0, out.ctypes.data_as(T.PD),
        out.size, C.byref(n)))
    return out


@pytest.mark.parametrize("N,seed", [(2, 0), (3, 1), (4, 2), (5, 3), (6, 4)])
def test_plane_basis_step_equals_dense_rodrigues(native, N, seed):
    from mbsolve_gb300 import _native
    from oracle import oracle as O
    dev, sce = setups.random_nlvl(N=N, num_gridpoints=16, num_timesteps=10,
                                  seed=seed)
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    dt = 2.5e-17
    L = _native.material_layout("cvr-rodr", N)
    V = L["V"]
    c = _constants(native, "cvr-rodr", mat, dt)
    Q = c[L["Q"]:L["Q"] + V * V].reshape(V, V)
    np.testing.assert_allclose(Q.T @ Q, np.eye(V), atol=1e-12)
    rng = np.random.default_rng(seed)
    for e in (0.0, 3e7, -8e8):
        o = O.rodr_constants(mat.qm.contents, dt, e * dt)
        d = rng.normal(size=V) * 0.3
        # reference update (algo_lindblad_cvr_rodr.hpp:234-268)
        d1 = o["A1"] @ (d + o["d_in"]) - o["d_in"]
        d2 = o["A2"] @ d1
        dr = o["A1"] @ (d2 + o["d_in"]) - o["d_in"]
        pr = o["M_CP"] * o["v"] @ (o["M"] @ dr + o["d_eq"])
        # plane-basis update of the engine
        dg, pg = helpers.plane_basis_step(c, L, d, e)
        np.testing.assert_allclose(dg, dr, rtol=0, atol=1e-12)
        assert abs(pg - pr) <= 1e-10 * max(1.0, abs(pr)) + 1e-6 * abs(
            o["M_CP"] * o["v"] @ (np.abs(o["M"]) @ np.abs(dr)))
    # the low words are the FP32 rounding errors of Bd
    Bd = c[L["Bd"]:L["Bd"] + V * V]
    Bdl = c[L["Bdl"]:L["Bdl"] + V * V]
    np.testing.assert_array_equal(Bd - Bd.astype(np.float32).astype(np.float64), Bdl)
    # the full step the kernels apply is two half steps: I + Bd = (I + Bh)^2
    # and k = (I + Bh) kh + kh
    Bh = c[L["Bh"]:L["Bh"] + V * V].reshape(V, V)
    kh = c[L["kh"]:L["kh"] + V]
    A = np.eye(V) + Bh
    np.testing.assert_allclose(Bd.reshape(V, V), A @ A - np.eye(V), rtol=0,
                               atol=1e-14)
    np.testing.assert_allclose(c[L["k"]:L["k"] + V], A @ kh + kh, rtol=0,
                               atol=1e-14 * max(1.0, np.abs(kh).max()))
    # observables act on the kernels' state v = (I + Bh) u + kh: inversion
    # is d[N(N-1)], populations are the reference's rho_mm
    d = rng.normal(size=V)
    u = Q.T @ d
    v = A @ u + kh
    inv = c[L["inv"]:L["inv"] + V] @ v + c[L["inv_c"]]
    assert abs(inv - d[N * (N - 1)]) < 1e-12
    pops = np.array([c[L["pop"] + m * V:L["pop"] + (m + 1) * V] @ v
                     + c[L["pop_c"] + m] for m in range(N)])
    assert abs(pops.sum() - 1.0) < 1e-12
    # the initial state is v0 = (I + Bh) u0 + kh with u0 = Q^T d0, and d0
    # gives the initial populations of the scenario's density matrix
    v0 = c[L["u0"]:L["u0"] + V]
    u0 = np.linalg.solve(A, v0 - kh)
    pop0 = np.array([c[L["pop"] + m * V:L["pop"] + (m + 1) * V] @ v0
                     + c[L["pop_c"] + m] for m in range(N)])
    np.testing.assert_allclose(pop0.sum(), 1.0, atol=1e-12)
    assert np.isfinite(u0).all()


def test_cayley_constants(native):
    from mbsolve_gb300 import _native
    dev, sce = setups.random_nlvl(N=3, num_gridpoints=16, num_timesteps=10,
                                  seed=7)
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    dt = 2.5e-17
    L = _native.material_layout("reg-cayley", 3)
    c = _constants(native, "reg-cayley", mat, dt)
    qm = mb.material.get_from_library(dev.get_used_materials()[0]).get_qm()
    S = np.array(qm.get_relaxation_superop().get_scattering_rates())
    dD1 = c[L["dD1"]:L["dD1"] + 9].reshape(3, 3)
    np.testing.assert_allclose(dD1, scipy.linalg.expm(S * dt / 2) - np.eye(3),
                               rtol=1e-9, atol=1e-20)
    deph = qm.get_relaxation_superop().get_dephasing_rates()
    np.testing.assert_allclose(c[L["dD2"]:L["dD2"] + 3],
                               np.expm1(np.array(deph) * dt / 2), rtol=1e-12)
    kappa = dt / (2 * mb.HBAR)
    hd = qm.get_hamiltonian().get_main_diagonal()
    np.testing.assert_allclose(c[L["kH0"]:L["kH0"] + 3], np.array(hd) * kappa,
                               rtol=1e-14)


def test_level_mismatch_is_rejected(native):
    from mbsolve_gb300 import _native
    dev, sce = setups.random_nlvl(N=3, num_gridpoints=16, num_timesteps=10)
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    n = C.c_size_t()
    # the engine derives N from the material; a 3-level material asked for
    # as Cayley works, a wrong relaxation kind is rejected
    mat.qm.contents.relax_kind = T.MBG_RELAX_NONE
    rc = native.mbg_material_constants(b"reg-cayley", C.byref(mat), 1e-17, 0,
                                       None, 0, C.byref(n))
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert b"Unsupported superoperator" in native.mbg_last_error()


@pytest.mark.parametrize("N", [2, 3, 5])
def test_cayley_polarisation_weights(native, N):
    """P = Re tr((-i [W0, rho] + D'(rho)) Mn) (reg_cayley.hpp:258-267) is
    linear in the packed density matrix; the precomputed weights gP equal
    the formula evaluated on each packed basis element, and give P of a
    random density matrix."""
    from mbsolve_gb300 import _native
    dev, sce = setups.random_nlvl(N=N, num_gridpoints=16, num_timesteps=10,
                                  seed=11)
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    L = _native.material_layout("reg-cayley", N)
    c = _constants(native, "reg-cayley", mat, 2.5e-17)
    pairs = [(j, k) for k in range(N) for j in range(k)]

    def full(p):
        m = np.diag(p[:N]).astype(complex)
        for q, (j, k) in enumerate(pairs):
            m[j, k] = p[N + 2 * q] + 1j * p[N + 2 * q + 1]
            m[k, j] = np.conj(m[j, k])
        return m

    W = full(c[L["W0"]:L["W0"] + N * N])
    Mn = full(c[L["Mn"]:L["Mn"] + N * N])
    d1 = c[L["d1"]:L["d1"] + N * N].reshape(N, N)
    d2 = c[L["d2"]:L["d2"] + len(pairs)]

    def P(r):
        rho = full(r)
        rhs = -1j * (W @ rho - rho @ W)
        rhs += np.diag(d1 @ np.real(np.diag(rho)))
        for q, (j, k) in enumerate(pairs):
            rhs[j, k] += d2[q] * rho[j, k]
            rhs[k, j] += d2[q] * rho[k, j]
        return np.real(np.trace(rhs @ Mn))

    g = c[L["gP"]:L["gP"] + N * N]
    want = np.array([P(np.eye(N * N)[i]) for i in range(N * N)])
    np.testing.assert_allclose(g, want, rtol=1e-12, atol=1e-12 * np.abs(want).max())
    r = np.random.default_rng(1).normal(size=N * N)
    assert g @ r == pytest.approx(P(r), rel=1e-12)


@pytest.mark.parametrize("N,seed", [(2, 0), (3, 1), (4, 2), (6, 4)])
def test_cayley_split_step_equals_reference_step(native, N, seed):
    """The FP32 kernels' form of the Cayley step, rho + B0 rho + D(E(D
    rho)) with E = Z (U0 + dU)^H + U0 Z^H, Z = dU D(rho),
    dU = 2 i e A(e)^-1 W, equals the reference's step D(U2 D(rho) U2^H)
    (algo_lindblad_reg_cayley.hpp:228-257) in FP64, for zero and nonzero
    fields; B0l holds B0's FP32 rounding error."""
    from mbsolve_gb300 import _native
    dev, sce = setups.random_nlvl(N=N, num_gridpoints=16, num_timesteps=10,
                                  seed=seed)
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    L = _native.material_layout("reg-cayley", N)
    NN = N * N
    c = _constants(native, "reg-cayley", mat, 2.5e-17)
    pairs = [(j, k) for k in range(N) for j in range(k)]

    def full(p):
        m = np.diag(p[:N]).astype(complex)
        for q, (j, k) in enumerate(pairs):
            m[j, k] = p[N + 2 * q] + 1j * p[N + 2 * q + 1]
            m[k, j] = np.conj(m[j, k])
        return m

    def pack(m):
        out = np.zeros(NN)
        out[:N] = np.real(np.diag(m))
        for q, (j, k) in enumerate(pairs):
            out[N + 2 * q] = m[j, k].real
            out[N + 2 * q + 1] = m[j, k].imag
        return out

    K0 = full(c[L["kH0"]:L["kH0"] + NN])
    K1 = full(c[L["kMu"]:L["kMu"] + NN])
    dD1 = c[L["dD1"]:L["dD1"] + NN].reshape(N, N)
    dD2 = c[L["dD2"]:L["dD2"] + len(pairs)]

    def D(r):
        o = r.copy()
        o[:N] += dD1 @ r[:N]
        for q in range(len(pairs)):
            o[N + 2 * q:N + 2 * q + 2] *= 1.0 + dD2[q]
        return o

    def cmat(o):
        return (c[o:o + NN] + 1j * c[o + NN:o + 2 * NN]).reshape(N, N)

    U0 = cmat(L["U0"])
    Wk = cmat(L["Wk"])
    NP = L["NP"]
    B0 = c[L["B0"]:L["B0"] + NN * NP].reshape(NN, NP)[:, :NN]
    B0l = c[L["B0l"]:L["B0l"] + NN * NP].reshape(NN, NP)[:, :NN]
    np.testing.assert_array_equal(B0l, B0 - B0.astype(np.float32))
    I = np.eye(N)
    rng = np.random.default_rng(seed)
    for e in (0.0, 4e7, -9e8):
        a = rng.normal(size=(N, N)) + 1j * rng.normal(size=(N, N))
        rho = a @ a.conj().T
        rho /= np.trace(rho).real
        r = pack(rho)
        K = K0 - e * K1
        U2 = np.linalg.solve(I + 1j * K, I - 1j * K)
        want = D(pack(U2 @ full(D(r)) @ U2.conj().T))
        A = I + 1j * K
        dU = 2j * e * np.linalg.solve(A, Wk)
        np.testing.assert_allclose(U0 + dU, U2, rtol=0, atol=1e-14)
        Z = dU @ full(D(r))
        E = Z @ (U0 + dU).conj().T + U0 @ Z.conj().T
        got = r + B0 @ r + D(pack(E))
        np.testing.assert_allclose(got, want, rtol=0, atol=1e-14)


@pytest.mark.parametrize("setup,kw", [
    ("lambda_3lvl", dict(num_gridpoints=16, num_timesteps=10)),
    ("marskar2011", dict(N=5, num_gridpoints=16, endtime=1e-13)),
    ("random_nlvl", dict(N=3, num_gridpoints=16, num_timesteps=10))])
def test_cayley_block_structure_flag(native, setup, kw):
    """With a diagonal H0 the field-free matrix B0 is block-diagonal, its
    other entries exactly zero, and the block flag is set (the kernels then
    skip those zeros); a Hamiltonian with couplings keeps the dense path."""
    from mbsolve_gb300 import _native
    dev, sce = helpers.build_setup({"setup": setup, "kw": kw})
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    N = mat.qm.contents.num_levels
    L = _native.material_layout("reg-cayley", N)
    c = _constants(native, "reg-cayley", mat, 2.5e-17)
    NN, NP = N * N, L["NP"]
    B0 = c[L["B0"]:L["B0"] + NN * NP].reshape(NN, NP)[:, :NN]
    mask = np.zeros((NN, NN), bool)
    mask[:N, :N] = True
    for q in range((NN - N) // 2):
        mask[N + 2 * q:N + 2 * q + 2, N + 2 * q:N + 2 * q + 2] = True
    diag = setup != "random_nlvl"
    assert c[L["blockB0"]] == (1.0 if diag else 0.0)
    if diag:
        assert np.all(B0[~mask] == 0.0)
    else:
        assert np.any(B0[~mask] != 0.0)


def _cvr2_zeros(block, L):
    """The entries that the 2-level pair kernel's sparse variant skips
    (cvr2_sparse in pair_steps.cuh), as FP32 values."""
    V = L["V"]
    Bd = block[L["Bd"]:L["Bd"] + V * V].reshape(V, V).astype(np.float32)
    Bdl = block[L["Bdl"]:L["Bdl"] + V * V].reshape(V, V).astype(np.float32)
    g = block[L["g"]:L["g"] + V].astype(np.float32)
    idx = [(0, 1), (1, 0), (1, 2), (2, 1)]
    return [Bd[i] for i in idx] + [Bdl[i] for i in idx] + [g[1]]


def test_two_level_presets_take_the_sparse_pair_update(native):
    """The benchmark's 2-level media (diagonal Hamiltonian, real dipole)
    give blocks with the exact zeros that let the pair kernel skip 10
    products per pair; a random 2-level medium (off-diagonal Hamiltonian,
    complex dipole) has none of them, so the GPU tests that use it run the
    general variant."""
    from mbsolve_gb300 import _native
    L = _native.material_layout("cvr-rodr", 2)
    runs, _ = setups.ensemble_2lvl(num_runs=8, num_timesteps=100, seed=0)
    runs.append(setups.sit_2lvl(num_gridpoints=64, num_timesteps=10))
    runs.append(setups.ziolkowski1995(num_gridpoints=256, endtime=1e-15))
    for dev, sce in runs:
        b = mb.to_pod(dev, sce)
        for i in range(b.device.num_materials):
            mat = b.device.materials[i]
            if not mat.qm:
                continue
            blk = _constants(native, "cvr-rodr", mat, 1.5e-17)
            assert all(v == 0.0 for v in _cvr2_zeros(blk, L))
    mb.material.clear_library()
    dev, sce = setups.random_nlvl(N=2, num_gridpoints=64, num_timesteps=10,
                                  seed=2)
    b = mb.to_pod(dev, sce)
    blk = _constants(native, "cvr-rodr", b.device.materials[0], 1.5e-17)
    assert all(v != 0.0 for v in _cvr2_zeros(blk, L))
