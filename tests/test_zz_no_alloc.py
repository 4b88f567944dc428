"""The allocation-free precompute entry point (mbg_material_constants_noalloc)
against the allocating one (mbg_material_constants on the device).

The no-alloc entry point serves callers that cannot call cudaMalloc (their
device memory belongs to another allocator, or their path cannot take the
synchronisation cudaMalloc implies): it writes into a device buffer the
caller owns and keeps its workspace in a fixed device array. This test owns
its output buffer (allocated here with torch, as such a caller's allocator
would), calls the entry point twice in a row plus once more for the first
material, in both forms (coherence vector and Cayley), and compares each
result with the existing entry point's. It also checks that both entry
points refuse the same bad materials with the same messages, including the
one the device reports through the fixed array's status slot.
Collected last so that a stop at the first failure has run every other
test first.
"""
import ctypes as C

import numpy as np
import pytest

from mbsolve_gb300 import capi_types as T
from mbsolve_gb300 import lib as mb
from mbsolve_gb300 import setups
from tests import helpers

pytestmark = pytest.mark.gpu


def _existing(native, mat, dt, algo=b"cvr-rodr"):
    from mbsolve_gb300 import _native
    n = C.c_size_t()
    _native.check(native.mbg_material_constants(algo, C.byref(mat), dt,
                                                1, None, 0, C.byref(n)))
    out = np.zeros(n.value)
    _native.check(native.mbg_material_constants(
        algo, C.byref(mat), dt, 1, out.ctypes.data_as(T.PD),
        out.size, C.byref(n)))
    return out


def _noalloc(native, mat, dt, algo=b"cvr-rodr"):
    import torch
    from mbsolve_gb300 import _native
    n = C.c_size_t()
    _native.check(native.mbg_material_constants_noalloc(
        algo, C.byref(mat), dt, None, 0, C.byref(n), None))
    buf = torch.full((n.value,), float("nan"), dtype=torch.float64,
                     device="cuda")
    torch.cuda.synchronize()
    _native.check(native.mbg_material_constants_noalloc(
        algo, C.byref(mat), dt, buf.data_ptr(), n.value, C.byref(n),
        None))
    return buf.cpu().numpy()


def test_noalloc_precompute_matches_allocating_entry_point(native):
    from mbsolve_gb300 import _native
    dt = 2.5e-17
    mats = []
    for N, seed in ((2, 0), (6, 4)):
        dev, sce = setups.random_nlvl(N=N, num_gridpoints=16,
                                      num_timesteps=10, seed=seed)
        b = mb.to_pod(dev, sce)
        mats.append((N, b, b.device.materials[0]))
    # two calls in a row (2 levels, then 6), then the first material again:
    # the shared workspace keeps the previous call's contents
    for N, b, mat in mats + mats[:1]:
        got = _noalloc(native, mat, dt)
        ref = _existing(native, mat, dt)
        assert not np.isnan(got).any()
        L = _native.material_layout("cvr-rodr", N)
        # same precompute code on the same device: equal within the
        # tolerance of the device-vs-host precompute test, compared through
        # what the constants compute (one plane-basis update)
        rng = np.random.default_rng(N)
        for e in (0.0, 2e8, -7e8):
            d = rng.normal(size=L["V"]) * 0.3
            dg, pg = helpers.plane_basis_step(got, L, d, e)
            dr, pr = helpers.plane_basis_step(ref, L, d, e)
            np.testing.assert_allclose(dg, dr, rtol=0, atol=1e-12)
            assert abs(pg - pr) <= 1e-8 * max(abs(pr), 1e10)
        np.testing.assert_allclose(got[:L["stage"]], ref[:L["stage"]],
                                   rtol=1e-12, atol=1e-300)


def test_noalloc_rejects_bad_requests(native):
    dev, sce = setups.random_nlvl(N=3, num_gridpoints=16, num_timesteps=10)
    b = mb.to_pod(dev, sce)
    mat = b.device.materials[0]
    n = C.c_size_t()
    # output buffer too small: refused before anything runs
    rc = native.mbg_material_constants_noalloc(b"cvr-rodr", C.byref(mat),
                                               1e-17, C.c_void_p(16), 3,
                                               C.byref(n), None)
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert b"needed" in native.mbg_last_error()
    # more levels than the fixed workspace serves
    mat.qm.contents.num_levels = 7
    rc = native.mbg_material_constants_noalloc(b"cvr-rodr", C.byref(mat),
                                               1e-17, None, 0, C.byref(n),
                                               None)
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert b"levels must be 2..6" in native.mbg_last_error()


def test_noalloc_cayley_matches_allocating_entry_point(native):
    """The Cayley branch (D1, D2, polarisation weights) through the fixed
    workspace: 3-level Lambda and 5-level ladder, twice in a row, then the
    first again."""
    dt = 1.5e-17
    mats = []
    for setup, kw in (("lambda_3lvl", dict(num_gridpoints=16,
                                           num_timesteps=10)),
                      ("marskar2011", dict(N=5, num_gridpoints=16,
                                           endtime=1e-13))):
        dev, sce = helpers.build_setup({"setup": setup, "kw": kw})
        b = mb.to_pod(dev, sce)
        mats.append((b, b.device.materials[0]))
    for b, mat in mats + mats[:1]:
        got = _noalloc(native, mat, dt, b"reg-cayley")
        ref = _existing(native, mat, dt, b"reg-cayley")
        assert not np.isnan(got).any()
        # no basis freedom in the Cayley constants: entry by entry
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-300)


def _material_pod(relax):
    H = mb.qm_operator([0.0, mb.HBAR * 1e15])
    u = mb.qm_operator([0.0, 0.0], [-mb.E0 * 1e-10])
    qm = mb.qm_description(1e24, H, u, relax)
    m = mb.material("noalloc-bad", qm)
    mb.material.add_to_library(m)
    dev = mb.device("d")
    dev.add_region(mb.region("a", m, 0, 1e-6))
    sce = mb.scenario("s", 16, 1e-15,
                      mb.ic_density_const(mb.qm_operator([1, 0])),
                      mb.ic_field_const(0.0))
    return mb.to_pod(dev, sce)


def _rc_msg(native, fn, algo, mat):
    n = C.c_size_t()
    if fn == "noalloc":
        import torch
        buf = torch.zeros(4096, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = native.mbg_material_constants_noalloc(
            algo, C.byref(mat), 2e-17, buf.data_ptr(), 4096, C.byref(n), None)
    else:
        out = np.zeros(4096)
        rc = native.mbg_material_constants(
            algo, C.byref(mat), 2e-17, 1, out.ctypes.data_as(T.PD), out.size,
            C.byref(n))
    return rc, native.mbg_last_error()


def test_noalloc_refuses_like_allocating_entry_point(native):
    # a scattering matrix with no steady state (a negative rate): the
    # precompute's d_in solve fails on the device and the status comes back
    # through the fixed array's status slot
    b = _material_pod(mb.qm_lindblad_relaxation([[0, 1e12], [-1e12, 0]],
                                                [0.0]))
    mat = b.device.materials[0]
    for fn in ("noalloc", "existing"):
        rc, msg = _rc_msg(native, fn, b"cvr-rodr", mat)
        assert rc == T.MBG_ERR_INVALID_ARGUMENT, (fn, msg)
        assert msg == b"Time-indepent matrix not invertible!", (fn, msg)
    # the Cayley form needs a Lindblad relaxation superoperator
    # (algo_lindblad_reg_cayley.hpp:150-155)
    mat.qm.contents.relax_kind = T.MBG_RELAX_NONE
    for fn in ("noalloc", "existing"):
        rc, msg = _rc_msg(native, fn, b"reg-cayley", mat)
        assert rc == T.MBG_ERR_INVALID_ARGUMENT, (fn, msg)
        assert msg == b"Unsupported superoperator!", (fn, msg)
    # the entry point still works after the refusals
    dev, sce = setups.random_nlvl(N=2, num_gridpoints=16, num_timesteps=10)
    good = mb.to_pod(dev, sce).device.materials[0]
    got = _noalloc(native, good, 2e-17)
    assert not np.isnan(got).any()


def test_noalloc_refuses_material_without_qm(native):
    """A material without a quantum-mechanical description has no constant
    block to compute here (the allocating entry point returns the vacuum
    block of its one-point device instead)."""
    b = _material_pod(mb.qm_lindblad_relaxation([[0, 1e9], [1e9, 0]], [0.0]))
    mat = b.device.materials[0]
    mat.qm = None
    n = C.c_size_t()
    rc = native.mbg_material_constants_noalloc(b"cvr-rodr", C.byref(mat),
                                               1e-17, None, 0, C.byref(n),
                                               None)
    assert rc == T.MBG_ERR_INVALID_ARGUMENT
    assert b"no quantum-mechanical description" in native.mbg_last_error()
