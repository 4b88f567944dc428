"""Pins the surrogate's CPU oracle (oracle/fno_oracle.py) before it is used
to check the GPU network: BF16 rounding against torch's, the truncated DFT
bases against numpy's FFT, the real block form against complex arithmetic,
and the hand-derived backward pass against central finite differences."""
import math

import numpy as np
import pytest

from oracle import fno_oracle as O


def test_bf16_round_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(0).normal(size=10000) * \
        np.exp(np.random.default_rng(1).uniform(-20, 20, size=10000))
    x = np.concatenate([x, [0.0, -0.0, 1.0, 1.00390625, 1.005859375,
                            3.4e38, -1e-40]])
    want = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16) \
        .to(torch.float64).numpy()
    np.testing.assert_array_equal(O.bf16_round(x), want)


def test_dft_bases_against_numpy_fft():
    S, Mo = 64, 8
    F, G = O.dft_bases(S, Mo)
    x = np.random.default_rng(2).normal(size=S)
    X = np.fft.rfft(x)[:Mo] / S
    z = F @ x
    np.testing.assert_allclose(z[:Mo], X.real, atol=1e-14)
    np.testing.assert_allclose(z[Mo:], X.imag, atol=1e-14)
    spec = np.zeros(S // 2 + 1, dtype=complex)
    spec[:Mo] = np.fft.rfft(x)[:Mo]
    np.testing.assert_allclose(G @ z, np.fft.irfft(spec, n=S), atol=1e-13)


def test_mode_blocks_are_complex_products():
    rng = np.random.default_rng(3)
    Mo, W = 3, 5
    wr, wi = rng.normal(size=(Mo, W, W)), rng.normal(size=(Mo, W, W))
    x = rng.normal(size=(Mo, W)) + 1j * rng.normal(size=(Mo, W))
    blk = O.mode_blocks(wr, wi)
    for m in range(Mo):
        y = x[m] @ (wr[m] + 1j * wi[m])       # y_o = sum_c w[c, o] x_c
        r = blk[m] @ np.concatenate([x[m].real, x[m].imag])
        np.testing.assert_allclose(r, np.concatenate([y.real, y.imag]),
                                   atol=1e-12)


def test_backward_matches_finite_differences():
    sh = O.Shapes(S=32, W=8, Mo=4, L=2, F=8, Hq=16)
    rng = np.random.default_rng(4)
    theta = O.init_params(sh, seed=5)
    X = rng.normal(size=(2, sh.S, sh.F))
    t = rng.normal(size=(2, sh.S))
    loss, grad, _ = O.forward_backward(sh, theta, X, t)
    eps = 1e-6
    for trial in range(6):
        u = rng.normal(size=theta.size)
        lp = O.forward_backward(sh, theta + eps * u, X, t)[0]
        lm = O.forward_backward(sh, theta - eps * u, X, t)[0]
        fd = (lp - lm) / (2 * eps)
        an = float(grad @ u)
        assert abs(fd - an) <= 1e-6 * max(abs(an), 1e-8), (fd, an)
    # every parameter block receives gradient
    p = O.unflatten(sh, grad)
    for name, _ in sh.param_spec():
        assert np.abs(p[name]).max() > 0, name


def test_bf16_mode_stays_close_to_float64():
    sh = O.Shapes(S=64, W=8, Mo=8, L=2, F=8, Hq=16)
    rng = np.random.default_rng(6)
    theta = O.init_params(sh, seed=7)
    X = rng.normal(size=(2, sh.S, sh.F))
    t = rng.normal(size=(2, sh.S))
    l64, g64, _ = O.forward_backward(sh, theta, X, t)
    l16, g16, _ = O.forward_backward(sh, theta, X, t, bf16=True)
    assert abs(l16 - l64) < 2e-2 * l64
    assert np.linalg.norm(g16 - g64) < 5e-2 * np.linalg.norm(g64)


def test_gelu_erf_formula_in_the_kernel_source():
    """The kernels' GELU evaluates erf by Abramowitz and Stegun 7.1.26; the
    constants as written in the CUDA source, evaluated in float64, keep
    |erf error| <= 1.5e-7 (the published bound) and the GELU error
    <= 0.5 |x| 1.5e-7 over -8..8 (the FP32 evaluation is checked on the
    GPU in tests/test_fno_gemm.py)."""
    import os
    import re
    path = os.path.join(os.path.dirname(__file__), "..", "mbsolve_gb300",
                        "csrc", "fno_common.cuh")
    src = open(path).read()
    body = src[src.index("float gelu(float x)"):]
    body = body[:body.index("\n}\n")]
    num = r"(-?\d+\.\d+)f"
    p = float(re.search(r"fmaf\(" + num + r", z, 1\.0f\)", body).group(1))
    first = re.search(r"fmaf\(t, " + num + r", " + num + r"\)", body)
    rest = [float(v) for v in re.findall(r"fmaf\(t, q, " + num + r"\)", body)]
    a = [rest[2], rest[1], rest[0], float(first.group(2)),
         float(first.group(1))]  # a1 .. a5
    assert p == 0.3275911 and len(rest) == 3
    z = np.linspace(0.0, 8.0 / math.sqrt(2.0), 20001)
    t = 1.0 / (1.0 + p * z)
    erfc = t * (a[0] + t * (a[1] + t * (a[2] + t * (a[3] + t * a[4])))) * \
        np.exp(-z * z)
    exact = np.array([math.erfc(v) for v in z])
    assert np.abs(erfc - exact).max() <= 1.5e-7
    x = z * math.sqrt(2.0)
    for s in (1.0, -1.0):
        xs = s * x
        got = np.where(xs < 0, 0.5 * xs * erfc, xs - 0.5 * xs * erfc)
        want = 0.5 * xs * (1.0 + np.array([math.erf(v / math.sqrt(2.0))
                                           for v in xs]))
        assert (np.abs(got - want) <= 0.5 * np.abs(xs) * 1.5e-7 + 1e-15).all()
