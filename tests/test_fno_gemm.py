"""The surrogate's tensor-core GEMM (tcgen05, BF16 x BF16 -> FP32) against
float64 products of the same BF16-rounded operands: strided and transposed
operands, FP32 and BF16 storage, several K segments with negation, ragged
sizes, batches, and every epilogue mode."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

TOL = 2e-5   # FP32 accumulation of exact BF16 products, relative to max |C|


@pytest.fixture(scope="module")
def K(native):
    from mbsolve_gb300 import surrogate_kernels
    assert torch.cuda.is_available()
    return surrogate_kernels


def _bf(x):
    return x.to(torch.bfloat16).double()


def _cmp(got, want, tol=TOL):
    got = got.double().cpu().numpy()
    want = want.cpu().numpy() if hasattr(want, "cpu") else want
    err = np.abs(got - want).max() / max(np.abs(want).max(), 1e-30)
    assert err < tol, err


def test_plain_and_ragged(K):
    from mbsolve_gb300 import capi_types as T
    g = torch.Generator().manual_seed(0)
    for (m, n, k) in [(128, 64, 64), (200, 70, 96), (1, 1, 1), (300, 130, 1000)]:
        a = torch.randn(m, k, generator=g).to(torch.bfloat16).cuda()
        b = torch.randn(n, k, generator=g).to(torch.bfloat16).cuda()
        c = torch.zeros(m, n, device="cuda")
        K.gemm(m, n, [K.Seg(a, 0, k, 1, 0, b, 0, k, 1, 0, k)], c, 0, n, 1)
        torch.cuda.synchronize()
        _cmp(c, _bf(a.cpu()) @ _bf(b.cpu()).T)
    assert K.status() == 0


def test_transposed_fp32_operands_and_batch(K):
    g = torch.Generator().manual_seed(1)
    Z, m, n, k = 3, 150, 40, 77
    at = torch.randn(Z, k, m, generator=g)          # A(i, k) = at[z, k, i]
    bt = torch.randn(Z, k, n, generator=g)          # B(j, k) = bt[z, k, j]
    c = torch.zeros(Z, n, m, device="cuda")         # C stored transposed
    K.gemm(m, n, [K.Seg(at.cuda(), 0, 1, m, k * m, bt.cuda().to(torch.bfloat16),
                        0, 1, n, k * n, k)],
           c, 0, 1, m, n * m, batch=Z)
    torch.cuda.synchronize()
    want = torch.einsum("zki,zkj->zji", _bf(at), _bf(bt))
    _cmp(c, want)


def test_segments_negate_accum_bias_gelu(K):
    from mbsolve_gb300 import capi_types as T
    g = torch.Generator().manual_seed(2)
    m, n = 260, 64
    k1, k2, k3 = 32, 40, 13
    a1 = torch.randn(m, k1, generator=g)
    b1 = torch.randn(n, k1, generator=g)
    a2 = torch.randn(k2, m, generator=g)           # transposed storage
    b2 = torch.randn(n, k2, generator=g)
    a3 = torch.randn(m, k3, generator=g)
    b3 = torch.randn(k3, n, generator=g)
    c0 = torch.randn(m, n, generator=g)
    bias = torch.randn(n, generator=g)
    c = c0.cuda().to(torch.bfloat16)
    pre = torch.zeros(m, n, device="cuda")
    segs = [K.Seg(a1.cuda(), 0, k1, 1, 0, b1.cuda(), 0, k1, 1, 0, k1),
            K.Seg(a2.cuda(), 0, 1, m, 0, b2.cuda(), 0, k2, 1, 0, k2,
                  negate=True),
            K.Seg(a3.cuda(), 0, k3, 1, 0, b3.cuda(), 0, 1, n, 0, k3)]
    K.gemm(m, n, segs, c, 0, n, 1, mode=T.MBG_GEMM_ACCUM, act=T.MBG_ACT_GELU,
           alpha=0.5, bias=bias.cuda(), pre=pre)
    torch.cuda.synchronize()
    acc = _bf(a1) @ _bf(b1).T - _bf(a2).T @ _bf(b2).T + _bf(a3) @ _bf(b3)
    v = 0.5 * acc + _bf(c0) + bias.double()
    _cmp(pre, v)
    gel = 0.5 * v * (1 + torch.erf(v / np.sqrt(2.0)))
    _cmp(c, gel, tol=1e-2)   # BF16 output


def test_gelu_epilogue_fp32(K):
    """The epilogues' GELU (erf by Abramowitz and Stegun 7.1.26, |error| <=
    1.5e-7) against the exact erf GELU in float64, stored in FP32: zero
    operands, so C(0, j) = GELU(bias[j]) over inputs from -12 to 12."""
    from mbsolve_gb300 import capi_types as T
    n = 8192
    x = torch.linspace(-12.0, 12.0, n, dtype=torch.float32)
    c = torch.zeros(1, n, device="cuda")
    K.gemm(1, n, [K.Seg(torch.zeros(1, 1).cuda(), 0, 1, 0, 0,
                        torch.zeros(n, 1).cuda(), 0, 1, 0, 0, 1)], c, 0, n, 1,
           act=T.MBG_ACT_GELU, bias=x.cuda())
    torch.cuda.synchronize()
    xd = x.double()
    want = 0.5 * xd * (1.0 + torch.erf(xd / np.sqrt(2.0)))
    err = (c.cpu().double()[0] - want).abs()
    # 0.5 |x| 1.5e-7 from the erf formula, a few FP32 roundings
    assert (err <= 4e-7 * xd.abs().clamp_min(1.0)).all(), float(err.max())


def test_gelu_backward_epilogue(K):
    from mbsolve_gb300 import capi_types as T
    g = torch.Generator().manual_seed(3)
    m, n, k = 128, 96, 1
    a = torch.randn(m, k, generator=g)
    b = torch.randn(n, k, generator=g)
    gate = torch.randn(m, n, generator=g)
    c = torch.zeros(m, n, device="cuda")
    K.gemm(m, n, [K.Seg(a.cuda(), 0, 1, 0, 0, b.cuda(), 0, 1, 0, 0, k)], c, 0,
           n, 1, act=T.MBG_ACT_GELU_BWD, gate=gate.cuda())
    torch.cuda.synchronize()
    x = gate.double()
    dg = 0.5 * (1 + torch.erf(x / np.sqrt(2.0))) + \
        x * torch.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)
    _cmp(c, (_bf(a) @ _bf(b).T) * dg, tol=1e-5)


def test_split_k_atomic(K):
    from mbsolve_gb300 import capi_types as T
    g = torch.Generator().manual_seed(4)
    m, n, k = 64, 64, 5000
    a = torch.randn(k, m, generator=g)      # weight-gradient shape: K = rows
    b = torch.randn(k, n, generator=g)
    c = torch.full((m, n), 1.0, device="cuda")
    K.gemm(m, n, [K.Seg(a.cuda(), 0, 1, m, 0, b.cuda(), 0, 1, n, 0, k)], c, 0,
           n, 1, mode=T.MBG_GEMM_ATOMIC, split_k=16)
    torch.cuda.synchronize()
    _cmp(c, 1.0 + _bf(a).T @ _bf(b), tol=5e-5)


def test_host_refuses_out_of_bounds_strides(K):
    a = torch.zeros(10, 8, device="cuda", dtype=torch.bfloat16)
    b = torch.zeros(4, 8, device="cuda", dtype=torch.bfloat16)
    c = torch.zeros(10, 4, device="cuda")
    with pytest.raises(ValueError):
        K.gemm(11, 4, [K.Seg(a, 0, 8, 1, 0, b, 0, 8, 1, 0, 8)], c, 0, 4, 1)
    with pytest.raises(ValueError):
        K.gemm(10, 4, [K.Seg(a, 0, 8, 1, 0, b, 0, 8, 1, 0, 9)], c, 0, 4, 1)
