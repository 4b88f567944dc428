"""The fused Fourier-layer kernel (mbg_fno_spectral_layer) against the CPU
model of its arithmetic (tests/fno_emulator.py: float64 sums of the same
BF16-rounded operands, FP32 accumulators, BF16 stores; operands and
activations as tile images), in all three modes, and the image kernel:
at the surrogate's full width with more samples than SMs (each CTA walks
several samples, tiles crossing sample boundaries in its pipeline) and at
ragged sizes (W, Mo, Hq, Fi below the kernel's tile sizes, one sample per
CTA)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from tests import fno_emulator as E

pytestmark = pytest.mark.gpu

# What differs from the model: FP32 accumulation order (1e-6 relative) and
# FP32 erf, which moves a few BF16 roundings by one unit (4e-3 relative on
# those entries). Relative L2 over each output:
TOL = 2e-3


@pytest.fixture(scope="module")
def K(native):
    from mbsolve_gb300 import surrogate_kernels
    assert torch.cuda.is_available()
    return surrogate_kernels


def _rel(a, b):
    a = a.double().cpu().numpy().ravel()
    b = b.double().cpu().numpy().ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


def _inputs(B, S, W, Mo, Fi, Hq, seed):
    """Random operands in the kernel's layouts: activations, bases and dense
    weights as BF16 tile images (channels, modes and rows beyond W, 2 Mo and
    Hq zero)."""
    g = torch.Generator().manual_seed(seed)
    b16, T = torch.bfloat16, S // 128
    r = lambda *s: torch.randn(*s, generator=g)

    def pad(x, R, K):
        out = torch.zeros(x.shape[0], R, K)
        out[:, :x.shape[1], :x.shape[2]] = x
        return out

    v = pad(r(B * T, 128, W), 128, 64)
    G = pad(r(T, 128, 2 * Mo), 128, 64)
    F = pad(r(T, 2 * Mo, 128) / S, 64, 128)
    return dict(
        X=r(B, S, Fi), P=E.to_image(pad(r(1, W, Fi) / Fi ** 0.5, 64, 16)).to(b16),
        v=E.to_image(v).to(b16), Y=r(B, 2, Mo, W).to(b16),
        G=E.to_image(G).to(b16), Wl=E.to_image(pad(r(1, W, W) / W ** 0.5, 64, 64)).to(b16),
        bias=r(W) * 0.1, F=E.to_image(F).to(b16),
        Q1=E.to_image(pad(r(1, Hq, W) / W ** 0.5, 128, 64)).to(b16),
        bq1=r(Hq) * 0.1, q2=r(Hq) / Hq ** 0.5, bq2=r(1))


@pytest.mark.parametrize("B,S,W,Mo,Fi,Hq", [(311, 256, 64, 32, 9, 128),
                                            (5, 128, 24, 16, 3, 40)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_layer_matches_model(K, mode, B, S, W, Mo, Fi, Hq):
    from mbsolve_gb300 import capi_types as T
    x = _inputs(B, S, W, Mo, Fi, Hq, seed=7 + mode)
    act = T.MBG_ACT_NONE if mode != T.MBG_LAYER_MID else T.MBG_ACT_GELU
    outs = dict(v_out=torch.zeros(B * S * 64, dtype=torch.bfloat16),
                vhT=torch.zeros(B * 2 * Mo * W, dtype=torch.bfloat16),
                y=torch.zeros(B * S))
    use = dict(x)
    if mode == T.MBG_LAYER_LIFT:
        for k in ("v", "Y", "G", "Wl", "Q1", "bq1", "q2", "bq2"):
            use.pop(k)
    else:
        for k in ("X", "P"):
            use.pop(k)
    if mode == T.MBG_LAYER_LAST:
        use.pop("F")
        want = dict(y=outs["y"])
    else:
        for k in ("Q1", "bq1", "q2", "bq2"):
            use.pop(k, None)
        want = dict(v_out=outs["v_out"], vhT=outs["vhT"])
    gpu = {k: v.contiguous().cuda() for k, v in use.items()}
    gout = {k: torch.full_like(v, float("nan")).cuda() for k, v in want.items()}
    K.spectral_layer(mode, act, B, S, W, Mo, Fi=Fi, Hq=Hq, **gpu, **gout)
    torch.cuda.synchronize()
    assert K.status() == 0
    E.spectral_layer(mode, act, B, S, W, Mo, Fi=Fi, Hq=Hq, **use, **want)
    for k in want:
        assert torch.isfinite(gout[k].float()).all(), k
        err = _rel(gout[k], want[k])
        assert err <= TOL, (k, err)


def test_layer_rejects_missing_operands(K):
    from mbsolve_gb300 import capi_types as T
    with pytest.raises(ValueError):
        K.spectral_layer(T.MBG_LAYER_MID, T.MBG_ACT_GELU, 2, 128, 64, 32)


def test_image_kernel_matches_model(K):
    g = torch.Generator().manual_seed(3)
    x = torch.randn(3, 100, 50, generator=g)
    for (batch, rows, cols, ld, zs, R, Kc) in [(3, 100, 50, 50, 5000, 104, 56),
                                                (1, 40, 30, 50, 0, 64, 32),
                                                (2, 50, 40, 50, 40, 64, 128)]:
        n = batch * R * Kc
        got = torch.zeros(n, dtype=torch.bfloat16, device="cuda")
        K.image_bf16(x.cuda(), batch, rows, cols, ld, zs, R, Kc, got)
        want = torch.zeros(n, dtype=torch.bfloat16)
        E.image_bf16(x, batch, rows, cols, ld, zs, R, Kc, want)
        torch.cuda.synchronize()
        assert torch.equal(got.cpu(), want)
