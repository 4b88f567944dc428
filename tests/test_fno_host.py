"""Host logic of the surrogate without a GPU: the network's plan of strided
products (operand offsets, strides, K segments, epilogues) evaluated by a
CPU model of the kernels equals the CPU oracle's forward and backward pass;
the prescreen feature builder and sweep sampling are deterministic."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from oracle import fno_oracle as O

from tests import fno_emulator as E


def _rel(a, b):
    a, b = np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)


@pytest.mark.parametrize("args", [dict(S=64, W=8, Mo=8, L=2, F=8, Hq=16),
                                  dict(S=128, W=16, Mo=8, L=3, F=9, Hq=32)])
def test_product_plan_equals_oracle(monkeypatch, args):
    from mbsolve_gb300 import surrogate as S
    E.install(monkeypatch)
    sh = S.Shapes(**args)
    net = S.FNO(sh, seed=4, device="cpu")
    rng = np.random.default_rng(9)
    B = 8
    X = rng.normal(size=(B, sh.S, sh.F)).astype(np.float32)
    t = rng.normal(size=(B, sh.S)).astype(np.float32)
    y = net.forward(torch.tensor(X)).clone()
    loss = net.loss(torch.tensor(t)).item()
    net.backward()
    theta = net.theta.double().numpy()
    osh = O.Shapes(**args)
    ol, og, oy = O.forward_backward(osh, theta, X.astype(np.float64),
                                    t.astype(np.float64), bf16=True)
    assert _rel(y.numpy(), oy) < 1e-3
    assert abs(loss - ol) < 1e-3 * ol
    gp = O.unflatten(osh, net.grad.double().numpy())
    op = O.unflatten(osh, og)
    for name, _ in osh.param_spec():
        assert _rel(gp[name], op[name]) < 1e-2, name


def test_training_step_moves_toward_lower_loss(monkeypatch):
    from mbsolve_gb300 import surrogate as S
    E.install(monkeypatch)
    sh = S.Shapes(S=64, W=8, Mo=8, L=2, F=8, Hq=16)
    net = S.FNO(sh, seed=1, device="cpu")
    rng = np.random.default_rng(3)
    X = torch.tensor(rng.normal(size=(8, sh.S, sh.F)).astype(np.float32))
    t = torch.tensor(rng.normal(size=(8, sh.S)).astype(np.float32))
    l0 = net.train_step(X, t, lr=1e-3).item()
    for _ in range(20):
        l1 = net.train_step(X, t, lr=1e-3).item()
    assert l1 < l0


def test_backward_refuses_batches_not_multiple_of_8(monkeypatch):
    from mbsolve_gb300 import surrogate as S
    E.install(monkeypatch)
    sh = S.Shapes(S=64, W=8, Mo=8, L=2, F=8, Hq=16)
    net = S.FNO(sh, seed=1, device="cpu")
    net.forward(torch.zeros(4, sh.S, sh.F))
    with pytest.raises(ValueError):
        net.backward()


def test_sweep_space_is_deterministic():
    from mbsolve_gb300 import prescreen as P
    a, b = P.SweepSpace(seed=0), P.SweepSpace(seed=0)
    assert a.f0 == b.f0 and 3e12 <= a.f0 <= 8e12
    pa, pb = a.sample(16, seed=5), b.sample(16, seed=5)
    for k in P.PARAM_NAMES:
        np.testing.assert_array_equal(pa[k], pb[k])
        lo, hi = P.RANGES[k]
        assert pa[k].min() >= lo and pa[k].max() <= hi
    X = a.features(pa, device="cpu")
    assert tuple(X.shape) == (16, a.samples, P.NUM_FEATURES)
    assert float(X[..., 0].max()) <= 1.0 + 1e-6
    assert float(X[..., 1:8].abs().max()) <= 1.0 + 1e-6
    dev, sce = a.run(pa, 0)
    assert sce.get_num_gridpoints() == a.n_x


@pytest.mark.parametrize("S_,fused", [(64, False), (128, True)])
def test_inference_plan_equals_forward(monkeypatch, S_, fused):
    """FNO.infer computes the same network as forward(), through the CPU
    model of the kernels: as fused layer launches (S a multiple of 128:
    lifting + DFT, inverse DFT + pointwise + DFT, last layer + projection,
    two mixing products per layer) and as products of the general kernel
    (K-contiguous BF16 layouts, transposed activation copies, BF16 weight
    copies)."""
    from mbsolve_gb300 import surrogate as S
    E.install(monkeypatch)
    sh = S.Shapes(S=S_, W=16, Mo=8, L=3, F=5, Hq=24)
    net = S.FNO(sh, seed=2, device="cpu")
    assert net.fused_ok() == fused
    X = torch.tensor(np.random.default_rng(4).normal(size=(3, S_, 5)),
                     dtype=torch.float32)
    yf = net.forward(X).clone().double().numpy()
    yi = net.infer(X).clone().double().numpy()
    assert np.linalg.norm(yi - yf) <= 1e-6 * np.linalg.norm(yf)



def test_spectral_layer_refuses_bad_sizes():
    """The fused layer's C entry point checks sizes and operands before it
    touches the GPU."""
    import ctypes as C
    from mbsolve_gb300 import _native
    from mbsolve_gb300 import capi_types as T
    L = _native.load()
    good = dict(mode=T.MBG_LAYER_MID, act=T.MBG_ACT_GELU, batch=4, S=256,
                W=64, Mo=32, Fi=0, Hq=0)
    bad = [dict(S=200), dict(W=72), dict(W=12), dict(Mo=40), dict(Mo=12),
           dict(mode=7), dict(act=2), dict(batch=0)]
    for b in bad:
        d = T.mbg_fno_layer_desc()
        for k, v in dict(good, **b).items():
            setattr(d, k, v)
        rc = L.mbg_fno_spectral_layer(C.byref(d), None)
        assert rc == T.MBG_ERR_INVALID_ARGUMENT, b
    d = T.mbg_fno_layer_desc()       # sizes fine, operands missing
    for k, v in good.items():
        setattr(d, k, v)
    assert L.mbg_fno_spectral_layer(C.byref(d), None) == T.MBG_ERR_INVALID_ARGUMENT
    assert b"v, Y, G and Wl" in L.mbg_last_error()
    assert L.mbg_fno_spectral_layer(None, None) == T.MBG_ERR_INVALID_ARGUMENT
