"""CPU oracle of the Fourier-neural-operator surrogate: forward pass, loss
and every parameter gradient in float64 numpy.

Test infrastructure only: the tests compare the GPU network
(mbsolve_gb300/surrogate.py, tensor-core kernels) with this restatement;
nothing in the package imports it.

The network (a 1-D Fourier neural operator in the form of Li et al.,
"Fourier Neural Operator for Parametric Partial Differential Equations",
ICLR 2021):

    v0 = X P^T + bp                            X: [B, S, F] input features
    for l < L:
        Vh[b, c, :] = F v_l[b, :, c]           truncated DFT, 2 Mo reals
        Y[b, m, :]  = blk_l[m] [Re Vh; Im Vh]  complex mode mixing
        pre_l = G Y + v_l W_l^T + bw_l         inverse DFT + pointwise path
        v_{l+1} = gelu(pre_l)  (no activation after the last layer)
    h = gelu(v_L Q1^T + bq1);  y = h q2 + bq2

F [2Mo, S]: cos(2 pi m s / S) / S and -sin(...) / S; G [S, 2Mo]: c_m cos and
-c_m sin with c_0 = 1, c_m = 2 (the inverse of the truncated real DFT).
blk_l[m] is the real 2x2 block form of the complex weights wr + i wi.

With `bf16=True` every product operand is rounded to bfloat16 and every
stored activation to the precision the GPU stores it in (BF16 for v_l and
h, FP32 for the pre-activations), so that the GPU and the oracle differ
only by FP32 accumulation order and FP32 elementwise math.
"""
import math

import numpy as np


def bf16_round(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    return np.where(np.isfinite(a), out, a.astype(np.float64))


def f32_round(x):
    return np.asarray(x, dtype=np.float32).astype(np.float64)


def dft_bases(S, Mo):
    """F [2Mo, S] and G [S, 2Mo] in float64."""
    s = np.arange(S)[None, :]
    m = np.arange(Mo)[:, None]
    ang = 2.0 * math.pi * m * s / S
    F = np.concatenate([np.cos(ang), -np.sin(ang)], axis=0) / S
    c = np.where(np.arange(Mo) == 0, 1.0, 2.0)[None, :]
    angT = ang.T
    G = np.concatenate([c * np.cos(angT), -c * np.sin(angT)], axis=1)
    return F, G


def gelu(x):
    from scipy.special import erf
    return 0.5 * x * (1.0 + erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    from scipy.special import erf
    return 0.5 * (1.0 + erf(x / math.sqrt(2.0))) + \
        x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


class Shapes:
    def __init__(self, S=1024, W=64, Mo=32, L=4, F=8, Hq=128):
        self.S, self.W, self.Mo, self.L, self.F, self.Hq = S, W, Mo, L, F, Hq

    def param_spec(self):
        """(name, shape) in the order of the flat parameter vector."""
        W, Mo, F, Hq = self.W, self.Mo, self.F, self.Hq
        spec = [("P", (W, F)), ("bp", (W,))]
        for l in range(self.L):
            spec += [("wr%d" % l, (Mo, W, W)), ("wi%d" % l, (Mo, W, W)),
                     ("W%d" % l, (W, W)), ("bw%d" % l, (W,))]
        spec += [("Q1", (Hq, W)), ("bq1", (Hq,)), ("q2", (Hq,)),
                 ("bq2", (1,))]
        return spec

    def num_params(self):
        return sum(int(np.prod(s)) for _, s in self.param_spec())


def unflatten(sh, theta):
    out, o = {}, 0
    for name, shape in sh.param_spec():
        n = int(np.prod(shape))
        out[name] = theta[o:o + n].reshape(shape)
        o += n
    return out


def flatten(sh, d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel()
                           for name, _ in sh.param_spec()])


def init_params(sh, seed=0):
    """Seeded initialisation: linear layers U(-1/sqrt(fan_in), +), spectral
    weights U(0, 1) / (W W) as in the reference FNO implementation."""
    rng = np.random.default_rng(seed)
    d = {}
    for name, shape in sh.param_spec():
        if name.startswith(("wr", "wi")):
            d[name] = rng.uniform(0.0, 1.0, size=shape) / (sh.W * sh.W)
        elif name in ("P", "Q1") or (name.startswith("W") and name[1:].isdigit()):
            fan = shape[1]
            d[name] = rng.uniform(-1, 1, size=shape) / math.sqrt(fan)
        elif name == "q2":
            d[name] = rng.uniform(-1, 1, size=shape) / math.sqrt(sh.Hq)
        else:
            fan = {"bp": sh.F, "bq1": sh.W, "bq2": sh.Hq}.get(name, sh.W)
            d[name] = rng.uniform(-1, 1, size=shape) / math.sqrt(fan)
    return flatten(sh, d)


def mode_blocks(wr, wi):
    """[Mo, 2W, 2W] real blocks: [Re y; Im y] = blk [Re x; Im x]."""
    Mo, W, _ = wr.shape
    blk = np.zeros((Mo, 2 * W, 2 * W))
    rT = np.transpose(wr, (0, 2, 1))   # [m, o, c]
    iT = np.transpose(wi, (0, 2, 1))
    blk[:, :W, :W] = rT
    blk[:, :W, W:] = -iT
    blk[:, W:, :W] = iT
    blk[:, W:, W:] = rT
    return blk


def forward_backward(sh, theta, X, target, bf16=False):
    """Loss (mean squared error) and its gradient w.r.t. the flat parameter
    vector. X [B, S, F], target [B, S]."""
    q = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    f32 = f32_round if bf16 else (lambda a: a)
    p = unflatten(sh, theta)
    B = X.shape[0]
    S, W, Mo, L = sh.S, sh.W, sh.Mo, sh.L
    F, G = dft_bases(S, Mo)
    Fq, Gq = q(F), q(G)
    Xq = q(X)

    # forward
    v = [q(f32(Xq @ q(p["P"]).T + p["bp"]))]
    Vh, pre, blks = [], [], []
    for l in range(L):
        blk = q(mode_blocks(p["wr%d" % l], p["wi%d" % l]))
        blks.append(blk)
        vh = f32(np.einsum("ms,bsc->bcm", Fq, v[l]))            # [B, W, 2Mo]
        Vh.append(vh)
        x = np.concatenate([vh[:, :, :Mo], vh[:, :, Mo:]], axis=1)  # [B, 2W, Mo]
        y = f32(np.einsum("mjk,bkm->bmj", blk, q(x)))            # [B, Mo, 2W]
        yq = q(y)
        spec = np.einsum("sm,bmo->bso", Gq[:, :Mo], yq[:, :, :W]) + \
            np.einsum("sm,bmo->bso", Gq[:, Mo:], yq[:, :, W:])
        pr = f32(spec + v[l] @ q(p["W%d" % l]).T + p["bw%d" % l])
        pre.append(pr)
        v.append(q(gelu(pr)) if l < L - 1 else q(pr))
    ph = f32(v[L] @ q(p["Q1"]).T + p["bq1"])
    h = q(gelu(ph))
    y = f32(h @ q(p["q2"]) + p["bq2"][0])
    n = y.size
    diff = y - target
    loss = float(np.sum(diff * diff) / n)

    # backward
    g = {k: np.zeros_like(vv) for k, vv in p.items()}
    dy = f32(2.0 * diff / n)
    dyq = q(dy)
    g["q2"] = np.einsum("bsj,bs->j", h, dyq)
    g["bq2"] = np.array([dy.sum()])
    dh = f32(dyq[..., None] * q(p["q2"])[None, None, :] * gelu_grad(ph))
    dhq = q(dh)
    g["Q1"] = np.einsum("bsj,bsc->jc", dhq, v[L])
    g["bq1"] = dh.sum(axis=(0, 1))
    dpre = f32(dhq @ q(p["Q1"]))                                  # [B, S, W]
    for l in range(L - 1, -1, -1):
        dq_ = q(dpre)
        g["W%d" % l] = np.einsum("bso,bsc->oc", dq_, v[l])
        g["bw%d" % l] = dpre.sum(axis=(0, 1))
        dY = f32(np.einsum("sm,bso->bmo", Gq, dq_))               # [B, 2Mo, W]
        dYq = q(dY)
        dre, dim = dYq[:, :Mo, :], dYq[:, Mo:, :]                 # [B, Mo, W]
        vre, vim = q(Vh[l][:, :, :Mo]), q(Vh[l][:, :, Mo:])       # [B, W, Mo]
        g["wr%d" % l] = np.einsum("bmo,bcm->mco", dre, vre) + \
            np.einsum("bmo,bcm->mco", dim, vim)
        g["wi%d" % l] = -np.einsum("bmo,bcm->mco", dre, vim) + \
            np.einsum("bmo,bcm->mco", dim, vre)
        blk = blks[l]
        dcat = np.concatenate([dre, dim], axis=2)                 # [B, Mo, 2W]
        dx = f32(np.einsum("bmj,mjk->bmk", dcat, blk))            # [B, Mo, 2W]
        dVh = np.concatenate([np.transpose(dx[:, :, :W], (0, 2, 1)),
                              np.transpose(dx[:, :, W:], (0, 2, 1))], axis=2)
        dv = np.einsum("ms,bcm->bsc", Fq, q(dVh)) + dq_ @ q(p["W%d" % l])
        if l > 0:
            dpre = f32(dv * gelu_grad(pre[l - 1]))
        else:
            dpre = f32(dv)
    dv0 = dpre
    g["P"] = np.einsum("bso,bsf->of", q(dv0), Xq)
    g["bp"] = dv0.sum(axis=(0, 1))
    return loss, flatten(sh, g), y


def predict(sh, theta, X, bf16=False):
    _, _, y = forward_backward(sh, theta, X, np.zeros(X.shape[:2]), bf16)
    return y
