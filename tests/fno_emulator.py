"""CPU model of the surrogate kernels' semantics (include/mbsolve_fno.h),
for tests of the host-side product plan without a GPU: the same arguments
surrogate_kernels receives, evaluated with torch on the CPU (BF16 operand
rounding, FP32 stores, the same epilogues). Test infrastructure only."""
import math

import torch


def _view(t, off, size, stride):
    # element offsets are relative to the tensor (a view into a flat buffer)
    return torch.as_strided(t, size, stride, t.storage_offset() + int(off))


def _bf(x):
    return x.to(torch.bfloat16).to(torch.float64)


def gemm(m, n, segs, c, c_off, c_sm, c_sn, c_sz=0, batch=1, mode=0, act=0,
         alpha=1.0, bias=None, pre=None, gate=None, split_k=1, c2=None,
         c2_sm=0, c2_sn=0, c2_sz=0, rowdot=None, rowdot_bias=None):
    acc = torch.zeros(batch, m, n, dtype=torch.float64)
    for s in segs:
        A = _bf(_view(s.a, s.a_off, (batch, m, s.k), (s.a_sz, s.a_sm, s.a_sk)))
        B = _bf(_view(s.b, s.b_off, (batch, n, s.k), (s.b_sz, s.b_sn, s.b_sk)))
        p = A @ B.transpose(1, 2)
        acc = acc - p if s.negate else acc + p
    # FP32 accumulator
    v = (alpha * acc.to(torch.float32).to(torch.float64))
    C = _view(c, c_off, (batch, m, n), (c_sz, c_sm, c_sn))
    if mode == 2:
        C.copy_((C.to(torch.float64) + v).to(C.dtype))
        return
    if mode == 1:
        v = v + C.to(torch.float64)
    if bias is not None:
        v = v + bias[:n].to(torch.float64)
    v = v.to(torch.float32).to(torch.float64)
    if rowdot is not None:
        if act == 1:
            v = 0.5 * v * (1.0 + torch.erf(v / math.sqrt(2.0)))
        s = (_bf(v) * _bf(rowdot[:n].to(torch.float64))).sum(-1)
        if rowdot_bias is not None:
            s = s + rowdot_bias[0].to(torch.float64)
        Cv = _view(c, c_off, (batch, m), (c_sz, c_sm))
        Cv.copy_((Cv.to(torch.float64) + s).to(Cv.dtype))
        return
    if pre is not None:
        _view(pre, c_off, (batch, m, n), (c_sz, c_sm, c_sn)).copy_(v.to(torch.float32))
    if act == 1:
        v = 0.5 * v * (1.0 + torch.erf(v / math.sqrt(2.0)))
    elif act == 2:
        g = _view(gate, c_off, (batch, m, n), (c_sz, c_sm, c_sn)).to(torch.float64)
        v = v * (0.5 * (1.0 + torch.erf(g / math.sqrt(2.0))) +
                 g * torch.exp(-0.5 * g * g) / math.sqrt(2.0 * math.pi))
    C.copy_(v.to(C.dtype))
    if c2 is not None:
        _view(c2, 0, (batch, m, n), (c2_sz, c2_sm, c2_sn)).copy_(v.to(c2.dtype))


def _gelu(v):
    return 0.5 * v * (1.0 + torch.erf(v / math.sqrt(2.0)))


def _flat(t, n, shape):
    return t.reshape(-1)[:n].reshape(shape)


def from_image(img, nblk, R, K):
    """[nblk, R, K] matrices from their K-major core-matrix images."""
    x = _flat(img, nblk * R * K, (nblk, R // 8, K // 8, 8, 8))
    return x.transpose(2, 3).reshape(nblk, R, K)


def to_image(x):
    """The K-major core-matrix images of x [nblk, R, K], flattened."""
    nblk, R, K = x.shape
    return x.reshape(nblk, R // 8, 8, K // 8, 8).transpose(2, 3).reshape(-1)


def image_bf16(x, batch, rows, cols, ld, zs, R, K, img):
    m = _view(x, 0, (batch, rows, cols), (zs, ld, 1)).to(torch.float32)
    pad = torch.zeros(batch, R, K, dtype=torch.float32)
    pad[:, :rows, :cols] = m
    img.reshape(-1)[:batch * R * K].copy_(to_image(pad).to(img.dtype))


def spectral_layer(mode, act, batch, S, W, Mo, Fi=0, Hq=0, X=None, P=None,
                   v=None, Y=None, G=None, Wl=None, bias=None, v_out=None,
                   F=None, vhT=None, Q1=None, bq1=None, q2=None, bq2=None,
                   y=None):
    B, M2, T = batch, 2 * Mo, S // 128
    f32, f64, b16 = torch.float32, torch.float64, torch.bfloat16
    if mode == 0:
        Pm = _bf(from_image(P, 1, 64, 16)[0, :W, :Fi])
        u = _bf(_flat(X, B * S * Fi, (B, S, Fi))) @ Pm.T
    else:
        Yv = _bf(_flat(Y, B * 2 * Mo * W, (B, 2, Mo, W)))
        Yf = Yv.permute(0, 3, 1, 2).reshape(B, W, M2)          # [B, W, 2 Mo]
        Gm = _bf(from_image(G, T, 128, 64).reshape(S, 64)[:, :M2])
        vm = _bf(from_image(v, B * T, 128, 64).reshape(B, S, 64)[..., :W])
        Wm = _bf(from_image(Wl, 1, 64, 64)[0, :W, :W])
        u = Gm @ Yf.transpose(1, 2) + vm @ Wm.T
    u = u.to(f32).to(f64)                                      # FP32 accumulator
    if bias is not None:
        u = (u + bias[:W].to(f64)).to(f32).to(f64)
    if act == 1:
        u = _gelu(u)
    ub = _bf(u)
    if mode != 2:
        pad = torch.zeros(B, S, 64, dtype=f64)
        pad[..., :W] = ub
        v_out.reshape(-1)[:B * S * 64].copy_(to_image(pad.reshape(B * T, 128, 64)).to(b16))
        Fm = _bf(from_image(F, T, 64, 128).permute(1, 0, 2).reshape(64, S)[:M2])
        d = (Fm @ ub).to(f32)                                  # [B, 2 Mo, W]
        vhT.reshape(-1)[:B * M2 * W].copy_(d.reshape(-1).to(b16))
    else:
        Qm = _bf(from_image(Q1, 1, 128, 64)[0, :Hq, :W])
        h = (ub @ Qm.T).to(f32).to(f64)
        h = (h + bq1[:Hq].to(f64)).to(f32).to(f64)
        z = _bf(_gelu(h))
        yv = (z * _bf(q2[:Hq].to(f64))).sum(-1) + bq2[0].to(f64)
        y.reshape(-1)[:B * S].copy_(yv.reshape(-1).to(f32))


def cast_bf16(x, y):
    y.copy_(x.reshape(-1)[:y.numel()].to(torch.bfloat16))


def mode_blocks(wr, wi, blk):
    Mo, W = wr.shape[0], wr.shape[1]
    r = wr.reshape(Mo, W, W).transpose(1, 2)
    i = wi.reshape(Mo, W, W).transpose(1, 2)
    top = torch.cat([r, -i], dim=2)
    bot = torch.cat([i, r], dim=2)
    blk.copy_(torch.cat([top, bot], dim=1).reshape(-1).to(blk.dtype))


def colsum(x, rows, cols, row_stride, out):
    v = _view(x, 0, (rows, cols), (row_stride, 1)).to(torch.float64).sum(0)
    out[:cols] += v.to(torch.float32)


def mse(y, t, grad, loss):
    n = y.numel()
    d = y.to(torch.float64) - t.to(torch.float64)
    grad.copy_((2.0 * d / n).to(torch.float32))
    loss += float((d * d).sum() / n)


def adam(w, g, m, v, lr, beta1, beta2, eps, weight_decay, step):
    m.mul_(beta1).add_((1 - beta1) * g)
    v.mul_(beta2).add_((1 - beta2) * g * g)
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    w.sub_(lr * (mh / (vh.sqrt() + eps) + weight_decay * w))


def install(monkeypatch):
    """Route the surrogate module's kernel calls to this model."""
    from mbsolve_gb300 import surrogate as S
    for name in ("gemm", "spectral_layer", "image_bf16", "mode_blocks",
                 "colsum", "mse", "adam", "cast_bf16"):
        monkeypatch.setattr(S.K, name, globals()[name])
