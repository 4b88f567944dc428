"""Python side of the surrogate's CUDA kernels (include/mbsolve_fno.h).

Tensors are torch CUDA tensors used as device memory only; every operation
runs in this package's own kernels (libmbsolve_gb300.so). Each call checks
on the host that every element the kernel will touch lies inside its
tensor, so a wrong stride raises here instead of reading out of bounds.
"""
import ctypes as C

import torch

from . import _native
from . import capi_types as T

_TYPES = {torch.float32: T.MBG_F32, torch.bfloat16: T.MBG_BF16}


def _lib():
    return _native.load()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t, off=0):
    return C.c_void_p(t.data_ptr() + int(off) * t.element_size())


def _check_span(t, off, extents_strides, what):
    """All of t's elements at off + sum_i idx_i * stride_i, 0 <= idx_i <
    extent_i, must exist (strides may be zero, none negative)."""
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("%s: need a contiguous CUDA tensor" % what)
    if t.dtype not in _TYPES:
        raise ValueError("%s: dtype %s not supported" % (what, t.dtype))
    hi = int(off)
    for ext, st in extents_strides:
        if st < 0:
            raise ValueError("%s: negative stride" % what)
        if ext > 0:
            hi += (int(ext) - 1) * int(st)
    if off < 0 or hi >= t.numel():
        raise ValueError("%s: operand span [%d, %d] outside a tensor of %d"
                         % (what, off, hi, t.numel()))


class Seg:
    """One operand pair of a product: A(i, k) = a[a_off + z a_sz + i a_sm +
    k a_sk], B(j, k) = b[b_off + z b_sz + j b_sn + k b_sk], k < `k`."""

    def __init__(self, a, a_off, a_sm, a_sk, a_sz, b, b_off, b_sn, b_sk,
                 b_sz, k, negate=False):
        self.a, self.a_off, self.a_sm, self.a_sk, self.a_sz = \
            a, a_off, a_sm, a_sk, a_sz
        self.b, self.b_off, self.b_sn, self.b_sk, self.b_sz = \
            b, b_off, b_sn, b_sk, b_sz
        self.k = int(k)
        self.negate = bool(negate)


def gemm(m, n, segs, c, c_off, c_sm, c_sn, c_sz=0, batch=1,
         mode=T.MBG_GEMM_STORE, act=T.MBG_ACT_NONE, alpha=1.0, bias=None,
         pre=None, gate=None, split_k=1, c2=None, c2_sm=0, c2_sn=0, c2_sz=0,
         rowdot=None, rowdot_bias=None):
    """C[z](i, j) = epilogue(alpha sum_s sum_k A_s(i, k) B_s(j, k)) for
    i < m, j < n, z < batch, on the tensor cores (BF16 x BF16 -> FP32);
    c2 (BF16, STORE mode): the same values again with strides c2_*;
    rowdot (FP32 [n]): C[z](i, 0) += rowdot . out(i, :) (+ rowdot_bias)
    instead of storing out (FP32 C holding the starting values)."""
    d = T.mbg_gemm_desc()
    d.m, d.n, d.batch, d.nseg = int(m), int(n), int(batch), len(segs)
    if not 1 <= len(segs) <= 3:
        raise ValueError("gemm: 1 to 3 segments")
    for i, s in enumerate(segs):
        _check_span(s.a, s.a_off, [(batch, s.a_sz), (m, s.a_sm), (s.k, s.a_sk)],
                    "gemm A[%d]" % i)
        _check_span(s.b, s.b_off, [(batch, s.b_sz), (n, s.b_sn), (s.k, s.b_sk)],
                    "gemm B[%d]" % i)
        g = d.seg[i]
        g.a, g.b = _ptr(s.a, s.a_off), _ptr(s.b, s.b_off)
        g.a_sm, g.a_sk, g.a_sz = s.a_sm, s.a_sk, s.a_sz
        g.b_sn, g.b_sk, g.b_sz = s.b_sn, s.b_sk, s.b_sz
        g.k = s.k
        g.a_type, g.b_type = _TYPES[s.a.dtype], _TYPES[s.b.dtype]
        g.negate = int(s.negate)
    span = [(batch, c_sz), (m, c_sm), (n, c_sn)]
    _check_span(c, c_off, span, "gemm C")
    for t, nm in ((pre, "pre"), (gate, "gate")):
        if t is not None:
            if t.dtype != torch.float32:
                raise ValueError("gemm %s: FP32 only" % nm)
            _check_span(t, c_off, span, "gemm " + nm)
    if bias is not None:
        if bias.dtype != torch.float32 or bias.numel() < n:
            raise ValueError("gemm bias: FP32 with n entries")
    d.c = _ptr(c, c_off)
    d.c_sm, d.c_sn, d.c_sz = c_sm, c_sn, c_sz
    d.c_type = _TYPES[c.dtype]
    d.mode, d.act, d.split_k = int(mode), int(act), int(split_k)
    d.alpha = float(alpha)
    d.bias = _ptr(bias) if bias is not None else None
    d.pre = _ptr(pre, c_off) if pre is not None else None
    d.gate = _ptr(gate, c_off) if gate is not None else None
    if c2 is not None:
        if c2.dtype != torch.bfloat16:
            raise ValueError("gemm c2: BF16 only")
        _check_span(c2, 0, [(batch, c2_sz), (m, c2_sm), (n, c2_sn)], "gemm c2")
        d.c2 = _ptr(c2)
        d.c2_sm, d.c2_sn, d.c2_sz = c2_sm, c2_sn, c2_sz
    if rowdot is not None:
        if rowdot.dtype != torch.float32 or rowdot.numel() < n:
            raise ValueError("gemm rowdot: FP32 with n entries")
        d.rowdot = _ptr(rowdot)
        if rowdot_bias is not None:
            d.rowdot_bias = _ptr(rowdot_bias)
    _native.check(_lib().mbg_fno_gemm(C.byref(d), _stream()))


def spectral_layer(mode, act, batch, S, W, Mo, Fi=0, Hq=0, X=None, P=None,
                   v=None, Y=None, G=None, Wl=None, bias=None, v_out=None,
                   F=None, vhT=None, Q1=None, bq1=None, q2=None, bq2=None,
                   y=None):
    """One Fourier layer of inference in one launch (mbg_fno_spectral_layer):
    mode MBG_LAYER_LIFT (X [B, S, Fi] FP32, P image [64 16] BF16), MBG_LAYER_MID (v
    activation images [B S 64], Y [B, 2, Mo, W], G images [S/128, 8192],
    Wl image [64 64], BF16) or MBG_LAYER_LAST (the same plus the Q1 image
    [128 64] BF16, bq1, q2 [Hq], bq2 [1] FP32 and y [B, S] FP32); LIFT and
    MID write the activation images v_out [B S 64] and the spectrum vhT
    [B, 2 Mo, W] (BF16) with the F images [S/128, 8192]. Images as
    written by image_bf16 (include/mbsolve_fno.h)."""
    B, ntile = int(batch), int(S) // 128
    need = {}
    if mode == T.MBG_LAYER_LIFT:
        need.update(X=(X, torch.float32, B * S * Fi), P=(P, torch.bfloat16, 64 * 16))
    else:
        need.update(v=(v, torch.bfloat16, B * S * 64),
                    Y=(Y, torch.bfloat16, B * 2 * W * Mo),
                    G=(G, torch.bfloat16, ntile * 8192),
                    Wl=(Wl, torch.bfloat16, 64 * 64))
    if mode == T.MBG_LAYER_LAST:
        need.update(Q1=(Q1, torch.bfloat16, 128 * 64), bq1=(bq1, torch.float32, Hq),
                    q2=(q2, torch.float32, Hq), bq2=(bq2, torch.float32, 1),
                    y=(y, torch.float32, B * S))
    else:
        need.update(v_out=(v_out, torch.bfloat16, B * S * 64),
                    F=(F, torch.bfloat16, ntile * 8192),
                    vhT=(vhT, torch.bfloat16, B * 2 * Mo * W))
    if bias is not None:
        need["bias"] = (bias, torch.float32, W)
    d = T.mbg_fno_layer_desc()
    for name, (t, dt, n) in need.items():
        if t is None:
            raise ValueError("spectral_layer: %s is required" % name)
        if t.dtype != dt or not t.is_cuda or not t.is_contiguous():
            raise ValueError("spectral_layer %s: contiguous CUDA %s" % (name, dt))
        if t.numel() < n:
            raise ValueError("spectral_layer %s: %d elements, %d needed"
                             % (name, t.numel(), n))
        setattr(d, name, _ptr(t))
    d.mode, d.act, d.batch = int(mode), int(act), B
    d.S, d.W, d.Mo, d.Fi, d.Hq = int(S), int(W), int(Mo), int(Fi), int(Hq)
    _native.check(_lib().mbg_fno_spectral_layer(C.byref(d), _stream()))


def mode_blocks(wr, wi, blk):
    modes, width = wr.shape[0], wr.shape[1]
    if blk.dtype != torch.bfloat16 or blk.numel() < modes * 4 * width * width:
        raise ValueError("mode_blocks: BF16 output of modes x 2w x 2w")
    _native.check(_lib().mbg_fno_mode_blocks(
        _ptr(wr), _ptr(wi), modes, width, _ptr(blk), _stream()))


def cast_bf16(x, y):
    if x.numel() != y.numel() or y.dtype != torch.bfloat16:
        raise ValueError("cast_bf16: sizes or dtype")
    _native.check(_lib().mbg_fno_cast_bf16(_ptr(x), _ptr(y), x.numel(),
                                           _stream()))


def image_bf16(x, batch, rows, cols, ld, zs, R, K, img):
    """img[z] = BF16 K-major core-matrix image of the R x K matrix with
    entries x[z zs + r ld + c] (r < rows, c < cols; zero elsewhere)."""
    if x.dtype != torch.float32 or img.dtype != torch.bfloat16:
        raise ValueError("image_bf16: FP32 input, BF16 image")
    _check_span(x, 0, [(batch, zs), (rows, ld), (cols, 1)], "image_bf16 x")
    if img.numel() < batch * R * K or not img.is_contiguous():
        raise ValueError("image_bf16: image too small")
    _native.check(_lib().mbg_fno_image_bf16(_ptr(x), batch, rows, cols, ld,
                                            zs, R, K, _ptr(img), _stream()))


def colsum(x, rows, cols, row_stride, out):
    _check_span(x, 0, [(rows, row_stride), (cols, 1)], "colsum x")
    if out.numel() < cols:
        raise ValueError("colsum: out too small")
    _native.check(_lib().mbg_fno_colsum(_ptr(x), rows, cols, row_stride,
                                        _ptr(out), _stream()))


def mse(y, t, grad, loss):
    n = y.numel()
    if t.numel() != n or grad.numel() != n or loss.numel() < 1:
        raise ValueError("mse: sizes")
    _native.check(_lib().mbg_fno_mse(_ptr(y), _ptr(t), n, _ptr(grad),
                                     _ptr(loss), _stream()))


def adam(w, g, m, v, lr, beta1, beta2, eps, weight_decay, step):
    n = w.numel()
    if not (g.numel() == m.numel() == v.numel() == n):
        raise ValueError("adam: sizes")
    _native.check(_lib().mbg_fno_adam(_ptr(w), _ptr(g), _ptr(m), _ptr(v), n,
                                      lr, beta1, beta2, eps, weight_decay,
                                      int(step), _stream()))


def envelope(e, t0, dt, f0, nout, tout0, dtout, out):
    """e: [runs, rows] FP64 CUDA tensor; out: [runs, nout] FP32."""
    runs, rows = e.shape
    if e.dtype != torch.float64 or not e.is_contiguous():
        raise ValueError("envelope: contiguous FP64 input")
    if out.shape != (runs, nout) or out.dtype != torch.float32:
        raise ValueError("envelope: FP32 output [runs, nout]")
    _native.check(_lib().mbg_fno_envelope(
        _ptr(e), runs, rows, rows, t0, dt, f0, nout, tout0, dtout, _ptr(out),
        _stream()))


def status():
    s = C.c_uint32()
    _native.check(_lib().mbg_fno_status(C.byref(s)))
    return s.value
