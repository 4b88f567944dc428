"""Fourier-neural-operator surrogate of the Maxwell-Bloch solver.

Maps an input pulse envelope (S samples) and medium parameters to the
transmitted envelope at the output facet, to prescreen parameter sweeps; the
solver stays the fallback and the judge of its error. The network is a 1-D
Fourier neural operator (Li et al., ICLR 2021): a lifting layer, L Fourier
layers (truncated real DFT to Mo modes, complex mode mixing, inverse DFT,
plus a pointwise channel mix; GELU between layers) and a two-layer
projection. It has no counterpart in the reference.

All arithmetic runs in this package's kernels (include/mbsolve_fno.h): every
product, forward and backward, is one launch of the tcgen05 tensor-core
GEMM (BF16 operands, FP32 accumulation), fused with its bias / GELU /
GELU-derivative epilogue; the truncated DFT and its inverse are products
with fixed BF16 bases. Master weights, gradients and Adam moments are FP32
in one flat buffer each. torch provides device memory and the stream only.

Layouts (row-major, element strides): activations v_l [B, S, W] BF16,
pre-activations [B, S, W] FP32, spectra Vh [B, W, 2 Mo] FP32 (Re modes then
Im modes), mixed spectra Y [B, Mo, 2 W] FP32, mode blocks [Mo, 2W, 2W] BF16.
"""
import math

import numpy as np
import torch

from . import capi_types as T
from . import surrogate_kernels as K
from .surrogate_kernels import Seg


class Shapes:
    """Network sizes: samples S, width W, modes Mo, layers L, input
    features F (envelope, medium parameters, grid coordinate), projection
    width Hq."""

    def __init__(self, S=1024, W=64, Mo=32, L=4, F=8, Hq=128):
        self.S, self.W, self.Mo, self.L, self.F, self.Hq = S, W, Mo, L, F, Hq
        if W % 8 or Mo % 8:
            raise ValueError("width and modes must be multiples of 8")
        if 2 * Mo > S // 2 + 1:
            raise ValueError("too many modes for S samples")

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


def dft_bases(S, Mo):
    """Truncated real DFT and its inverse (float64):
    F [2Mo, S] = [cos(2 pi m s / S); -sin(2 pi m s / S)] / S and
    G [S, 2Mo] = [c_m cos, -c_m sin] with c_0 = 1, c_m = 2, so that
    G F x is x low-passed to its first Mo harmonics."""
    s = np.arange(S)[None, :]
    m = np.arange(Mo)[:, None]
    ang = 2.0 * math.pi * m * s / S
    F = np.concatenate([np.cos(ang), -np.sin(ang)], axis=0) / S
    c = np.where(np.arange(Mo) == 0, 1.0, 2.0)[None, :]
    G = np.concatenate([c * np.cos(ang.T), -c * np.sin(ang.T)], axis=1)
    return np.ascontiguousarray(F), np.ascontiguousarray(G)


def init_params(sh, seed=0):
    """Seeded initialisation: linear layers uniform in +-1/sqrt(fan_in),
    spectral weights uniform in [0, 1) / W^2."""
    rng = np.random.default_rng(seed)
    out = []
    for name, shape in sh.param_spec():
        if name.startswith(("wr", "wi")):
            a = rng.uniform(0.0, 1.0, size=shape) / (sh.W * sh.W)
        elif name in ("P", "Q1") or (name[0] == "W" and name[1:].isdigit()):
            a = rng.uniform(-1, 1, size=shape) / math.sqrt(shape[1])
        elif name == "q2":
            a = rng.uniform(-1, 1, size=shape) / math.sqrt(sh.Hq)
        else:
            fan = {"bp": sh.F, "bq1": sh.W, "bq2": sh.Hq}.get(name, sh.W)
            a = rng.uniform(-1, 1, size=shape) / math.sqrt(fan)
        out.append(a.ravel())
    return np.concatenate(out)


class FNO:
    """The network on one GPU. forward(X) -> y; backward(dy) fills grad;
    train_step(X, t) runs forward, loss, backward and one Adam step."""

    def __init__(self, shapes=None, seed=0, device="cuda"):
        self.sh = sh = shapes or Shapes()
        self.dev = torch.device(device)
        n = sh.num_params()
        self.theta = torch.tensor(init_params(sh, seed), dtype=torch.float32,
                                  device=self.dev)
        self.grad = torch.zeros(n, dtype=torch.float32, device=self.dev)
        self.m1 = torch.zeros_like(self.grad)
        self.m2 = torch.zeros_like(self.grad)
        self.step_count = 0
        self.p = self._views(self.theta)
        self.g = self._views(self.grad)
        F, G = dft_bases(sh.S, sh.Mo)
        self.F = torch.tensor(F, dtype=torch.float32).to(torch.bfloat16).to(self.dev).contiguous()
        self.G = torch.tensor(G, dtype=torch.float32).to(torch.bfloat16).to(self.dev).contiguous()
        self.blk = [torch.empty(sh.Mo * 4 * sh.W * sh.W, dtype=torch.bfloat16,
                                device=self.dev) for _ in range(sh.L)]
        self._bufs = {}
        self._ibufs = {}
        self._blk_valid = False
        self._wb = {}   # BF16 copies of the dense weights (inference)
        self._img = {}  # BF16 tile images for the fused layer kernel

    # ------------------------------------------------------------ helpers
    def _views(self, flat):
        out, o = {}, 0
        for name, shape in self.sh.param_spec():
            k = int(np.prod(shape))
            out[name] = flat[o:o + k]
            o += k
        return out

    def load_params(self, theta):
        self.theta.copy_(torch.as_tensor(theta, dtype=torch.float32))
        self._blk_valid = False

    def _buffers(self, B):
        if B in self._bufs:
            return self._bufs[B]
        sh, d = self.sh, self.dev
        S, W, Mo, L, Hq = sh.S, sh.W, sh.Mo, sh.L, sh.Hq
        f32, b16 = torch.float32, torch.bfloat16
        b = dict(
            v=[torch.empty(B * S * W, dtype=b16, device=d) for _ in range(L + 1)],
            pre=[torch.empty(B * S * W, dtype=f32, device=d) for _ in range(L - 1)],
            Vh=[torch.empty(B * W * 2 * Mo, dtype=f32, device=d) for _ in range(L)],
            Y=torch.empty(B * Mo * 2 * W, dtype=f32, device=d),
            ph=torch.empty(B * S * Hq, dtype=f32, device=d),
            h=torch.empty(B * S * Hq, dtype=b16, device=d),
            y=torch.empty(B * S, dtype=f32, device=d),
            dy=torch.empty(B * S, dtype=f32, device=d),
            dh=torch.empty(B * S * Hq, dtype=f32, device=d),
            dpre=[torch.empty(B * S * W, dtype=f32, device=d) for _ in range(2)],
            dY=torch.empty(B * 2 * Mo * W, dtype=f32, device=d),
            dVh=torch.empty(B * W * 2 * Mo, dtype=f32, device=d),
            loss=torch.zeros(1, dtype=f32, device=d),
        )
        self._bufs[B] = b
        return b

    def _mode_blocks(self):
        for l in range(self.sh.L):
            K.mode_blocks(self.p["wr%d" % l].view(self.sh.Mo, self.sh.W, self.sh.W),
                          self.p["wi%d" % l], self.blk[l])
        # BF16 copies of the dense weights for infer() (the same rounding the
        # products apply to the FP32 weights when they load them)
        for name in ["W%d" % l for l in range(self.sh.L)] + ["Q1", "q2"]:
            w = self._wb.get(name)
            if w is None:
                w = self._wb[name] = torch.empty(self.p[name].numel(), dtype=torch.bfloat16,
                                                 device=self.dev)
            K.cast_bf16(self.p[name], w)
        if self.fused_ok():
            self._layer_images()
        self._blk_valid = True

    @staticmethod
    def _split(rows):
        """K splits of a weight-gradient product over `rows` rows (two
        64-row K blocks per CTA)."""
        return max(1, min(1024, rows // 128))

    # the truncated DFT and its gradient contract over the S samples: split
    # K 8 ways (atomic FP32 accumulation) so that B x 8 CTAs share the work
    DFT_SPLIT = 8

    # ------------------------------------------------------------ forward
    def forward(self, X):
        """X: FP32 CUDA tensor [B, S, F]. Returns y [B, S] (FP32, a view of
        an internal buffer: copy it to keep it past the next call)."""
        sh = self.sh
        S, W, Mo, L, Fi, Hq = sh.S, sh.W, sh.Mo, sh.L, sh.F, sh.Hq
        B = X.shape[0]
        if tuple(X.shape) != (B, S, Fi) or X.dtype != torch.float32:
            raise ValueError("X must be FP32 [B, %d, %d]" % (S, Fi))
        X = X.contiguous()
        b = self._buffers(B)
        p = self.p
        if not self._blk_valid:
            self._mode_blocks()
        self._X = X
        # lifting: v0 = X P^T + bp
        K.gemm(B * S, W, [Seg(X, 0, Fi, 1, 0, p["P"], 0, Fi, 1, 0, Fi)],
               b["v"][0], 0, W, 1, bias=p["bp"])
        for l in range(L):
            v, vh = b["v"][l], b["Vh"][l]
            # truncated DFT: Vh[b, c, m'] = sum_s F[m', s] v[b, s, c]
            vh.zero_()
            K.gemm(W, 2 * Mo, [Seg(v, 0, 1, W, S * W, self.F, 0, S, 1, 0, S)],
                   vh, 0, 2 * Mo, 1, W * 2 * Mo, batch=B,
                   mode=T.MBG_GEMM_ATOMIC, split_k=self.DFT_SPLIT)
            # mode mixing, per mode m: Y[b, m, :] = blk[m] [Re; Im]
            blk = self.blk[l]
            K.gemm(B, 2 * W,
                   [Seg(vh, 0, W * 2 * Mo, 2 * Mo, 1, blk, 0, 2 * W, 1, 4 * W * W, W),
                    Seg(vh, Mo, W * 2 * Mo, 2 * Mo, 1, blk, W, 2 * W, 1, 4 * W * W, W)],
                   b["Y"], 0, Mo * 2 * W, 1, 2 * W, batch=Mo)
            # inverse DFT + pointwise path + bias (+ GELU), per sample
            last = l == L - 1
            K.gemm(S, W,
                   [Seg(self.G, 0, 2 * Mo, 1, 0, b["Y"], 0, 1, 2 * W, Mo * 2 * W, Mo),
                    Seg(self.G, Mo, 2 * Mo, 1, 0, b["Y"], W, 1, 2 * W, Mo * 2 * W, Mo),
                    Seg(v, 0, W, 1, S * W, p["W%d" % l], 0, W, 1, 0, W)],
                   b["v"][l + 1], 0, W, 1, S * W, batch=B, bias=p["bw%d" % l],
                   act=T.MBG_ACT_NONE if last else T.MBG_ACT_GELU,
                   pre=None if last else b["pre"][l])
        # projection
        K.gemm(B * S, Hq, [Seg(b["v"][L], 0, W, 1, 0, p["Q1"], 0, W, 1, 0, W)],
               b["h"], 0, Hq, 1, bias=p["bq1"], act=T.MBG_ACT_GELU, pre=b["ph"])
        K.gemm(B * S, 1, [Seg(b["h"], 0, Hq, 1, 0, p["q2"], 0, 0, 1, 0, Hq)],
               b["y"], 0, 1, 1, bias=p["bq2"])
        return b["y"].view(B, S)

    def _ibuffers(self, B):
        if B in self._ibufs:
            return self._ibufs[B]
        sh, d = self.sh, self.dev
        S, W, Mo, Hq = sh.S, sh.W, sh.Mo, sh.Hq
        b16 = torch.bfloat16
        b = dict(
            v=[torch.empty(B * S * W, dtype=b16, device=d) for _ in range(2)],
            vT=[torch.empty(B * W * S, dtype=b16, device=d) for _ in range(2)],
            Vh=torch.empty(B * W * 2 * Mo, dtype=torch.float32, device=d),
            VhT=torch.empty(B * 2 * Mo * W, dtype=b16, device=d),
            Y=torch.empty(B * W * 2 * Mo, dtype=b16, device=d),
            y=torch.empty(B * S, dtype=torch.float32, device=d))
        self._ibufs[B] = b
        return b

    def fused_ok(self):
        """Whether infer() can run each Fourier layer as one fused launch
        (mbg_fno_spectral_layer): S a multiple of 128, W <= 64, 2 Mo <= 64,
        Hq <= 128 and F <= 16."""
        sh = self.sh
        return (sh.S % 128 == 0 and sh.W <= 64 and 2 * sh.Mo <= 64
                and sh.Hq <= 128 and sh.F <= 16)

    def _layer_images(self):
        """BF16 tile images for the fused layer kernel: the DFT bases (once)
        and the dense weights (after every parameter change)."""
        sh = self.sh
        S, W, Mo, Hq = sh.S, sh.W, sh.Mo, sh.Hq
        T, b16, d = S // 128, torch.bfloat16, self.dev
        im = self._img
        if "G" not in im:
            F, G = dft_bases(S, Mo)
            F32 = torch.tensor(F, dtype=torch.float32, device=d)
            G32 = torch.tensor(G, dtype=torch.float32, device=d)
            im["G"] = torch.empty(T * 8192, dtype=b16, device=d)
            im["F"] = torch.empty(T * 8192, dtype=b16, device=d)
            K.image_bf16(G32, T, 128, 2 * Mo, 2 * Mo, 128 * 2 * Mo, 128, 64, im["G"])
            K.image_bf16(F32, T, 2 * Mo, 128, S, 128, 64, 128, im["F"])
        for l in range(sh.L):
            name = "W%d" % l
            if name not in im:
                im[name] = torch.empty(64 * 64, dtype=b16, device=d)
            K.image_bf16(self.p[name], 1, W, W, W, 0, 64, 64, im[name])
        if "Q1" not in im:
            im["Q1"] = torch.empty(128 * 64, dtype=b16, device=d)
            im["P"] = torch.empty(64 * 16, dtype=b16, device=d)
        K.image_bf16(self.p["Q1"], 1, Hq, W, W, 0, 128, 64, im["Q1"])
        K.image_bf16(self.p["P"], 1, W, sh.F, sh.F, 0, 64, 16, im["P"])

    def _fbuffers(self, B):
        key = ("fused", B)
        if key in self._ibufs:
            return self._ibufs[key]
        sh, d = self.sh, self.dev
        S, W, Mo = sh.S, sh.W, sh.Mo
        b16 = torch.bfloat16
        b = dict(
            v=[torch.empty(B * S * 64, dtype=b16, device=d) for _ in range(2)],
            VhT=torch.empty(B * 2 * Mo * W, dtype=b16, device=d),
            Y=torch.empty(B * 2 * W * Mo, dtype=b16, device=d),
            y=torch.empty(B * S, dtype=torch.float32, device=d))
        self._ibufs[key] = b
        return b

    def infer(self, X):
        """The forward pass for inference (prescreening sweeps): the same
        network and the same BF16 rounding of every product operand as
        forward(). Where the sizes allow (fused_ok), each Fourier layer is
        one launch that keeps its products on chip: the lifting with the
        first truncated DFT; the inverse DFT, pointwise mix, bias and GELU
        with the next DFT; the last layer with the projection and the
        output layer. Between them two products per layer mix the modes of
        all samples (M = batch, N = W, per mode; the Re and the Im outputs),
        writing the mixed spectrum as BF16 [B, 2, Mo, W]. Activations pass between the fused
        launches as BF16 tile images (the layout their products read), the
        DFT bases and dense weights likewise (_layer_images). Otherwise the
        products of _infer_products run. X: FP32 [B, S, F]; returns y [B, S] (a view of
        an internal buffer)."""
        sh = self.sh
        S, W, Mo, L, Fi, Hq = sh.S, sh.W, sh.Mo, sh.L, sh.F, sh.Hq
        B = X.shape[0]
        if tuple(X.shape) != (B, S, Fi) or X.dtype != torch.float32:
            raise ValueError("X must be FP32 [B, %d, %d]" % (S, Fi))
        if not self.fused_ok():
            return self._infer_products(X)
        X = X.contiguous()
        b = self._fbuffers(B)
        p = self.p
        if not self._blk_valid:
            self._mode_blocks()
        im = self._img
        vhT, Y = b["VhT"], b["Y"]
        K.spectral_layer(T.MBG_LAYER_LIFT, T.MBG_ACT_NONE, B, S, W, Mo, Fi=Fi,
                         X=X, P=im["P"], bias=p["bp"], v_out=b["v"][0],
                         F=im["F"], vhT=vhT)
        cur = 0
        for l in range(L):
            # mode mixing per mode m, the Re and the Im outputs:
            # Y[b, part, m, :] = blk[m][part] [Re; Im] (contiguous stores)
            blk = self.blk[l]
            for part in range(2):
                K.gemm(B, W,
                       [Seg(vhT, 0, 2 * Mo * W, 1, W, blk, part * W * 2 * W,
                            2 * W, 1, 4 * W * W, W),
                        Seg(vhT, Mo * W, 2 * Mo * W, 1, W, blk,
                            part * W * 2 * W + W, 2 * W, 1, 4 * W * W, W)],
                       Y, part * Mo * W, 2 * Mo * W, 1, W, batch=Mo)
            if l < L - 1:
                K.spectral_layer(T.MBG_LAYER_MID, T.MBG_ACT_GELU, B, S, W, Mo,
                                 v=b["v"][cur], Y=Y, G=im["G"], Wl=im["W%d" % l],
                                 bias=p["bw%d" % l], v_out=b["v"][1 - cur],
                                 F=im["F"], vhT=vhT)
                cur = 1 - cur
            else:
                K.spectral_layer(T.MBG_LAYER_LAST, T.MBG_ACT_NONE, B, S, W, Mo,
                                 Hq=Hq, v=b["v"][cur], Y=Y, G=im["G"],
                                 Wl=im["W%d" % l], bias=p["bw%d" % l],
                                 Q1=im["Q1"], bq1=p["bq1"], q2=p["q2"],
                                 bq2=p["bq2"], y=b["y"])
        return b["y"].view(B, S)

    def _infer_products(self, X):
        """infer() for sizes the fused layer kernel does not take, as
        products of the general kernel: the same network and the same BF16
        rounding of every product operand as forward(), with the operands
        laid out so that every heavy product
        reads BF16 with K contiguous (the GEMM then stages them by
        asynchronous copies, four stages deep): each activation is kept as
        [B, S, W] and, written by the same epilogue, as [B, W, S]; the mixed
        spectrum as BF16 [B, W, 2 Mo]; the spectrum also as BF16
        [B, 2 Mo, W] for the mixing; BF16 copies of the dense weights. The
        truncated DFT runs without split-K (K = S per sample); the output
        layer is folded into the hidden projection's epilogue; no
        pre-activations are stored. X: FP32 [B, S, F]; returns
        y [B, S] (a view of an internal buffer)."""
        sh = self.sh
        S, W, Mo, L, Fi, Hq = sh.S, sh.W, sh.Mo, sh.L, sh.F, sh.Hq
        B = X.shape[0]
        X = X.contiguous()
        b = self._ibuffers(B)
        p = self.p
        if not self._blk_valid:
            self._mode_blocks()
        wb = self._wb
        # lifting, per sample: v0[b] = X[b] P^T + bp, also as vT0[b] [W, S]
        K.gemm(S, W, [Seg(X, 0, Fi, 1, S * Fi, p["P"], 0, Fi, 1, 0, Fi)],
               b["v"][0], 0, W, 1, S * W, batch=B, bias=p["bp"],
               c2=b["vT"][0], c2_sm=1, c2_sn=S, c2_sz=W * S)
        cur = 0
        for l in range(L):
            v, vT = b["v"][cur], b["vT"][cur]
            vh, vhT, Y = b["Vh"], b["VhT"], b["Y"]
            # truncated DFT per sample: Vh[b](c, m') = vT[b](c, :) F(m', :),
            # also as BF16 VhT[b](m', c), the mixing's operand with K contiguous
            K.gemm(W, 2 * Mo, [Seg(vT, 0, S, 1, W * S, self.F, 0, S, 1, 0, S)],
                   vh, 0, 2 * Mo, 1, W * 2 * Mo, batch=B,
                   c2=vhT, c2_sm=1, c2_sn=W, c2_sz=2 * Mo * W)
            # mode mixing per mode m, the Re and the Im outputs into
            # Y[b, o, m] and Y[b, o, Mo + m] (BF16)
            blk = self.blk[l]
            for part in range(2):
                K.gemm(B, W,
                       [Seg(vhT, 0, 2 * Mo * W, 1, W, blk, part * W * 2 * W,
                            2 * W, 1, 4 * W * W, W),
                        Seg(vhT, Mo * W, 2 * Mo * W, 1, W, blk,
                            part * W * 2 * W + W, 2 * W, 1, 4 * W * W, W)],
                       Y, part * Mo, W * 2 * Mo, 2 * Mo, 1, batch=Mo)
            # inverse DFT + pointwise path + bias (+ GELU), per sample,
            # written as [S, W] and as [W, S]
            last = l == L - 1
            nxt = 1 - cur
            K.gemm(S, W,
                   [Seg(self.G, 0, 2 * Mo, 1, 0, Y, 0, 2 * Mo, 1, W * 2 * Mo, 2 * Mo),
                    Seg(v, 0, W, 1, S * W, wb["W%d" % l], 0, W, 1, 0, W)],
                   b["v"][nxt], 0, W, 1, S * W, batch=B, bias=p["bw%d" % l],
                   act=T.MBG_ACT_NONE if last else T.MBG_ACT_GELU,
                   c2=None if last else b["vT"][nxt], c2_sm=1, c2_sn=S,
                   c2_sz=W * S)
            cur = nxt
        # projection: y = q2 . GELU(v Q1^T + bq1) + bq2, the second product
        # folded into the first one's epilogue (no hidden activation stored)
        b["y"].zero_()
        K.gemm(B * S, Hq, [Seg(b["v"][cur], 0, W, 1, 0, wb["Q1"], 0, W, 1, 0, W)],
               b["y"], 0, 1, 0, bias=p["bq1"], act=T.MBG_ACT_GELU,
               rowdot=p["q2"], rowdot_bias=p["bq2"])
        return b["y"].view(B, S)

    # ------------------------------------------------------------ backward
    def backward(self, dy=None):
        """Gradient of the loss into self.grad (zeroed first). dy: FP32
        [B, S] gradient of the loss w.r.t. the last forward's output, or
        None when loss() already wrote it."""
        sh = self.sh
        S, W, Mo, L, Fi, Hq = sh.S, sh.W, sh.Mo, sh.L, sh.F, sh.Hq
        X = self._X
        B = X.shape[0]
        if B % 8:
            raise ValueError("backward needs a batch that is a multiple of 8")
        b = self._buffers(B)
        p, g = self.p, self.g
        if dy is not None:
            b["dy"].copy_(dy.reshape(-1))
        dyb = b["dy"]
        R = B * S
        self.grad.zero_()
        ATOM = T.MBG_GEMM_ATOMIC
        # output layer
        K.gemm(Hq, 1, [Seg(b["h"], 0, 1, Hq, 0, dyb, 0, 0, 1, 0, R)],
               g["q2"], 0, 1, 1, mode=ATOM, split_k=self._split(R))
        K.colsum(dyb, R, 1, 1, g["bq2"])
        K.gemm(R, Hq, [Seg(dyb, 0, 1, 1, 0, p["q2"], 0, 1, 1, 0, 1)],
               b["dh"], 0, Hq, 1, act=T.MBG_ACT_GELU_BWD, gate=b["ph"])
        K.gemm(Hq, W, [Seg(b["dh"], 0, 1, Hq, 0, b["v"][L], 0, 1, W, 0, R)],
               g["Q1"], 0, W, 1, mode=ATOM, split_k=self._split(R))
        K.colsum(b["dh"], R, Hq, Hq, g["bq1"])
        cur = 0
        K.gemm(R, W, [Seg(b["dh"], 0, Hq, 1, 0, p["Q1"], 0, 1, W, 0, Hq)],
               b["dpre"][cur], 0, W, 1)
        for l in range(L - 1, -1, -1):
            dpre = b["dpre"][cur]
            vh, blk = b["Vh"][l], self.blk[l]
            K.gemm(W, W, [Seg(dpre, 0, 1, W, 0, b["v"][l], 0, 1, W, 0, R)],
                   g["W%d" % l], 0, W, 1, mode=ATOM, split_k=self._split(R))
            K.colsum(dpre, R, W, W, g["bw%d" % l])
            # dY[b, m', o] = sum_s G[s, m'] dpre[b, s, o]
            b["dY"].zero_()
            K.gemm(2 * Mo, W, [Seg(self.G, 0, 1, 2 * Mo, 0, dpre, 0, 1, W, S * W, S)],
                   b["dY"], 0, W, 1, 2 * Mo * W, batch=B,
                   mode=T.MBG_GEMM_ATOMIC, split_k=self.DFT_SPLIT)
            dY = b["dY"]
            a_re = dict(a_sm=1, a_sk=2 * Mo * W, a_sz=W)
            b_v = dict(b_sn=2 * Mo, b_sk=W * 2 * Mo, b_sz=1)

            def sg(a_off, b_off, neg=False):
                return Seg(dY, a_off, a_re["a_sm"], a_re["a_sk"], a_re["a_sz"],
                           vh, b_off, b_v["b_sn"], b_v["b_sk"], b_v["b_sz"], B,
                           negate=neg)
            # spectral weights, per mode
            K.gemm(W, W, [sg(0, 0), sg(Mo * W, Mo)],
                   g["wr%d" % l], 0, 1, W, W * W, batch=Mo)
            K.gemm(W, W, [sg(0, Mo, True), sg(Mo * W, 0)],
                   g["wi%d" % l], 0, 1, W, W * W, batch=Mo)
            # spectra: dVh = blk^T dY, Re and Im halves, per mode
            for half in range(2):
                K.gemm(B, W,
                       [Seg(dY, 0, 2 * Mo * W, 1, W, blk, half * W, 1, 2 * W, 4 * W * W, W),
                        Seg(dY, Mo * W, 2 * Mo * W, 1, W, blk, 2 * W * W + half * W, 1, 2 * W,
                            4 * W * W, W)],
                       b["dVh"], half * Mo, W * 2 * Mo, 2 * Mo, 1, batch=Mo)
            # activations: dv = F^T dVh + dpre W_l, then GELU'
            nxt = 1 - cur
            K.gemm(S, W,
                   [Seg(self.F, 0, 1, S, 0, b["dVh"], 0, 2 * Mo, 1, W * 2 * Mo, 2 * Mo),
                    Seg(dpre, 0, W, 1, S * W, p["W%d" % l], 0, 1, W, 0, W)],
                   b["dpre"][nxt], 0, W, 1, S * W, batch=B,
                   act=T.MBG_ACT_GELU_BWD if l > 0 else T.MBG_ACT_NONE,
                   gate=b["pre"][l - 1] if l > 0 else None)
            cur = nxt
        dv0 = b["dpre"][cur]
        K.gemm(W, Fi, [Seg(dv0, 0, 1, W, 0, X, 0, 1, Fi, 0, R)],
               g["P"], 0, Fi, 1, mode=ATOM, split_k=self._split(R))
        K.colsum(dv0, R, W, W, g["bp"])

    def loss(self, target):
        """Mean squared error of the last forward against target [B, S];
        writes the output gradient for backward(). Returns the loss as a
        one-element CUDA tensor (no synchronisation)."""
        B = self._X.shape[0]
        b = self._buffers(B)
        b["loss"].zero_()
        K.mse(b["y"], target.reshape(-1), b["dy"], b["loss"])
        return b["loss"]

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step_count += 1
        K.adam(self.theta, self.grad, self.m1, self.m2, lr, beta1, beta2, eps,
               weight_decay, self.step_count)
        self._blk_valid = False

    def train_step(self, X, target, lr=1e-3, weight_decay=0.0):
        self.forward(X)
        loss = self.loss(target)
        self.backward()
        self.adam(lr=lr, weight_decay=weight_decay)
        return loss


def main(argv=None):
    """Time training steps (forward, loss, backward, Adam) and inference on
    random inputs: python -m mbsolve_gb300.surrogate [--batch 64]
    [--steps 50] [--samples 1024] [--width 64] [--modes 32] [--layers 4]."""
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description="surrogate step timing")
    ap.add_argument("--batch", type=int, default=64)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--samples", type=int, default=1024)
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--modes", type=int, default=32)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--features", type=int, default=9)
    ap.add_argument("--only", choices=["all", "infer"], default="all",
                    help="infer: time the inference path only")
    a = ap.parse_args(argv)
    sh = Shapes(S=a.samples, W=a.width, Mo=a.modes, L=a.layers, F=a.features)
    net = FNO(sh, seed=0)
    g = torch.Generator(device="cpu").manual_seed(0)
    X = torch.randn(a.batch, sh.S, sh.F, generator=g).cuda()
    t = torch.randn(a.batch, sh.S, generator=g).cuda()
    dt_train = dt_fwd = float("nan")
    loss = torch.zeros(1)
    if a.only == "all":
        for _ in range(3):
            net.train_step(X, t)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            loss = net.train_step(X, t)
        torch.cuda.synchronize()
        dt_train = (time.perf_counter() - t0) / a.steps
        t0 = time.perf_counter()
        for _ in range(a.steps):
            net.forward(X)
        torch.cuda.synchronize()
        dt_fwd = (time.perf_counter() - t0) / a.steps
    net.infer(X)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        net.infer(X)
    torch.cuda.synchronize()
    dt_inf = (time.perf_counter() - t0) / a.steps
    print(json.dumps({"shapes": vars(sh), "batch": a.batch,
                      "train_step_ms": dt_train * 1e3,
                      "forward_ms": dt_fwd * 1e3, "infer_ms": dt_inf * 1e3,
                      "samples_per_s_train": a.batch / dt_train,
                      "samples_per_s_forward": a.batch / dt_fwd,
                      "samples_per_s_infer": a.batch / dt_inf,
                      "loss": float(loss.item()), "status": K.status()}))


if __name__ == "__main__":
    main()
