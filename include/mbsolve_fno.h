/*
 * mbsolve_fno.h - C-ABI of the surrogate's GPU kernels.
 *
 * The surrogate is a Fourier neural operator that maps an input pulse
 * envelope and medium parameters to the transmitted probe envelope. It has
 * no counterpart in the reference (mbsolve has no learned component); the
 * reference's only spectral tool is the FFT helper of its MATLAB scripts.
 * These entry points are the kernels its training and inference run on:
 *
 *   mbg_fno_gemm       BF16 tensor-core product (tcgen05, FP32 accumulator
 *                      in tensor memory) over up to three strided operand
 *                      pairs, with bias / GELU / GELU-derivative epilogues,
 *                      accumulate and split-K atomic modes
 *   mbg_fno_spectral_layer  one Fourier layer of inference in one launch:
 *                      lifting or inverse DFT + pointwise mix, bias, GELU,
 *                      then the next truncated DFT or the projection, the
 *                      intermediate products kept on chip
 *   mbg_fno_mode_blocks  complex spectral weights -> real 2x2 block matrices
 *   mbg_fno_cast_bf16  FP32 -> BF16 copies of the master weights
 *   mbg_fno_colsum     bias gradients (column sums)
 *   mbg_fno_mse        mean squared error and its gradient
 *   mbg_fno_adam       Adam step on FP32 master weights
 *   mbg_fno_envelope   demodulated envelope of recorded probe fields
 *
 * Every pointer argument except `stream` is a device pointer; `stream` is a
 * cudaStream_t (NULL: the legacy default stream). Calls are asynchronous on
 * the stream; argument errors are reported at once, kernel-side failures
 * (a tensor-core wait that ran out) through mbg_fno_status.
 * Status codes and mbg_last_error() are those of mbsolve_gb300.h.
 */
#ifndef MBSOLVE_FNO_H
#define MBSOLVE_FNO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { MBG_F32 = 0, MBG_BF16 = 1 };

enum {
    MBG_GEMM_STORE = 0,   /* C = epilogue(alpha acc) */
    MBG_GEMM_ACCUM = 1,   /* C = epilogue(alpha acc + C) */
    MBG_GEMM_ATOMIC = 2   /* C += alpha acc (FP32 C, atomic; split-K) */
};

enum {
    MBG_ACT_NONE = 0,
    MBG_ACT_GELU = 1,     /* exact GELU, x Phi(x) */
    MBG_ACT_GELU_BWD = 2  /* v * GELU'(gate) */
};

/* One operand pair of a product: element (i, k) of A is at
 * a + z a_sz + i a_sm + k a_sk, element (j, k) of B at
 * b + z b_sz + j b_sn + k b_sk (element strides, z the batch index). */
typedef struct mbg_gemm_segment {
    const void* a;
    const void* b;
    int64_t a_sm, a_sk, a_sz;
    int64_t b_sn, b_sk, b_sz;
    int32_t k;        /* length of this segment's K range */
    int32_t a_type;   /* MBG_F32 or MBG_BF16 */
    int32_t b_type;
    int32_t negate;   /* nonzero: subtract this segment's product */
} mbg_gemm_segment;

/* C[z](i, j) = sum over segments s of sum_k A_s(i, k) B_s(j, k), in BF16
 * products with FP32 accumulation; then the epilogue:
 *   v = alpha acc (+ C if ACCUM) (+ bias[j]); pre[i, j] = v if pre;
 *   GELU: v = gelu(v); GELU_BWD: v = v gelu'(gate[i, j]); store C.
 * pre and gate are FP32 with C's strides. All segments but the last need
 * k % 8 == 0. ATOMIC mode takes no bias, pre or activation and may split K
 * over `split_k` CTAs. */
typedef struct mbg_gemm_desc {
    int32_t m, n, batch;
    int32_t nseg;
    mbg_gemm_segment seg[3];
    void* c;
    int64_t c_sm, c_sn, c_sz;
    int32_t c_type;
    int32_t mode;
    int32_t act;
    int32_t split_k;
    float alpha;
    const float* bias;
    float* pre;
    const float* gate;
    /* optional second output (NULL: none; STORE mode without pre, gate
     * or GELU_BWD): the same values as BF16 at
     * c2 + z c2_sz + i c2_sm + j c2_sn, e.g. the transposed copy of an
     * activation that the next product reads with K contiguous */
    void* c2;
    int64_t c2_sm, c2_sn, c2_sz;
    /* optional (NULL: none; STORE mode without pre, gate or GELU_BWD, an
     * FP32 C, no second output): instead of storing the outputs v(i, j),
     * add sum_j rowdot[j] v(i, j) (both rounded to BF16) to C[z](i, 0),
     * atomically, plus *rowdot_bias once (when not NULL): a following
     * product with one output column folded into this one's epilogue.
     * C must hold the starting values (e.g. zeros). */
    const float* rowdot;
    const float* rowdot_bias;
} mbg_gemm_desc;

int mbg_fno_gemm(const mbg_gemm_desc* d, void* stream);

enum {
    MBG_LAYER_LIFT = 0,   /* lifting, then the first layer's truncated DFT */
    MBG_LAYER_MID = 1,    /* inverse DFT + pointwise mix, then the next DFT */
    MBG_LAYER_LAST = 2    /* inverse DFT + pointwise mix, then the projection */
};

/* One Fourier layer of inference for every sample in one launch, the
 * layer's products kept on chip (one CTA per SM owns whole samples).
 * Tile images: a matrix stored as its K-major core-matrix image, element
 * (r, k) of an R x K block at ((r/8) (K/8) + k/8) 64 + (r%8) 8 + k%8
 * (mbg_fno_image_bf16 writes them). T = S / 128 tiles per sample.
 *   v, v_out  activations: for sample b and tile i the 128 x 64 image of
 *             rows 128 i .. 128 i + 127 (channels W..63 zero) at
 *             (b T + i) 8192 (BF16, B S 64 elements)
 *   G         inverse DFT basis [S][2 Mo]: the 128 x 64 image of tile i's
 *             rows at i 8192 (columns 2 Mo..63 zero)
 *   F         forward DFT basis [2 Mo][S]: the 64 x 128 image of tile i's
 *             columns at i 8192 (rows 2 Mo..63 zero)
 *   Wl        pointwise weights [W][W]: their 64 x 64 image
 *   Q1        projection weights [Hq][W]: their 128 x 64 image
 *   P         lifting weights [W][Fi]: their 64 x 16 image
 * Plain layouts (row-major): X [B][S][Fi] FP32,
 * Y [B][2][Mo][W] BF16 (Re then Im of the mixed spectrum), bias [W] FP32
 * (NULL: zero), vhT [B][2 Mo][W] BF16, bq1, q2 [Hq], bq2 [1], y [B][S]
 * FP32. Every pointer 16-byte aligned.
 * Arithmetic: every product operand rounded to BF16, FP32 accumulation.
 *   u(s, o) = sum_f X(s, f) P(o, f) + bias(o)                      (LIFT)
 *   u(s, o) = sum_m G(s, m) Y(o, m) + sum_c v(s, c) Wl(o, c) + bias(o)
 *             with Y(o, m) = Y[p][m mod Mo][o], p = m / Mo    (MID, LAST)
 *   then u = GELU(u) when act is MBG_ACT_GELU, and
 *   LIFT, MID: v_out = BF16(u); vhT(m, c) = BF16(sum_s F(m, s) v_out(s, c))
 *   LAST: h(s, j) = sum_c BF16(u(s, c)) Q1(j, c) + bq1(j),
 *         y(s) = sum_j BF16(GELU(h(s, j))) q2(j) + bq2
 * Sizes: S a positive multiple of 128; W in 8..64 and Mo in 8..32, both
 * multiples of 8; Fi in 1..16 (LIFT); Hq in 1..128 (LAST). */
typedef struct mbg_fno_layer_desc {
    int32_t mode;     /* MBG_LAYER_* */
    int32_t act;      /* MBG_ACT_NONE or MBG_ACT_GELU */
    int32_t batch, S, W, Mo, Fi, Hq;
    const float* X;
    const void* P;
    const void* v;
    const void* Y;
    const void* G;
    const void* Wl;
    const float* bias;
    void* v_out;
    const void* F;
    void* vhT;
    const void* Q1;
    const float* bq1;
    const float* q2;
    const float* bq2;
    float* y;
} mbg_fno_layer_desc;

int mbg_fno_spectral_layer(const mbg_fno_layer_desc* d, void* stream);

/* Spectral weights of one layer, wr/wi [modes][width c][width o] (FP32),
 * as the real block matrices blk[modes][2 width][2 width] (BF16) with
 * [Re y; Im y] = blk [Re x; Im x] for y_o = sum_c (wr + i wi)[c][o] x_c. */
int mbg_fno_mode_blocks(const float* wr, const float* wi, int32_t modes,
                        int32_t width, void* blk, void* stream);

int mbg_fno_cast_bf16(const float* x, void* y, int64_t n, void* stream);

/* K-major core-matrix image (the operand layout of
 * mbg_fno_spectral_layer): for z < batch, the R x K matrix whose (r, c)
 * entry is x[z zs + r ld + c] for r < rows, c < cols and zero elsewhere,
 * as BF16 at img + z R K with (r, c) at ((r/8) (K/8) + c/8) 64 +
 * (r%8) 8 + c%8. R, K multiples of 8. */
int mbg_fno_image_bf16(const float* x, int32_t batch, int32_t rows,
                       int32_t cols, int64_t ld, int64_t zs, int32_t R,
                       int32_t K, void* img, void* stream);

/* out[j] += sum_i x[i row_stride + j], i < rows, j < cols (FP32) */
int mbg_fno_colsum(const float* x, int64_t rows, int32_t cols,
                   int64_t row_stride, float* out, void* stream);

/* loss[0] += sum (y - t)^2 / n; grad = 2 (y - t) / n */
int mbg_fno_mse(const float* y, const float* t, int64_t n, float* grad,
                float* loss, void* stream);

/* Adam (bias-corrected, step >= 1) with decoupled weight decay */
int mbg_fno_adam(float* w, const float* g, float* m, float* v, int64_t n,
                 float lr, float beta1, float beta2, float eps,
                 float weight_decay, int32_t step, void* stream);

/* Envelope of recorded fields e[r][i] (FP64, rows i = 0..rows-1 at times
 * t0 + i dt): out[r][j] = 2 |mean of e(t) exp(-2 pi i f0 t)| over the
 * samples within half a carrier period of t_j = tout0 + j dtout. */
int mbg_fno_envelope(const double* e, int32_t runs, int32_t rows,
                     int64_t run_stride, double t0, double dt, double f0,
                     int32_t nout, double tout0, double dtout, float* out,
                     void* stream);

/* Kernel-side status since the last call (bit 0: a tensor-core wait ran
 * out; bit 1: TMEM allocation refused); cleared by the call. */
int mbg_fno_status(uint32_t* status);

#ifdef __cplusplus
}
#endif

#endif
