// One Fourier layer of surrogate inference per launch
// (include/mbsolve_fno.h, mbg_fno_spectral_layer).
//
// The layer's products never leave the SM between them. A CTA owns whole
// samples (one CTA per SM, the samples strided over the CTAs) and walks
// each sample's S rows in tiles of 128:
//
//   first product   MID/LAST: acc = G Y^T + v Wl^T on the tensor cores
//                   (two K = 64 operand pairs, tcgen05.mma, FP32 in TMEM);
//                   LIFT: acc = X P^T (K = Fi <= 16, padded to 16)
//   epilogue        u = acc + bias, GELU, rounded to BF16 once; stored as
//                   the next activation v_out (MID, LIFT) and written into
//                   shared memory as an MMA operand
//   second product  MID/LIFT: the truncated DFT of v_out, accumulated over
//                   the sample's tiles in TMEM (D = F_tile vT_tile^T) and
//                   stored as vhT [2 Mo][W] when the sample ends, the next
//                   mode mixing's operand; LAST: the hidden projection
//                   H = v_tile Q1^T, whose epilogue reduces GELU(H + bq1)
//                   against q2 into the output y
//
// Warp roles, coupled only by mbarriers (no block-wide barrier inside the
// tile loop): warp 16 stages operands by bulk copies (TMA engine, one
// instruction per 16 KB tile image) into rings of two (G, v) pairs (six X
// tiles for the lifting, which the epilogue warps convert into BF16
// operand images two tiles ahead) and four DFT-basis tiles, and transposes
// a sample's mixed spectrum Y into its operand image; one thread of warp 17
// issues the MMAs into two first-product and two
// second-product TMEM accumulators; warps 0-15 run the epilogues (warp w
// reads TMEM lanes 32 (w % 4) .. +31, columns 16 (w / 4) .. +15) and write
// each output tile as an image in shared memory that one bulk copy stores.
// Activations, the DFT bases and the dense weights are kept as K-major
// core-matrix images (8 rows x 16 bytes per core matrix, no swizzle), the
// layout the MMA reads, so a tile moves between HBM and shared memory as
// one contiguous block. The transposed activation tile (K = samples) is
// written by 2-byte stores; its K-direction core matrices are 144 bytes
// apart instead of 128, so that a warp's stores of one channel for 32
// consecutive samples land in four distinct bank groups. The DFT product
// has M = 64 mode rows; it is issued as M = 128, and the 64 rows above the
// basis tile read whatever lies behind it in shared memory: they only feed
// TMEM lanes 64-127, which nothing reads. Every wait is bounded; when one
// runs out the kernel raises an abort flag that ends every other wait,
// records the failure in the status word and returns after freeing its
// TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "fno_common.cuh"

namespace mbg {
namespace fno {
namespace {

constexpr int LT = 128;                   // rows (samples s) per tile
constexpr int NEPI = 512;                 // epilogue threads: warps 0-15
constexpr int PROD_WARP = 16, MMA_WARP = 17;
constexpr int LNTH = 576;

constexpr int IMG = 128 * 64 * 2;         // 128 x 64 BF16 image: v, G, projection input, Q1
constexpr int F_IMG = 64 * LT * 2;        // 64 mode rows x 128 samples
constexpr int B_IMG = 64 * 64 * 2;        // Y or Wl
constexpr int IMG_ELEMS = IMG / 2;
constexpr int NGV = 2, NX = 6, NFR = 4, NYR = 2;  // ring depths: (G, v) pairs, X tiles (LIFT), basis tiles, Y
constexpr int X_SLOT = LT * 16 * 4;       // lifting input tile: 128 rows x <= 16 FP32 features
constexpr int NXI = 3;                    // ring of lifting input images (BF16, 128 x 16)
constexpr int XI_IMG = LT * 16 * 2;
constexpr int OFF_XI = NX * X_SLOT;       // after the X tiles, in the first ring's space
constexpr uint32_t VT_LBO = 144;          // transposed tile: K-direction core-matrix stride
constexpr uint32_t VT_SBO = 16 * VT_LBO;  // 8-channel group stride
constexpr int VT_IMG = 8 * VT_SBO;        // 64 channel rows x 128 samples

// shared memory map (bytes from a 128-aligned base); LAST keeps Q1 in the
// basis ring and its two projection-input images where the transposed
// tiles are
constexpr int GV_SLOT = 2 * IMG;
constexpr int OFF_GV = 0;
constexpr int OFF_F = OFF_GV + NGV * GV_SLOT;
constexpr int OFF_Q = OFF_F;
constexpr int OFF_VT = OFF_F + NFR * F_IMG;  // two transposed tiles (LAST: projection inputs)
constexpr int OFF_OUT = OFF_VT + 2 * VT_IMG;  // output image (LIFT, MID)
constexpr int OFF_Y = OFF_OUT + IMG;
constexpr int OFF_W = OFF_Y + NYR * B_IMG;
constexpr int OFF_SMALL = OFF_W + B_IMG;
constexpr int SM_BIAS = 0, SM_BQ1 = 64, SM_Q2 = 192, SM_RED = 320;  // floats
constexpr int SMALL_FLOATS = SM_RED + 2 * 4 * 128;
constexpr int LAYER_SMEM = OFF_SMALL + SMALL_FLOATS * 4 + 128;  // + alignment slack
// the epilogues read bias, bq1 and q2 as float2 pairs at even columns
static_assert(OFF_SMALL % 8 == 0 && SM_BIAS % 2 == 0 && SM_BQ1 % 2 == 0 && SM_Q2 % 2 == 0,
              "small parameters: 8-byte aligned pairs");
// the last basis slot's unread M rows (32 KB from its start) stay inside the map
static_assert(OFF_F + (NFR - 1) * F_IMG + 2 * F_IMG <= OFF_OUT, "basis slot overrun");
static_assert(NX * X_SLOT + NXI * XI_IMG <= NGV * GV_SLOT && IMG <= NFR * F_IMG && IMG <= VT_IMG, "aliases");
static_assert(LAYER_SMEM + 512 <= 227 * 1024, "shared memory");

constexpr uint32_t ID64 = idesc_bf16(128, 64);
constexpr uint32_t ID128 = idesc_bf16(128, 128);
// columns: first-product accumulators at 0 and 64; DFT accumulators at 128
// and 192 (by sample parity); projection accumulators at 256 and 384
constexpr uint32_t LAYER_TMEM_COLS = 512;

// mbarriers: full (data ready) / empty (slot free) pairs
enum {
    B_FGV = 0, B_EGV = 6,    // (G, v) / X ring: bulk bytes / inverse MMA (LIFT: the epilogue warps read X)
    B_FF = 12, B_EF = 16,    // basis ring: bulk bytes / DFT MMA
    B_FY = 20, B_EY = 22,    // Y ring: copy warp / a sample's last inverse MMA
    B_FACC = 24, B_EACC = 26,  // first-product accumulators: MMA / epilogue warps
    B_FOP = 28, B_EOP = 30,  // epilogue-written MMA operand: epilogue warps / second-product MMA
    B_FD = 32, B_ED = 34,    // DFT accumulators: a sample's last DFT MMA / epilogue warps
    B_FH = 36, B_EH = 38,    // projection accumulators: MMA / epilogue warps
    B_FXI = 40, B_EXI = 43,  // lifting input images: copy warp / lifting MMA
    NBAR = 46
};

struct layer_params {
    int32_t mode, act, batch, S, W, Mo, Fi, Hq;
    const float* X;
    const __nv_bfloat16* P;
    const __nv_bfloat16* v;
    const __nv_bfloat16* Y;
    const __nv_bfloat16* G;
    const __nv_bfloat16* Wl;
    const float* bias;
    __nv_bfloat16* v_out;
    const __nv_bfloat16* F;
    __nv_bfloat16* vhT;
    const __nv_bfloat16* Q1;
    const float* bq1;
    const float* q2;
    const float* bq2;
    float* y;
    uint32_t* status;
};

// byte offset of 16-byte chunk (row, kc) in a K-major image with `kch`
// chunks per row (core matrices 128 bytes apart along K)
__device__ __forceinline__ uint32_t koff(int row, int kc, int kch)
{
    return (uint32_t) (((row >> 3) * kch + kc) * 128 + (row & 7) * 16);
}

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

__device__ __forceinline__ void st_shared_u16(uint32_t addr, uint32_t v)
{
    asm volatile("st.shared.b16 [%0], %1;" ::"r"(addr), "h"((unsigned short) v) : "memory");
}

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}

// bounded wait; gives up at once when another wait has run out
__device__ __forceinline__ bool wait_bar(uint32_t mbar, uint32_t parity, volatile int* abort)
{
    for (uint32_t i = 0; i < WAIT_LIMIT; i++) {
        if (mbar_test(mbar, parity)) return true;
        if (*abort) return false;
    }
    *abort = 1;
    return false;
}

// the same, polled by lane 0 for the whole warp
__device__ __forceinline__ bool wait_bar_warp(uint32_t mbar, uint32_t parity, volatile int* abort, int lane)
{
    int ok = 0;
    if (lane == 0) ok = wait_bar(mbar, parity, abort) ? 1 : 0;
    return __shfl_sync(0xFFFFFFFFu, ok, 0) != 0;
}

template<int MODE, bool GELU>
__global__ void __launch_bounds__(LNTH, 1) spectral_layer_kernel(const layer_params p)
{
    extern __shared__ __align__(128) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t mbar[NBAR];
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;

    constexpr bool lift = MODE == MBG_LAYER_LIFT, last = MODE == MBG_LAYER_LAST;
    constexpr int NG = lift ? NX : NGV;  // depth of the first ring
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sb = (smem_u32(smem_raw) + 127u) & ~127u;
    uint8_t* const sbp = smem_raw + (sb - smem_u32(smem_raw));
    float* small = reinterpret_cast<float*>(sbp + OFF_SMALL);
    const uint32_t bar0 = smem_u32(&mbar[0]);
    auto bar = [&](int k) { return bar0 + 8u * (uint32_t) k; };
    volatile int* abort = &abort_sh;
    const int T = p.S / LT;
    const int nsamp = (p.batch - (int) blockIdx.x + (int) gridDim.x - 1) / (int) gridDim.x;
    const int n = nsamp * T;
    auto sample = [&](int s) { return (int64_t) blockIdx.x + (int64_t) s * gridDim.x; };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(LAYER_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < NBAR; k++) {
            uint32_t cnt = 1;
            if (k == B_EACC || k == B_EACC + 1 || k == B_FOP || k == B_FOP + 1 || k == B_ED || k == B_ED + 1 ||
                k == B_EH || k == B_EH + 1 || (k >= B_FXI && k < B_FXI + NXI) ||
                (lift && k >= B_EGV && k < B_EGV + NX))
                cnt = NEPI / 32;  // one arrival per epilogue warp
            mbar_init(bar(k), cnt);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        abort_sh = 0;
    }
    // per-CTA constants: bias, projection vectors (q2 in BF16, as a product
    // operand); the dense weights' images
    for (int c = tid; c < 64; c += LNTH) small[SM_BIAS + c] = (p.bias && c < p.W) ? p.bias[c] : 0.0f;
    if (last) {
        for (int j = tid; j < 128; j += LNTH) {
            small[SM_BQ1 + j] = j < p.Hq ? p.bq1[j] : 0.0f;
            small[SM_Q2 + j] = j < p.Hq ? bf16r(p.q2[j]) : 0.0f;
        }
    }
    if (lift) {
        for (int e = tid; e < 64 * 16 * 2 / 16; e += LNTH) cp_async16(sb + OFF_W + e * 16, p.P + e * 8, 16u);
    } else {
        for (int e = tid; e < B_IMG / 16; e += LNTH) cp_async16(sb + OFF_W + e * 16, p.Wl + e * 8, 16u);
    }
    if (last)
        for (int e = tid; e < IMG / 16; e += LNTH) cp_async16(sb + OFF_Q + e * 16, p.Q1 + e * 8, 16u);
    if (!lift)  // the Y images' padding (rows o >= W, K >= 2 Mo) is never written again
        for (int e = tid; e < NYR * B_IMG / 16; e += LNTH)
            st_shared_v4(sb + OFF_Y + (uint32_t) (e * 16), 0u, 0u, 0u, 0u);
    cp_async_wait_all();
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_sh;

    if (warp == PROD_WARP) {
        // ---------------------------------------------------------- copies
        // Two queues, each served as soon as its next slot is free: tile
        // ug's (G, v) pair (LIFT: its X tile), with the sample's mixed
        // spectrum Y at a sample's first tile; tile uf's DFT-basis tile
        // (after tile uf's pair). Lane 0 polls; the warp follows.
        int ug = 0, uf = last ? n : 0;
        uint32_t idle = 0;
        while (ug < n || uf < n) {
            int did = 0;
            if (ug < n) {
                const int s = ug / T, i = ug % T, g = ug % NG;
                const bool needy = !lift && i == 0;
                int ok = 0;
                if (lane == 0)
                    ok = mbar_peek(bar(B_EGV + g), ((ug / NG) & 1) ^ 1) &&
                        (!needy || mbar_peek(bar(B_EY + s % NYR), ((s / NYR) & 1) ^ 1));
                if (__shfl_sync(0xFFFFFFFFu, ok, 0)) {
                    const int64_t b = sample(s);
                    if (lane == 0) {
                        if (lift) {
                            const uint32_t bytes = (uint32_t) (LT * p.Fi * 4);
                            mbar_arrive_tx(bar(B_FGV + g), bytes);
                            bulk_g2s(sb + OFF_GV + (uint32_t) (g * X_SLOT), p.X + (b * p.S + (int64_t) i * LT) * p.Fi,
                                     bytes, bar(B_FGV + g));
                        } else {
                            const uint32_t dst = sb + OFF_GV + (uint32_t) (g * GV_SLOT);
                            mbar_arrive_tx(bar(B_FGV + g), 2 * IMG);
                            bulk_g2s(dst, p.G + (int64_t) i * IMG_ELEMS, IMG, bar(B_FGV + g));
                            bulk_g2s(dst + IMG, p.v + (b * T + i) * IMG_ELEMS, IMG, bar(B_FGV + g));
                        }
                    }
                    if (needy) {
                        // the sample's mixed spectrum [2 Mo][W] transposed into the B
                        // image (rows o, K = [Re | Im] modes); entries beyond W, 2 Mo
                        // stay zero
                        const int ys = s % NYR;
                        const uint32_t dy = sb + OFF_Y + (uint32_t) (ys * B_IMG);
                        const int wc = p.W / 8, nch = 2 * p.Mo * wc;  // <= 512 chunks of 8 channels
#pragma unroll 1
                        for (int t0 = 0; t0 < 16; t0 += 8) {  // 8 loads in flight per lane
                            uint4 q[8];
#pragma unroll
                            for (int t = 0; t < 8; t++) {
                                const int e = lane + 32 * (t0 + t), m = e / wc, o0 = (e % wc) * 8;
                                if (e < nch)
                                    q[t] = *reinterpret_cast<const uint4*>(p.Y + (b * 2 * p.Mo + m) * p.W + o0);
                            }
#pragma unroll
                            for (int t = 0; t < 8; t++) {
                                const int e = lane + 32 * (t0 + t), m = e / wc, o0 = (e % wc) * 8;
                                if (e >= nch) break;
                                const uint32_t w[4] = {q[t].x, q[t].y, q[t].z, q[t].w};
                                const uint32_t base = dy + (uint32_t) ((m >> 3) * 128 + (m & 7) * 2);
#pragma unroll
                                for (int k = 0; k < 8; k++) {
                                    const int o = o0 + k;
                                    st_shared_u16(base + (uint32_t) ((o >> 3) * 1024 + (o & 7) * 16),
                                                  (k & 1) ? (w[k >> 1] >> 16) : (w[k >> 1] & 0xFFFFu));
                                }
                            }
                        }
                        fence_async_smem();
                        __syncwarp();
                        if (lane == 0) mbar_arrive(bar(B_FY + ys));
                    }
                    ug++;
                    did = 1;
                }
            }
            if (uf < ug) {
                const int f = uf % NFR;
                int ok = 0;
                if (lane == 0) ok = mbar_peek(bar(B_EF + f), ((uf / NFR) & 1) ^ 1);
                if (__shfl_sync(0xFFFFFFFFu, ok, 0)) {
                    if (lane == 0) {
                        mbar_arrive_tx(bar(B_FF + f), F_IMG);
                        bulk_g2s(sb + OFF_F + (uint32_t) (f * F_IMG), p.F + (int64_t) (uf % T) * IMG_ELEMS, F_IMG,
                                 bar(B_FF + f));
                    }
                    uf++;
                    did = 1;
                }
            }
            int stop = 0;
            if (lane == 0) {
                idle = did ? 0 : idle + 1;
                if (idle >= WAIT_LIMIT) *abort = 1;
                stop = *abort;
            }
            if (__shfl_sync(0xFFFFFFFFu, stop, 0)) break;
        }
    } else if (warp == MMA_WARP) {
        // ---------------------------------------------------------- MMAs
        // Two queues, each issued as soon as its operands and accumulator are
        // ready: tile ui's first product, tile ud's second product (after
        // tile ud's first).
        if (lane == 0) {
            const int nk1 = (2 * p.Mo + 15) / 16, nk2 = (p.W + 15) / 16;
            int ui = 0, ud = 0;
            uint32_t idle = 0;
            while (ud < n) {
                bool did = false;
                if (lift && ui < n) {
                    // lifting: acc = X_image P_image^T (K = 16)
                    const int xi = ui % NXI;
                    if (mbar_peek(bar(B_FXI + xi), (ui / NXI) & 1) &&
                        mbar_peek(bar(B_EACC + (ui & 1)), ((ui >> 1) & 1) ^ 1)) {
                        fence_after();
                        mma_bf16(tmem + (uint32_t) ((ui & 1) * 64),
                                 smem_desc_nsw(sb + OFF_GV + OFF_XI + (uint32_t) (xi * XI_IMG), 128, 256),
                                 smem_desc_nsw(sb + OFF_W, 128, 256), ID64, 0u);
                        mma_commit(bar(B_FACC + (ui & 1)));
                        mma_commit(bar(B_EXI + xi));
                        ui++;
                        did = true;
                    }
                } else if (ui < n) {
                    const int s = ui / T, i = ui % T, g = ui % NG;
                    if (mbar_peek(bar(B_FGV + g), (ui / NG) & 1) &&
                        (i != 0 || mbar_peek(bar(B_FY + s % NYR), (s / NYR) & 1)) &&
                        mbar_peek(bar(B_EACC + (ui & 1)), ((ui >> 1) & 1) ^ 1)) {
                        fence_after();
                        const uint32_t sg = sb + OFF_GV + (uint32_t) (g * GV_SLOT), sv = sg + IMG;
                        const uint32_t sy = sb + OFF_Y + (uint32_t) ((s % NYR) * B_IMG), sw = sb + OFF_W;
                        const uint32_t d = tmem + (uint32_t) ((ui & 1) * 64);
                        for (int kk = 0; kk < nk1; kk++)
                            mma_bf16(d, smem_desc_nsw(sg + kk * 256, 128, 1024),
                                     smem_desc_nsw(sy + kk * 256, 128, 1024), ID64, kk > 0 ? 1u : 0u);
                        for (int kk = 0; kk < nk2; kk++)
                            mma_bf16(d, smem_desc_nsw(sv + kk * 256, 128, 1024),
                                     smem_desc_nsw(sw + kk * 256, 128, 1024), ID64, 1u);
                        mma_commit(bar(B_FACC + (ui & 1)));
                        mma_commit(bar(B_EGV + g));
                        if (i == T - 1) mma_commit(bar(B_EY + s % NYR));
                        ui++;
                        did = true;
                    }
                }
                if (ud < ui) {
                    const int w = ud, sw = w / T, iw = w % T;
                    if (last) {
                        if (mbar_peek(bar(B_FOP + (w & 1)), (w >> 1) & 1) &&
                            mbar_peek(bar(B_EH + (w & 1)), ((w >> 1) & 1) ^ 1)) {
                            fence_after();
                            const uint32_t so = sb + OFF_VT + (uint32_t) ((w & 1) * VT_IMG);
                            for (int kk = 0; kk < nk2; kk++)
                                mma_bf16(tmem + 256u + (uint32_t) ((w & 1) * 128),
                                         smem_desc_nsw(so + kk * 256, 128, 1024),
                                         smem_desc_nsw(sb + OFF_Q + kk * 256, 128, 1024), ID128, kk > 0 ? 1u : 0u);
                            mma_commit(bar(B_EOP + (w & 1)));
                            mma_commit(bar(B_FH + (w & 1)));
                            ud++;
                            did = true;
                        }
                    } else {
                        const int f = w % NFR;
                        if (mbar_peek(bar(B_FOP + (w & 1)), (w >> 1) & 1) && mbar_peek(bar(B_FF + f), (w / NFR) & 1) &&
                            (iw != 0 || mbar_peek(bar(B_ED + (sw & 1)), ((sw >> 1) & 1) ^ 1))) {
                            fence_after();
                            const uint32_t sf = sb + OFF_F + (uint32_t) (f * F_IMG);
                            const uint32_t d = tmem + 128u + (uint32_t) ((sw & 1) * 64);
#pragma unroll
                            for (int kk = 0; kk < LT / 16; kk++)
                                mma_bf16(d, smem_desc_nsw(sf + kk * 256, 128, 2048),
                                         smem_desc_nsw(sb + OFF_VT + (uint32_t) ((w & 1) * VT_IMG) + kk * 2 * VT_LBO,
                                                       VT_LBO, VT_SBO),
                                         ID64, (iw != 0 || kk > 0) ? 1u : 0u);
                            mma_commit(bar(B_EOP + (w & 1)));
                            mma_commit(bar(B_EF + f));
                            if (iw == T - 1) mma_commit(bar(B_FD + (sw & 1)));
                            ud++;
                            did = true;
                        }
                    }
                }
                idle = did ? 0 : idle + 1;
                if (idle >= WAIT_LIMIT) *abort = 1;
                if (*abort) break;
            }
        }
    } else {
        // ---------------------------------------------------------- epilogues
        const int lrow = (warp & 3) * 32 + lane;  // tile row = TMEM lane
        const int qt = warp >> 2;                 // columns 16 qt .. +15 (32 qt .. +31 of H)
        const uint32_t tlane = (uint32_t) ((warp & 3) * 32) << 16;

        // a finished sample's spectrum: D rows = modes (lanes 0..63)
        auto readout = [&](int sr) {
            wait_bar_warp(bar(B_FD + (sr & 1)), (sr >> 1) & 1, abort, lane);
            fence_after();
            if ((warp & 3) < 2) {
                float d[16];
                tmem_ld16(tmem + tlane + 128u + (uint32_t) ((sr & 1) * 64 + qt * 16), d);
                if (lrow < 2 * p.Mo) {
                    __nv_bfloat16* dst = p.vhT + (sample(sr) * 2 * p.Mo + lrow) * p.W + qt * 16;
#pragma unroll
                    for (int c8 = 0; c8 < 2; c8++)
                        if (qt * 16 + c8 * 8 < p.W)
                            *reinterpret_cast<uint4*>(dst + c8 * 8) =
                                make_uint4(pack_bf16(d[8 * c8], d[8 * c8 + 1]), pack_bf16(d[8 * c8 + 2], d[8 * c8 + 3]),
                                           pack_bf16(d[8 * c8 + 4], d[8 * c8 + 5]),
                                           pack_bf16(d[8 * c8 + 6], d[8 * c8 + 7]));
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(B_ED + (sr & 1)));
        };
        // a tile's output: the column quarters' GELU(H + bq1) . q2 sums
        auto project = [&](int w) {
            wait_bar_warp(bar(B_FH + (w & 1)), (w >> 1) & 1, abort, lane);
            fence_after();
            // two partial sums (even and odd columns), packed FP32 pairs
            float2 ys = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int q = 0; q < 2; q++) {
                float h[16];
                tmem_ld16(tmem + tlane + 256u + (uint32_t) ((w & 1) * 128 + qt * 32 + q * 16), h);
#pragma unroll
                for (int k = 0; k < 16; k += 2) {
                    const int j = qt * 32 + q * 16 + k;
                    const float2 v = __fadd2_rn(make_float2(h[k], h[k + 1]),
                                                *reinterpret_cast<const float2*>(small + SM_BQ1 + j));
                    const float2 z = __bfloat1622float2(__float22bfloat162_rn(gelu2(v)));
                    ys = __ffma2_rn(z, *reinterpret_cast<const float2*>(small + SM_Q2 + j), ys);
                }
            }
            const float ysum = ys.x + ys.y;
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(bar(B_EH + (w & 1)));
            float* red = small + SM_RED + (w & 1) * 512;
            red[qt * 128 + lrow] = ysum;
            named_sync(3, NEPI);
            if (qt == 0)
                p.y[sample(w / T) * p.S + (int64_t) (w % T) * LT + lrow] =
                    ((red[lrow] + red[128 + lrow]) + (red[256 + lrow] + red[384 + lrow])) + p.bq2[0];
        };

        // (LIFT) X tile uc (FP32 [128][Fi]) -> its BF16 input image 128 x 16
        // (features >= Fi zero); each thread four features of one row
        auto convert = [&](int uc) {
            const int x = uc % NX, xi = uc % NXI;
            wait_bar_warp(bar(B_FGV + x), (uc / NX) & 1, abort, lane);
            wait_bar_warp(bar(B_EXI + xi), ((uc / NXI) & 1) ^ 1, abort, lane);
            const int r = tid >> 2, k0 = (tid & 3) * 4;
            const float* xs = reinterpret_cast<const float*>(sbp + OFF_GV + x * X_SLOT) + r * p.Fi;
            float f4[4];
#pragma unroll
            for (int k = 0; k < 4; k++) f4[k] = (k0 + k < p.Fi) ? xs[k0 + k] : 0.0f;
            const uint32_t a = sb + OFF_GV + OFF_XI + (uint32_t) (xi * XI_IMG) + koff(r, k0 >> 3, 2) +
                (uint32_t) ((k0 & 7) * 2);
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(a), "r"(pack_bf16(f4[0], f4[1])),
                         "r"(pack_bf16(f4[2], f4[3]))
                         : "memory");
            fence_async_smem();
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(bar(B_FXI + xi));
                mbar_arrive(bar(B_EGV + x));
            }
        };
        if (lift) {
            if (n > 0) convert(0);
            if (n > 1) convert(1);
        }

        int s = 0, i = 0;  // sample and tile of tile u
        for (int u = 0; u < n; u++) {
            float x[16];
            {
                wait_bar_warp(bar(B_FACC + (u & 1)), (u >> 1) & 1, abort, lane);
                fence_after();
                tmem_ld16(tmem + tlane + (uint32_t) ((u & 1) * 64 + qt * 16), x);
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(B_EACC + (u & 1)));
            }
            uint32_t pk[8];
#pragma unroll
            for (int j = 0; j < 16; j += 2) {
                float2 v = __fadd2_rn(make_float2(x[j], x[j + 1]),
                                      *reinterpret_cast<const float2*>(small + SM_BIAS + qt * 16 + j));
                if (GELU) v = gelu2(v);
                pk[j >> 1] = pack_bf16(v.x, v.y);
            }
            if (!last) {
                // the output image (free once the bulk store of tile u-1 has read it)
                const uint32_t so = sb + OFF_OUT;
                if (tid == 0) bulk_wait_read<0>();
                named_sync(1, NEPI);
#pragma unroll
                for (int c8 = 0; c8 < 2; c8++)
                    st_shared_v4(so + koff(lrow, qt * 2 + c8, 8), pk[4 * c8], pk[4 * c8 + 1], pk[4 * c8 + 2],
                                 pk[4 * c8 + 3]);
                // transposed tile u % 2 (free once the DFT of tile u-2 is done)
                wait_bar_warp(bar(B_EOP + (u & 1)), ((u >> 1) & 1) ^ 1, abort, lane);
                const uint32_t tb = sb + OFF_VT + (uint32_t) ((u & 1) * VT_IMG) + (uint32_t) (lrow >> 3) * VT_LBO +
                    (uint32_t) (lrow & 7) * 2;
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int c = qt * 16 + j;
                    st_shared_u16(tb + (uint32_t) (c >> 3) * VT_SBO + (uint32_t) (c & 7) * 16,
                                  (j & 1) ? (pk[j >> 1] >> 16) : (pk[j >> 1] & 0xFFFFu));
                }
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(B_FOP + (u & 1)));
                named_sync(2, NEPI);
                if (tid == 0) {
                    bulk_s2g(p.v_out + (sample(s) * T + i) * IMG_ELEMS, so, IMG);
                    bulk_commit();
                }
                if (i == 0 && s >= 1) readout(s - 1);
            } else {
                // the projection's input image (free once the projection of tile u-2 is done)
                wait_bar_warp(bar(B_EOP + (u & 1)), ((u >> 1) & 1) ^ 1, abort, lane);
                const uint32_t so = sb + OFF_VT + (uint32_t) ((u & 1) * VT_IMG);
#pragma unroll
                for (int c8 = 0; c8 < 2; c8++)
                    st_shared_v4(so + koff(lrow, qt * 2 + c8, 8), pk[4 * c8], pk[4 * c8 + 1], pk[4 * c8 + 2],
                                 pk[4 * c8 + 3]);
                fence_async_smem();
                __syncwarp();
                if (lane == 0) mbar_arrive(bar(B_FOP + (u & 1)));
                if (u >= 1) project(u - 1);
            }
            if (lift && u + 2 < n) convert(u + 2);
            if (++i == T) {
                i = 0;
                s++;
            }
        }
        if (n > 0) {
            if (!last) readout(nsamp - 1);
            else project(n - 1);
        }
        if (tid == 0) bulk_wait<0>();
    }
    if (tid == 0 && abort_sh) atomicOr(p.status, ST_WAIT);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(LAYER_TMEM_COLS)
                     : "memory");
    }
}

bool aligned16(const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15) == 0; }

void spectral_layer(const mbg_fno_layer_desc* d, cudaStream_t s)
{
    require(d != nullptr, "spectral_layer: null descriptor");
    require(d->mode >= MBG_LAYER_LIFT && d->mode <= MBG_LAYER_LAST, "spectral_layer: bad mode");
    require(d->act == MBG_ACT_NONE || d->act == MBG_ACT_GELU, "spectral_layer: act must be NONE or GELU");
    require(d->batch >= 1 && d->S >= LT && d->S % LT == 0, "spectral_layer: S must be a positive multiple of 128");
    require(d->W >= 8 && d->W <= 64 && d->W % 8 == 0, "spectral_layer: W must be 8..64, a multiple of 8");
    require(d->Mo >= 8 && 2 * d->Mo <= 64 && d->Mo % 8 == 0, "spectral_layer: Mo must be 8..32, a multiple of 8");
    require((int64_t) d->batch * d->S * 64 < ((int64_t) 1 << 62), "spectral_layer: too large");
    if (d->mode == MBG_LAYER_LIFT) {
        require(d->X && d->P && d->Fi >= 1 && d->Fi <= 16, "spectral_layer: LIFT needs X, P and 1 <= Fi <= 16");
        require(aligned16(d->X), "spectral_layer: X must be 16-byte aligned");
    } else {
        require(d->v && d->Y && d->G && d->Wl, "spectral_layer: MID/LAST need v, Y, G and Wl");
        require(aligned16(d->v) && aligned16(d->Y) && aligned16(d->G) && aligned16(d->Wl),
                "spectral_layer: v, Y, G and Wl must be 16-byte aligned");
    }
    if (d->mode == MBG_LAYER_LAST) {
        require(d->Q1 && d->bq1 && d->q2 && d->bq2 && d->y, "spectral_layer: LAST needs Q1, bq1, q2, bq2 and y");
        require(d->Hq >= 1 && d->Hq <= 128, "spectral_layer: Hq must be 1..128");
        require(aligned16(d->Q1), "spectral_layer: Q1 must be 16-byte aligned");
    } else {
        require(d->v_out && d->F && d->vhT, "spectral_layer: LIFT/MID need v_out, F and vhT");
        require(aligned16(d->v_out) && aligned16(d->F) && aligned16(d->vhT),
                "spectral_layer: v_out, F and vhT must be 16-byte aligned");
    }
    layer_params p{};
    p.mode = d->mode;
    p.act = d->act;
    p.batch = d->batch;
    p.S = d->S;
    p.W = d->W;
    p.Mo = d->Mo;
    p.Fi = d->Fi;
    p.Hq = d->Hq;
    p.X = d->X;
    p.P = static_cast<const __nv_bfloat16*>(d->P);
    p.v = static_cast<const __nv_bfloat16*>(d->v);
    p.Y = static_cast<const __nv_bfloat16*>(d->Y);
    p.G = static_cast<const __nv_bfloat16*>(d->G);
    p.Wl = static_cast<const __nv_bfloat16*>(d->Wl);
    p.bias = d->bias;
    p.v_out = static_cast<__nv_bfloat16*>(d->v_out);
    p.F = static_cast<const __nv_bfloat16*>(d->F);
    p.vhT = static_cast<__nv_bfloat16*>(d->vhT);
    p.Q1 = static_cast<const __nv_bfloat16*>(d->Q1);
    p.bq1 = d->bq1;
    p.q2 = d->q2;
    p.bq2 = d->bq2;
    p.y = d->y;
    p.status = status_ptr();
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        throw std::runtime_error("CUDA: device query failed");
    static std::once_flag attr;
    std::call_once(attr, [] {
        const void* ks[] = {(const void*) spectral_layer_kernel<MBG_LAYER_LIFT, false>,
                            (const void*) spectral_layer_kernel<MBG_LAYER_LIFT, true>,
                            (const void*) spectral_layer_kernel<MBG_LAYER_MID, false>,
                            (const void*) spectral_layer_kernel<MBG_LAYER_MID, true>,
                            (const void*) spectral_layer_kernel<MBG_LAYER_LAST, false>,
                            (const void*) spectral_layer_kernel<MBG_LAYER_LAST, true>};
        for (const void* k : ks) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, LAYER_SMEM);
    });
    const int grid = d->batch < sms ? d->batch : sms;
    const bool g = d->act == MBG_ACT_GELU;
    if (d->mode == MBG_LAYER_LIFT) {
        if (g)
            spectral_layer_kernel<MBG_LAYER_LIFT, true><<<grid, LNTH, LAYER_SMEM, s>>>(p);
        else
            spectral_layer_kernel<MBG_LAYER_LIFT, false><<<grid, LNTH, LAYER_SMEM, s>>>(p);
    } else if (d->mode == MBG_LAYER_MID) {
        if (g)
            spectral_layer_kernel<MBG_LAYER_MID, true><<<grid, LNTH, LAYER_SMEM, s>>>(p);
        else
            spectral_layer_kernel<MBG_LAYER_MID, false><<<grid, LNTH, LAYER_SMEM, s>>>(p);
    } else {
        if (g)
            spectral_layer_kernel<MBG_LAYER_LAST, true><<<grid, LNTH, LAYER_SMEM, s>>>(p);
        else
            spectral_layer_kernel<MBG_LAYER_LAST, false><<<grid, LNTH, LAYER_SMEM, s>>>(p);
    }
    check_launch("spectral_layer_kernel");
}

}  // namespace
}  // namespace fno
}  // namespace mbg

extern "C" int mbg_fno_spectral_layer(const mbg_fno_layer_desc* d, void* stream)
{
    return mbg::fno::guard([&] { mbg::fno::spectral_layer(d, (cudaStream_t) stream); });
}
