// One Fourier layer of surrogate inference per launch
// (include/mbsolve_fno.h, mbg_fno_spectral_layer).
//
// The layer's products never leave the SM between them. A CTA owns whole
// samples (one CTA per SM, the samples strided over the CTAs) and walks
// each sample's S rows in tiles of 128:
//
//   first product   MID/LAST: acc = G Y^T + v Wl^T on the tensor cores
//                   (two K = 64 operand pairs, tcgen05.mma, FP32 in TMEM);
//                   LIFT: acc = X P^T on the CUDA cores (K = Fi <= 16)
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
// Pipeline: one iteration per tile t, 8 warps in lock step, one thread
// issuing the MMAs. In iteration t the first product of tile t is issued,
// the epilogue of tile t-1 runs, the second product of tile t-1 is issued
// and the second product of tile t-3 is read out; the per-sample
// activations of tile t+2 (v, or X) and the shared operands of tile t+1
// (the G and DFT-basis tiles, L2-resident) are copied (cp.async) meanwhile.
// So no step waits for work issued less than an iteration before it: the
// rings hold three v (four X) tiles, two G tiles, four basis tiles and
// three Y tiles; TMEM holds two first-product accumulators and two
// second-product ones; the MMA operands written by the epilogue are
// double-buffered. Operand tiles use the no-swizzle K-major core-matrix
// layout. The transposed activation tile (K = samples) has its K-direction
// core matrices 144 bytes apart instead of 128, so that a warp's 2-byte
// stores of one channel for 32 consecutive samples land in four distinct
// bank groups. The DFT product has M = 64 mode rows; it is issued as
// M = 128, and the 64 rows above the basis tile read whatever lies behind
// it in shared memory: they only feed TMEM lanes 64-127, which nothing
// reads. Every wait is bounded; on time-out the kernel records it in the
// status word and returns after freeing its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "fno_common.cuh"

namespace mbg {
namespace fno {
namespace {

constexpr int LT = 128;    // rows (samples s) per tile
constexpr int LNTH = 256;  // warp w: TMEM lanes 32 (w % 4) .. +31, columns 32 (w / 4) .. +31

constexpr int F_TILE = 64 * LT * 2;             // DFT basis tile: 64 mode rows x 128 samples
constexpr int X_TILE = LT * 16 * 4;             // lifting input tile: 128 rows x <= 16 FP32 features
constexpr int NF = 4, NG = 2, NV = 3, NX = 4, NY = 3;  // ring depths
constexpr uint32_t VT_LBO = 144;                // transposed tile: K-direction core-matrix stride
constexpr uint32_t VT_SBO = 16 * VT_LBO;        // 8-channel group stride
constexpr int VT_TILE = 8 * VT_SBO;             // 64 channel rows x 128 samples
constexpr int A_TILE = LT * 64 * 2;             // G, v or projection-input tile: 128 rows x K 64
constexpr int B_TILE = 64 * 64 * 2;             // Y or Wl tile: 64 rows x K 64
constexpr int Q_TILE = 128 * 64 * 2;            // Q1 tile: 128 rows x K 64

// shared memory map (bytes from a 128-aligned base); LAST keeps Q1 where
// the basis ring is, its projection inputs where the transposed tiles
// are; LIFT keeps its X ring where the v ring is
constexpr int OFF_F = 0;
constexpr int OFF_Q = 0;
constexpr int OFF_VT = OFF_F + NF * F_TILE;
constexpr int OFF_G = OFF_VT + 2 * VT_TILE;
constexpr int OFF_V = OFF_G + NG * A_TILE;
constexpr int OFF_X = OFF_V;
constexpr int OFF_Y = OFF_V + NV * A_TILE;
constexpr int OFF_W = OFF_Y + NY * B_TILE;
constexpr int OFF_SMALL = OFF_W + B_TILE;
constexpr int SM_BIAS = 0, SM_BQ1 = 64, SM_Q2 = 192, SM_RED = 320, SM_P = 448;  // floats
constexpr int SMALL_FLOATS = SM_P + 16 * 64;
constexpr int LAYER_SMEM = OFF_SMALL + SMALL_FLOATS * 4 + 128;  // + alignment slack
// the last basis slot's unread M rows (32 KB from its start) stay inside the map
static_assert(OFF_F + (NF - 1) * F_TILE + 2 * F_TILE <= OFF_G, "basis slot overrun");
static_assert(Q_TILE <= NF * F_TILE && 2 * A_TILE <= 2 * VT_TILE && NX * X_TILE <= NV * A_TILE, "aliases");
static_assert(LAYER_SMEM + 128 <= 227 * 1024, "shared memory");

constexpr uint32_t ID64 = idesc_bf16(128, 64);
constexpr uint32_t ID128 = idesc_bf16(128, 128);
// columns: first-product accumulators at 0 and 64; DFT accumulators at 128
// and 192 (by sample parity); projection accumulators at 256 and 384
constexpr uint32_t LAYER_TMEM_COLS = 512;

struct layer_params {
    int32_t mode, act, batch, S, W, Mo, Fi, Hq;
    const float* X;
    const float* P;
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

// byte offset of 16-byte chunk (row, kc) in a K-major tile with `kch`
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

// the sample (global index) of this CTA's tile u
__device__ __forceinline__ int64_t tile_sample(int u, int T)
{
    return blockIdx.x + (int64_t) (u / T) * gridDim.x;
}

// Shared operands of tile u: its G tile (MID, LAST) and DFT-basis tile
// (LIFT, MID), both the same for every sample; chunks outside the operands
// are zero-filled.
__device__ __forceinline__ void copy_shared_ops(const layer_params& p, int u, int T, uint32_t sb, int tid)
{
    const int s0 = (u % T) * LT, two_mo = 2 * p.Mo;
    if (p.mode != MBG_LAYER_LIFT) {
        const uint32_t sg = sb + OFF_G + (uint32_t) ((u % NG) * A_TILE);
#pragma unroll
        for (int q = 0; q < 1024 / LNTH; q++) {
            const int e = tid + q * LNTH, r = e >> 3, kc = e & 7;
            const bool ok = kc * 8 < two_mo;
            cp_async16(sg + koff(r, kc, 8), ok ? p.G + (int64_t) (s0 + r) * two_mo + kc * 8 : p.G, ok ? 16u : 0u);
        }
    }
    if (p.mode != MBG_LAYER_LAST) {
        const uint32_t sf = sb + OFF_F + (uint32_t) ((u % NF) * F_TILE);
#pragma unroll
        for (int q = 0; q < 1024 / LNTH; q++) {
            const int e = tid + q * LNTH, r = e >> 4, kc = e & 15;
            const bool ok = r < two_mo;
            cp_async16(sf + koff(r, kc, 16), ok ? p.F + (int64_t) r * p.S + s0 + kc * 8 : p.F, ok ? 16u : 0u);
        }
    }
}

// Per-sample operands of tile u: its v tile and, for a sample's first
// tile, the sample's Y (MID, LAST), or its X tile (LIFT).
__device__ __forceinline__ void copy_sample_ops(const layer_params& p, int u, int T, uint32_t sb, int tid)
{
    const int i = u % T, s0 = i * LT, two_mo = 2 * p.Mo;
    const int64_t b = tile_sample(u, T);
    if (p.mode == MBG_LAYER_LIFT) {
        // the tile's X rows are contiguous: 128 Fi floats, 16-byte aligned
        const float* xs = p.X + (b * p.S + s0) * p.Fi;
        const uint32_t sx = sb + OFF_X + (uint32_t) ((u % NX) * X_TILE);
        for (int e = tid; e < LT * p.Fi / 4; e += LNTH) cp_async16(sx + e * 16, xs + e * 4, 16u);
        return;
    }
    const uint32_t sv = sb + OFF_V + (uint32_t) ((u % NV) * A_TILE);
#pragma unroll
    for (int q = 0; q < 1024 / LNTH; q++) {
        const int e = tid + q * LNTH, r = e >> 3, kc = e & 7;
        const bool ok = kc * 8 < p.W;
        cp_async16(sv + koff(r, kc, 8), ok ? p.v + (b * p.S + s0 + r) * p.W + kc * 8 : p.v, ok ? 16u : 0u);
    }
    if (i == 0) {
        const uint32_t sy = sb + OFF_Y + (uint32_t) (((u / T) % NY) * B_TILE);
#pragma unroll
        for (int q = 0; q < 512 / LNTH; q++) {
            const int e = tid + q * LNTH, o = e >> 3, kc = e & 7, k = kc * 8;
            const bool ok = o < p.W && k < two_mo;
            const int part = ok ? k / p.Mo : 0, m = ok ? k % p.Mo : 0;
            cp_async16(sy + koff(o, kc, 8), ok ? p.Y + ((b * 2 + part) * p.W + o) * p.Mo + m : p.Y, ok ? 16u : 0u);
        }
    }
}

__global__ void __launch_bounds__(LNTH, 1) spectral_layer_kernel(const layer_params p)
{
    extern __shared__ __align__(128) uint8_t smem_raw[];
    // first product of an even / odd tile, second product of an even / odd tile
    __shared__ __align__(8) uint64_t mbar[4];
    __shared__ uint32_t tmem_sh;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int lrow = (warp & 3) * 32 + lane;  // tile row = TMEM lane
    const int half = warp >> 2;               // columns 32 half .. +31 (64 half .. +63 of H)
    const uint32_t sb = (smem_u32(smem_raw) + 127u) & ~127u;
    uint8_t* const sbp = smem_raw + (sb - smem_u32(smem_raw));
    float* small = reinterpret_cast<float*>(sbp + OFF_SMALL);
    const uint32_t mb_inv0 = smem_u32(&mbar[0]), mb_aux0 = smem_u32(&mbar[2]);
    const int T = p.S / LT;
    const int nsamp = (p.batch - (int) blockIdx.x + (int) gridDim.x - 1) / (int) gridDim.x;
    const int n = nsamp * T;
    const bool lift = p.mode == MBG_LAYER_LIFT, last = p.mode == MBG_LAYER_LAST;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(LAYER_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int k = 0; k < 4; k++) mbar_init(smem_u32(&mbar[k]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // per-CTA constants: bias, projection vectors (q2 in BF16, as a product
    // operand), lifting weights (BF16-rounded, [feature][channel])
    for (int c = tid; c < 64; c += LNTH) small[SM_BIAS + c] = (p.bias && c < p.W) ? p.bias[c] : 0.0f;
    if (last) {
        for (int j = tid; j < 128; j += LNTH) {
            small[SM_BQ1 + j] = j < p.Hq ? p.bq1[j] : 0.0f;
            small[SM_Q2 + j] = j < p.Hq ? bf16r(p.q2[j]) : 0.0f;
        }
    }
    if (lift) {
        for (int e = tid; e < 16 * 64; e += LNTH) {
            const int f = e >> 6, c = e & 63;
            small[SM_P + e] = (f < p.Fi && c < p.W) ? bf16r(p.P[c * p.Fi + f]) : 0.0f;
        }
    }
    // copy groups: the once-per-CTA tiles with tile 0, then tile 1's
    // per-sample operands; iteration t commits tile t+1's shared operands,
    // then tile t+2's per-sample ones
    if (!lift) {
        for (int e = tid; e < 512; e += LNTH) {
            const int o = e >> 3, kc = e & 7;
            const bool ok = o < p.W && kc * 8 < p.W;
            cp_async16(sb + OFF_W + koff(o, kc, 8), ok ? p.Wl + (int64_t) o * p.W + kc * 8 : p.Wl, ok ? 16u : 0u);
        }
    }
    if (last) {
        for (int e = tid; e < 1024; e += LNTH) {
            const int j = e >> 3, kc = e & 7;
            const bool ok = j < p.Hq && kc * 8 < p.W;
            cp_async16(sb + OFF_Q + koff(j, kc, 8), ok ? p.Q1 + (int64_t) j * p.W + kc * 8 : p.Q1, ok ? 16u : 0u);
        }
    }
    if (n > 0) {
        copy_shared_ops(p, 0, T, sb, tid);
        copy_sample_ops(p, 0, T, sb, tid);
    }
    cp_async_commit();
    if (n > 1) copy_sample_ops(p, 1, T, sb, tid);
    cp_async_commit();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_sh;
    const uint32_t tlane = (uint32_t) ((warp & 3) * 32) << 16;
    const int nk1 = (2 * p.Mo + 15) / 16, nk2 = (p.W + 15) / 16;

    bool fail = false;
    for (int t = 0; t <= n + 2; t++) {
        // tile t's operands have landed (only tile t+1's per-sample copies may be in flight)
        if (t < n) {
            cp_async_wait<1>();
            fence_async_smem();
        }
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        // first product of tile t into accumulator t % 2
        if (t < n && !lift && tid == 0) {
            fence_after();
            const uint32_t sg = sb + OFF_G + (uint32_t) ((t % NG) * A_TILE);
            const uint32_t sv = sb + OFF_V + (uint32_t) ((t % NV) * A_TILE);
            const uint32_t sy = sb + OFF_Y + (uint32_t) (((t / T) % NY) * B_TILE), sw = sb + OFF_W;
            const uint32_t d = tmem + (uint32_t) ((t & 1) * 64);
            for (int kk = 0; kk < nk1; kk++)
                mma_bf16(d, smem_desc_nsw(sg + kk * 256, 128, 1024), smem_desc_nsw(sy + kk * 256, 128, 1024), ID64,
                         kk > 0 ? 1u : 0u);
            for (int kk = 0; kk < nk2; kk++)
                mma_bf16(d, smem_desc_nsw(sv + kk * 256, 128, 1024), smem_desc_nsw(sw + kk * 256, 128, 1024), ID64,
                         1u);
            mma_commit(mb_inv0 + 8u * (uint32_t) (t & 1));
        }
        // first product of tile t-1 and second product of tile t-3 done
        if (t >= 1 && t <= n && !lift && !mbar_wait(mb_inv0 + 8u * (uint32_t) ((t - 1) & 1), ((t - 1) >> 1) & 1))
            fail = true;
        if (t >= 3 && !mbar_wait(mb_aux0 + 8u * (uint32_t) ((t - 3) & 1), ((t - 3) >> 1) & 1)) fail = true;
        fail = __any_sync(0xFFFFFFFFu, fail);  // warp-uniform: the TMEM loads below are warp-wide
        fence_after();
        // copies (their ring slots were last read by the products just waited for)
        if (!fail && t + 1 < n) copy_shared_ops(p, t + 1, T, sb, tid);
        cp_async_commit();
        if (!fail && t + 2 < n) copy_sample_ops(p, t + 2, T, sb, tid);
        cp_async_commit();

        // second product of tile t-3: a finished sample's spectrum, or y
        float ysum = 0.0f;
        if (!fail && t >= 3) {
            const int u = t - 3;
            if (last) {
#pragma unroll 1
                for (int q = 0; q < 4; q++) {
                    float h[16];
                    tmem_ld16(tmem + tlane + 256u + (uint32_t) ((u & 1) * 128 + half * 64 + q * 16), h);
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        const int j = half * 64 + q * 16 + k;
                        const float z = bf16r(gelu(h[k] + small[SM_BQ1 + j]));
                        ysum = fmaf(z, small[SM_Q2 + j], ysum);
                    }
                }
                if (half == 1) small[SM_RED + lrow] = ysum;
            } else if (u % T == T - 1 && (warp & 3) < 2) {
                float d0[16], d1[16];
                const uint32_t ta = tmem + tlane + 128u + (uint32_t) (((u / T) & 1) * 64 + half * 32);
                tmem_ld16(ta, d0);
                tmem_ld16(ta + 16u, d1);
                if (lrow < 2 * p.Mo) {
                    __nv_bfloat16* dst = p.vhT + (tile_sample(u, T) * 2 * p.Mo + lrow) * p.W + half * 32;
#pragma unroll
                    for (int c8 = 0; c8 < 4; c8++) {
                        if (half * 32 + c8 * 8 >= p.W) break;
                        const float* s8 = c8 < 2 ? d0 + c8 * 8 : d1 + (c8 - 2) * 8;
                        *reinterpret_cast<uint4*>(dst + c8 * 8) =
                            make_uint4(pack_bf16(s8[0], s8[1]), pack_bf16(s8[2], s8[3]), pack_bf16(s8[4], s8[5]),
                                       pack_bf16(s8[6], s8[7]));
                    }
                }
            }
        }

        // epilogue of tile t-1
        if (!fail && t >= 1 && t <= n) {
            const int u = t - 1;
            const int64_t grow = tile_sample(u, T) * p.S + (int64_t) (u % T) * LT + lrow;
            float x[32];
            if (lift) {
                const float* xs = reinterpret_cast<const float*>(sbp + OFF_X + (u % NX) * X_TILE) + lrow * p.Fi;
#pragma unroll
                for (int j = 0; j < 32; j++) x[j] = 0.0f;
                for (int f = 0; f < p.Fi; f++) {
                    const float xv = bf16r(xs[f]);
                    const float4* w4 = reinterpret_cast<const float4*>(small + SM_P + f * 64 + half * 32);
#pragma unroll
                    for (int q = 0; q < 8; q++) {
                        const float4 w = w4[q];
                        x[4 * q] = fmaf(xv, w.x, x[4 * q]);
                        x[4 * q + 1] = fmaf(xv, w.y, x[4 * q + 1]);
                        x[4 * q + 2] = fmaf(xv, w.z, x[4 * q + 2]);
                        x[4 * q + 3] = fmaf(xv, w.w, x[4 * q + 3]);
                    }
                }
            } else {
                float a0[16], a1[16];
                const uint32_t ta = tmem + tlane + (uint32_t) ((u & 1) * 64 + half * 32);
                tmem_ld16(ta, a0);
                tmem_ld16(ta + 16u, a1);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    x[j] = a0[j];
                    x[16 + j] = a1[j];
                }
            }
            uint32_t pk[16];
#pragma unroll
            for (int j = 0; j < 32; j += 2) {
                float v0 = x[j] + small[SM_BIAS + half * 32 + j];
                float v1 = x[j + 1] + small[SM_BIAS + half * 32 + j + 1];
                if (p.act == MBG_ACT_GELU) {
                    v0 = gelu(v0);
                    v1 = gelu(v1);
                }
                pk[j >> 1] = pack_bf16(v0, v1);
            }
            const uint32_t so = sb + OFF_VT + (uint32_t) ((u & 1) * VT_TILE);
            if (!last) {
                __nv_bfloat16* dst = p.v_out + grow * p.W + half * 32;
#pragma unroll
                for (int c8 = 0; c8 < 4; c8++)
                    if (half * 32 + c8 * 8 < p.W)
                        *reinterpret_cast<uint4*>(dst + c8 * 8) =
                            make_uint4(pk[4 * c8], pk[4 * c8 + 1], pk[4 * c8 + 2], pk[4 * c8 + 3]);
                // element (channel c, sample lrow) of the transposed tile
                const uint32_t tb = so + (uint32_t) (lrow >> 3) * VT_LBO + (uint32_t) (lrow & 7) * 2;
#pragma unroll
                for (int j = 0; j < 32; j++) {
                    const int c = half * 32 + j;
                    st_shared_u16(tb + (uint32_t) (c >> 3) * VT_SBO + (uint32_t) (c & 7) * 16,
                                  (j & 1) ? (pk[j >> 1] >> 16) : (pk[j >> 1] & 0xFFFFu));
                }
            } else {
#pragma unroll
                for (int c8 = 0; c8 < 4; c8++)
                    st_shared_v4(so + koff(lrow, half * 4 + c8, 8), pk[4 * c8], pk[4 * c8 + 1], pk[4 * c8 + 2],
                                 pk[4 * c8 + 3]);
            }
        }
        fence_async_smem();
        fence_before();
        if (__syncthreads_or(fail)) {
            fail = true;
            break;
        }
        // output of tile t-3 (the two column halves' partial sums)
        if (last && t >= 3 && half == 0) {
            const int u = t - 3;
            p.y[tile_sample(u, T) * p.S + (int64_t) (u % T) * LT + lrow] = (ysum + small[SM_RED + lrow]) + p.bq2[0];
        }
        // second product of tile t-1
        if (t >= 1 && t <= n && tid == 0) {
            fence_after();
            const int u = t - 1;
            const uint32_t so = sb + OFF_VT + (uint32_t) ((u & 1) * VT_TILE);
            if (last) {
                for (int kk = 0; kk < nk2; kk++)
                    mma_bf16(tmem + 256u + (uint32_t) ((u & 1) * 128), smem_desc_nsw(so + kk * 256, 128, 1024),
                             smem_desc_nsw(sb + OFF_Q + kk * 256, 128, 1024), ID128, kk > 0 ? 1u : 0u);
            } else {
                const uint32_t sf = sb + OFF_F + (uint32_t) ((u % NF) * F_TILE);
                const uint32_t d = tmem + 128u + (uint32_t) (((u / T) & 1) * 64);
#pragma unroll
                for (int kk = 0; kk < LT / 16; kk++)
                    mma_bf16(d, smem_desc_nsw(sf + kk * 256, 128, 2048),
                             smem_desc_nsw(so + kk * 2 * VT_LBO, VT_LBO, VT_SBO), ID64,
                             (u % T != 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(mb_aux0 + 8u * (uint32_t) (u & 1));
        }
    }
    cp_async_wait<0>();
    if (fail && tid == 0) atomicOr(p.status, ST_WAIT);
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
    p.P = d->P;
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
        cudaFuncSetAttribute(spectral_layer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, LAYER_SMEM);
    });
    const int grid = d->batch < sms ? d->batch : sms;
    spectral_layer_kernel<<<grid, LNTH, LAYER_SMEM, s>>>(p);
    check_launch("spectral_layer_kernel");
}

}  // namespace
}  // namespace fno
}  // namespace mbg

extern "C" int mbg_fno_spectral_layer(const mbg_fno_layer_desc* d, void* stream)
{
    return mbg::fno::guard([&] { mbg::fno::spectral_layer(d, (cudaStream_t) stream); });
}
