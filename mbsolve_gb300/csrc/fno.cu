// Kernels of the Fourier-neural-operator surrogate (include/mbsolve_fno.h).
//
// The network's products (lifting, truncated DFT and its inverse, spectral
// mode mixing, pointwise channel mixing, projection, and all of their
// gradients) are small strided GEMMs. One tensor-core kernel serves all of
// them: a 128 x 64 output tile per CTA, accumulated in tensor memory (TMEM)
// by tcgen05.mma (kind::f16, BF16 operands, FP32 accumulator), K in blocks
// of 64 staged in shared memory. Operands are written into the no-swizzle K-major
// core-matrix layout the tensor core reads: 8 rows x 16 bytes per core
// matrix, core matrices 128 bytes apart along K (leading byte offset) and
// 1024 bytes apart along M/N (stride byte offset). When every operand of a
// product is BF16 with K contiguous (16-byte aligned rows), each 16-byte
// chunk is copied asynchronously (cp.async, zero-filled outside the
// operand) into a ring of four stages filled two blocks ahead of the MMAs;
// otherwise it is gathered with plain loads (any strides, FP32 or BF16,
// converted to BF16 on the way) into two stages, each loaded while the
// MMAs of the other run (the smaller footprint keeps four CTAs per SM for
// the short-K gathers of training). One elected thread issues the MMAs;
// tcgen05.commit arrives on the stage's mbarrier when they have read the
// stage. Every wait is bounded: on time-out the kernel records it in the
// status word and returns after freeing its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "fno_common.cuh"

namespace mbg {
namespace fno {

constexpr int BM = 128;          // rows of a tile (TMEM lanes)
constexpr int BN = 64;           // columns of a tile (TMEM columns, FP32)
constexpr int BK = 64;           // K per stage (128 bytes of BF16 per row)
constexpr int NTH = 128;         // 4 warps: warp w reads TMEM lanes 32w..32w+31
// stage ring of the asynchronous path (K blocks staged ahead of the MMAs)
// and of the gather path; products of at most two K blocks (per split)
// take an asynchronous two-stage ring (half the shared memory: twice the
// CTAs per SM)
constexpr int STAGES_ASYNC = 4, AHEAD_ASYNC = 2;
constexpr int STAGES_SHORT = 2, AHEAD_SHORT = 2;
constexpr int STAGES_GATHER = 2, AHEAD_GATHER = 0;
constexpr int A_BYTES = BM * BK * 2;
constexpr int B_BYTES = BN * BK * 2;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int smem_bytes(int stages) { return stages * STAGE_BYTES + 128; }  // + alignment slack
static_assert(BM * (BN + 1) * 4 <= STAGES_GATHER * STAGE_BYTES, "epilogue tile must fit the stages");
constexpr int TMEM_COLS = 64;    // power of two >= 32
constexpr uint32_t LBO = 128;    // K-direction core-matrix stride (bytes)
constexpr uint32_t SBO = 1024;   // M/N-direction 8-row-group stride (bytes)
struct seg_t {
    const void* a;
    const void* b;
    int64_t a_sm, a_sk, a_sz;
    int64_t b_sn, b_sk, b_sz;
    int32_t k, a_type, b_type, neg;
};

struct gemm_params {
    int32_t m, n, nseg, ktotal;
    int32_t kstart[4];
    seg_t seg[3];
    int32_t async_ok;  // every operand BF16, K contiguous, 16-byte aligned rows
    int32_t vec_c;     // STORE epilogue as 16-byte stores of 8 outputs along C's rows
    int32_t vec_c2;    // the second output as 16-byte stores of 8 outputs along its columns
    int32_t fin;       // STORE mode without pre or gate: bias and activation applied once, on
                       // the way from TMEM into the shared tile
    void* c;
    int64_t c_sm, c_sn, c_sz;
    void* c2;          // optional second (BF16) copy of C with its own strides
    int64_t c2_sm, c2_sn, c2_sz;
    const float* rowdot;       // optional: C(i) += sum_j rowdot[j] out(i, j) instead of storing out
    const float* rowdot_bias;
    int32_t c_type, mode, act;
    int32_t kblocks_per_split;
    float alpha;
    const float* bias;
    float* pre;
    const float* gate;
    uint32_t* status;
};

// ------------------------------------------------------------ helpers

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) { return smem_desc_nsw(addr, LBO, SBO); }

constexpr uint32_t IDESC = idesc_bf16(BM, BN);

__device__ __forceinline__ float ld_elem(const void* base, int32_t type, int64_t off)
{
    if (type == MBG_BF16) return __bfloat162float(reinterpret_cast<const __nv_bfloat16*>(base)[off]);
    return reinterpret_cast<const float*>(base)[off];
}

// Gather 8 consecutive K elements (k0 .. k0+7, global K index) of row `row`
// of operand A (is_a) or B, negated for a negated segment's A, zero outside
// the operand.
__device__ __forceinline__ void gather_chunk(
    const gemm_params& p, bool is_a, int z, int row, int rows, int k0, float (&v)[8])
{
#pragma unroll
    for (int e = 0; e < 8; e++) v[e] = 0.0f;
    if (row < rows && k0 < p.ktotal) {
        int s = 0;
        if (p.nseg > 1 && k0 >= p.kstart[1]) s = 1;
        if (p.nseg > 2 && k0 >= p.kstart[2]) s = 2;
        const seg_t& g = p.seg[s];
        const int kl = k0 - p.kstart[s];
        const void* base = is_a ? g.a : g.b;
        const int32_t type = is_a ? g.a_type : g.b_type;
        const int64_t sr = is_a ? g.a_sm : g.b_sn;
        const int64_t sk = is_a ? g.a_sk : g.b_sk;
        const int64_t sz = is_a ? g.a_sz : g.b_sz;
        const int64_t off = (int64_t) z * sz + (int64_t) row * sr + (int64_t) kl * sk;
        const int nv = min(8, g.k - kl);
        const size_t esz = type == MBG_BF16 ? 2 : 4;
        const uintptr_t addr = reinterpret_cast<uintptr_t>(base) + (uintptr_t) (off * (int64_t) esz);
        if (sk == 1 && nv == 8 && type == MBG_BF16 && (addr & 15) == 0) {
            const uint4 q = *reinterpret_cast<const uint4*>(addr);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const float2 f = __bfloat1622float2(h[e]);
                v[2 * e] = f.x;
                v[2 * e + 1] = f.y;
            }
        } else if (sk == 1 && nv == 8 && type == MBG_F32 && (addr & 15) == 0) {
            const float4 a = reinterpret_cast<const float4*>(addr)[0];
            const float4 b = reinterpret_cast<const float4*>(addr)[1];
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
            v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        } else {
#pragma unroll
            for (int e = 0; e < 8; e++)
                if (e < nv) v[e] = ld_elem(base, type, off + (int64_t) e * sk);
        }
        if (g.neg && is_a) {  // negate the product: A only
#pragma unroll
            for (int e = 0; e < 8; e++) v[e] = -v[e];
        }
    }
}

// the 16-byte chunk (k0 .. k0+7) of row `row` of operand A (is_a) or B, copied
// asynchronously to dst (zeros outside the operand); async_ok products only
__device__ __forceinline__ void async_chunk(
    const gemm_params& p, bool is_a, int z, int row, int rows, int k0, uint32_t dst)
{
    const void* src = is_a ? p.seg[0].a : p.seg[0].b;  // any valid address for a zero fill
    uint32_t bytes = 0;
    if (row < rows && k0 < p.ktotal) {
        int s = 0;
        if (p.nseg > 1 && k0 >= p.kstart[1]) s = 1;
        if (p.nseg > 2 && k0 >= p.kstart[2]) s = 2;
        const seg_t& g = p.seg[s];
        const int64_t kl = k0 - p.kstart[s];
        const int64_t off = is_a ? (int64_t) z * g.a_sz + (int64_t) row * g.a_sm + kl
                                 : (int64_t) z * g.b_sz + (int64_t) row * g.b_sn + kl;
        src = reinterpret_cast<const __nv_bfloat16*>(is_a ? g.a : g.b) + off;
        const int nv = min(8, (int) (g.k - kl));
        bytes = (uint32_t) nv * 2u;
    }
    cp_async16(dst, src, bytes);
}

// the A and B tiles of K block kb by asynchronous copies (async_ok products)
__device__ __forceinline__ void async_stage(
    const gemm_params& p, int z, int m0, int n0, int kb, uint32_t sa, uint32_t sb)
{
    const int k0 = kb * BK;
    // K chunks first: a warp's 32 copies cover four rows of 128 contiguous bytes
#pragma unroll
    for (int i = 0; i < BM * (BK / 8) / NTH; i++) {
        const int c = threadIdx.x + i * NTH, row = c >> 3, kc = c & 7;
        async_chunk(p, true, z, m0 + row, p.m, k0 + kc * 8, sa + (uint32_t) (((row >> 3) * (BK / 8) + kc) * 128 +
                                                                                 (row & 7) * 16));
    }
#pragma unroll
    for (int i = 0; i < BN * (BK / 8) / NTH; i++) {
        const int c = threadIdx.x + i * NTH, row = c >> 3, kc = c & 7;
        async_chunk(p, false, z, n0 + row, p.n, k0 + kc * 8, sb + (uint32_t) (((row >> 3) * (BK / 8) + kc) * 128 +
                                                                                  (row & 7) * 16));
    }
}

// one 16-byte row of a core matrix, as BF16
__device__ __forceinline__ void store_chunk(uint32_t dst, const float (&v)[8])
{
    const uint32_t w0 = pack_bf16(v[0], v[1]), w1 = pack_bf16(v[2], v[3]);
    const uint32_t w2 = pack_bf16(v[4], v[5]), w3 = pack_bf16(v[6], v[7]);
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(dst), "r"(w0), "r"(w1), "r"(w2), "r"(w3)
                 : "memory");
}

// smem byte offset of the 16-byte chunk (row, kc) of a tile
__device__ __forceinline__ uint32_t chunk_off(int row, int kc)
{
    return (uint32_t) (((row >> 3) * (BK / 8) + kc) * 128 + (row & 7) * 16);
}

constexpr int A_CHUNKS = BM * (BK / 8) / NTH;  // 8 per thread
constexpr int B_CHUNKS = BN * (BK / 8) / NTH;  // 4 per thread

// row and K chunk of chunk c: rows first when the operand's rows are
// adjacent in memory (row stride 1), 16-byte K chunks first otherwise
__device__ __forceinline__ void chunk_pos(int c, int R, bool rows_first, int& row, int& kc)
{
    if (rows_first) {
        row = c % R;
        kc = c / R;
    } else {
        row = (c >> 6) * 8 + (c & 7);
        kc = (c >> 3) & 7;
    }
}

// Stage the A (BM x BK) and B (BN x BK) tiles of K block kb: every global
// load of the thread is issued before the first shared-memory store, so
// that their latencies overlap.
__device__ __forceinline__ void load_stage(
    const gemm_params& p, int z, int m0, int n0, int kb, uint32_t sa, uint32_t sb)
{
    const int k0 = kb * BK;
    int s = 0;
    if (p.nseg > 1 && k0 >= p.kstart[1]) s = 1;
    if (p.nseg > 2 && k0 >= p.kstart[2]) s = 2;
    const bool a_rows = p.seg[s].a_sm == 1;
    const bool b_rows = p.seg[s].b_sn == 1;
    float va[A_CHUNKS][8], vb[B_CHUNKS][8];
#pragma unroll
    for (int i = 0; i < A_CHUNKS; i++) {
        int row, kc;
        chunk_pos(threadIdx.x + i * NTH, BM, a_rows, row, kc);
        gather_chunk(p, true, z, m0 + row, p.m, k0 + kc * 8, va[i]);
    }
#pragma unroll
    for (int i = 0; i < B_CHUNKS; i++) {
        int row, kc;
        chunk_pos(threadIdx.x + i * NTH, BN, b_rows, row, kc);
        gather_chunk(p, false, z, n0 + row, p.n, k0 + kc * 8, vb[i]);
    }
#pragma unroll
    for (int i = 0; i < A_CHUNKS; i++) {
        int row, kc;
        chunk_pos(threadIdx.x + i * NTH, BM, a_rows, row, kc);
        store_chunk(sa + chunk_off(row, kc), va[i]);
    }
#pragma unroll
    for (int i = 0; i < B_CHUNKS; i++) {
        int row, kc;
        chunk_pos(threadIdx.x + i * NTH, BN, b_rows, row, kc);
        store_chunk(sb + chunk_off(row, kc), vb[i]);
    }
}

template<int STAGES, int AHEAD>
__global__ void __launch_bounds__(NTH) gemm_kernel(const gemm_params p)
{
    extern __shared__ __align__(128) uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t mbar[STAGES];
    __shared__ uint32_t tmem_sh;
    __shared__ int fail_sh;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ntn = (p.n + BN - 1) / BN;
    const int m0 = (blockIdx.x / ntn) * BM;
    const int n0 = (blockIdx.x % ntn) * BN;
    const int z = blockIdx.z;
    const int kblocks = (p.ktotal + BK - 1) / BK;
    const int kb0 = blockIdx.y * p.kblocks_per_split;
    const int kb1 = min(kblocks, kb0 + p.kblocks_per_split);
    const int nit = kb1 - kb0;

    const uint32_t base = (smem_u32(smem_raw) + 127u) & ~127u;
    const uint32_t mb0 = smem_u32(&mbar[0]);

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_sh)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) mbar_init(mb0 + 8u * s, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fail_sh = 0;
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_sh;

    // stage block j: asynchronously where every operand allows it, else by
    // plain loads (complete when the call returns)
    auto stage = [&](int j) {
        const uint32_t sa = base + (uint32_t) ((j % STAGES) * STAGE_BYTES);
        if (AHEAD > 0)  // only the asynchronous instantiation stages ahead
            async_stage(p, z, m0, n0, kb0 + j, sa, sa + (uint32_t) A_BYTES);
        else
            load_stage(p, z, m0, n0, kb0 + j, sa, sa + (uint32_t) A_BYTES);
    };
    // exactly AHEAD copy groups before the loop (empty ones when there are
    // fewer blocks), so that waiting for all but the AHEAD most recent groups
    // in iteration it always covers block it
    for (int j = 0; j < AHEAD; j++) {
        if (j < nit) stage(j);
        cp_async_commit();
    }
    for (int it = 0; it < nit; it++) {
        const int st = it % STAGES;
        const int ahead = it + AHEAD;
        bool ok_wait = true;
        if (ahead < nit) {
            // the MMAs that read this stage STAGES blocks ago must be done
            if (ahead >= STAGES)
                ok_wait = mbar_wait(mb0 + 8u * (ahead % STAGES), (uint32_t) (((ahead - STAGES) / STAGES) & 1));
            if (ok_wait) stage(ahead);
        }
        if (!ok_wait) fail_sh = 1;
        cp_async_commit();
        cp_async_wait<AHEAD>();  // block it has landed (this thread's copies)
        fence_async_smem();
        __syncthreads();
        if (fail_sh) break;
        if (tid == 0) {
            fence_after();
            const uint32_t sa = base + (uint32_t) (st * STAGE_BYTES);
            const uint32_t sb = sa + (uint32_t) A_BYTES;
#pragma unroll
            for (int kk = 0; kk < BK / 16; kk++) {
                const uint64_t ad = smem_desc(sa + (uint32_t) (kk * 256));
                const uint64_t bd = smem_desc(sb + (uint32_t) (kk * 256));
                mma_bf16(tmem, ad, bd, IDESC, (it > 0 || kk > 0) ? 1u : 0u);
            }
            mma_commit(mb0 + 8u * st);
        }
    }
    cp_async_wait<0>();  // no copy outlives the loop (a break leaves some in flight)

    bool ok = !fail_sh && nit > 0;
    if (ok) {
        const int last = nit - 1;
        if (!mbar_wait(mb0 + 8u * (last % STAGES), (uint32_t) ((last / STAGES) & 1))) fail_sh = 1;
    }
    __syncthreads();
    ok = ok && !fail_sh;
    fence_after();

    if (ok) {
        // The accumulator comes out of TMEM one row per thread; it goes
        // through shared memory (the stages are free: every MMA has
        // completed) so that the epilogue reads and writes C, pre and gate
        // along their contiguous dimension (a row per thread would make a
        // warp's every access touch 32 rows).
        constexpr int LD = BN + 1;  // odd stride: conflict-free both ways
        float* tile = reinterpret_cast<float*>(smem_raw + (base - smem_u32(smem_raw)));
        const int r0 = warp * 32 + lane;
#pragma unroll 1
        for (int cb = 0; cb < BN / 16; cb++) {
            float acc[16];
            tmem_ld16(tmem + ((uint32_t) (warp * 32) << 16) + (uint32_t) (cb * 16), acc);
            if (p.fin) {
#pragma unroll
                for (int i = 0; i < 16; i++) {
                    const int col = n0 + cb * 16 + i;
                    float v = p.alpha * acc[i];
                    if (p.bias && col < p.n) v += p.bias[col];
                    if (p.act == MBG_ACT_GELU) v = gelu(v);
                    acc[i] = v;
                }
            }
#pragma unroll
            for (int i = 0; i < 16; i++) tile[r0 * LD + cb * 16 + i] = acc[i];
        }
        __syncthreads();
        // final value of tile entry (r, cc) in STORE mode without pre or gate
        auto value = [&](int r, int cc) { return tile[r * LD + cc]; };
        const bool rows_fast = p.c_sn != 1 && p.c_sm == 1;
        if (p.rowdot) {
            // a second product folded into the epilogue: each row's outputs
            // dotted with rowdot (both rounded to BF16, as a product's
            // operands), one atomic add per row and tile into the FP32
            // vector C (the first column tile adds rowdot_bias)
            const int row = m0 + tid;
            if (row < p.m) {
                float s = (n0 == 0 && p.rowdot_bias) ? *p.rowdot_bias : 0.0f;
                for (int cc = 0; cc < BN && n0 + cc < p.n; cc++) {
                    const float a = __bfloat162float(__float2bfloat16_rn(value(tid, cc)));
                    const float w = __bfloat162float(__float2bfloat16_rn(p.rowdot[n0 + cc]));
                    s = fmaf(a, w, s);
                }
                atomicAdd(reinterpret_cast<float*>(p.c) + (int64_t) z * p.c_sz + (int64_t) row * p.c_sm, s);
            }
        } else if (p.vec_c) {
            // 8 consecutive outputs of a row per 16-byte (BF16) or 2 x 16-byte
            // (FP32) store; a warp writes four rows of 64 outputs
#pragma unroll 1
            for (int e = tid; e < BM * (BN / 8); e += NTH) {
                const int r = e >> 3, c0 = (e & 7) * 8;
                const int row = m0 + r, col0 = n0 + c0;
                if (row >= p.m || col0 >= p.n) continue;
                const int64_t off = (int64_t) z * p.c_sz + (int64_t) row * p.c_sm + col0;
                if (col0 + 8 <= p.n) {
                    float v[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) v[i] = value(r, c0 + i);
                    if (p.c_type == MBG_BF16) {
                        const uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]),
                                                   pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
                        *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(p.c) + off) = q;
                    } else {
                        float4* d4 = reinterpret_cast<float4*>(reinterpret_cast<float*>(p.c) + off);
                        d4[0] = make_float4(v[0], v[1], v[2], v[3]);
                        d4[1] = make_float4(v[4], v[5], v[6], v[7]);
                    }
                } else {
                    for (int i = 0; col0 + i < p.n; i++) {
                        const float v = value(r, c0 + i);
                        if (p.c_type == MBG_BF16)
                            reinterpret_cast<__nv_bfloat16*>(p.c)[off + i] = __float2bfloat16_rn(v);
                        else
                            reinterpret_cast<float*>(p.c)[off + i] = v;
                    }
                }
            }
        }
#pragma unroll 1
        for (int e = (p.vec_c || p.rowdot) ? BM * BN : tid; e < BM * BN; e += NTH) {
            const int r = rows_fast ? e % BM : e / BN;
            const int cc = rows_fast ? e / BM : e % BN;
            const int row = m0 + r, col = n0 + cc;
            if (row >= p.m || col >= p.n) continue;
            const int64_t off = (int64_t) z * p.c_sz + (int64_t) row * p.c_sm + (int64_t) col * p.c_sn;
            if (p.fin) {
                const float v = tile[r * LD + cc];
                if (p.c_type == MBG_BF16)
                    reinterpret_cast<__nv_bfloat16*>(p.c)[off] = __float2bfloat16_rn(v);
                else
                    reinterpret_cast<float*>(p.c)[off] = v;
                continue;
            }
            float v = p.alpha * tile[r * LD + cc];
            if (p.mode == MBG_GEMM_ATOMIC) {
                atomicAdd(reinterpret_cast<float*>(p.c) + off, v);
                continue;
            }
            if (p.mode == MBG_GEMM_ACCUM) v += ld_elem(p.c, p.c_type, off);
            if (p.bias) v += p.bias[col];
            if (p.pre) p.pre[off] = v;
            if (p.act == MBG_ACT_GELU)
                v = gelu(v);
            else if (p.act == MBG_ACT_GELU_BWD)
                v *= gelu_grad(p.gate[off]);
            if (p.c_type == MBG_BF16)
                reinterpret_cast<__nv_bfloat16*>(p.c)[off] = __float2bfloat16_rn(v);
            else
                reinterpret_cast<float*>(p.c)[off] = v;
        }
        if (p.c2 && p.vec_c2) {
            // the same values (STORE mode) as BF16 in a second layout whose
            // rows are contiguous (e.g. the transposed copy the next product
            // reads with K contiguous): 8 rows of a column per 16-byte store,
            // a warp writes two columns of 128 rows
#pragma unroll 1
            for (int e = tid; e < BM * BN / 8; e += NTH) {
                const int rc = e & (BM / 8 - 1), cc = e / (BM / 8);
                const int r0 = rc * 8, row0 = m0 + r0, col = n0 + cc;
                if (row0 >= p.m || col >= p.n) continue;
                const int64_t off = (int64_t) z * p.c2_sz + row0 + (int64_t) col * p.c2_sn;
                if (row0 + 8 <= p.m) {
                    float v[8];
#pragma unroll
                    for (int i = 0; i < 8; i++) v[i] = value(r0 + i, cc);
                    const uint4 q = make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]),
                                               pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
                    *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(p.c2) + off) = q;
                } else {
                    for (int i = 0; row0 + i < p.m; i++)
                        reinterpret_cast<__nv_bfloat16*>(p.c2)[off + i] = __float2bfloat16_rn(value(r0 + i, cc));
                }
            }
        } else if (p.c2) {
            // the same values (STORE mode) as BF16 in a second layout,
            // written along its own contiguous dimension
            const bool rows_fast2 = p.c2_sn != 1 && p.c2_sm == 1;
#pragma unroll 1
            for (int e = tid; e < BM * BN; e += NTH) {
                const int r = rows_fast2 ? e % BM : e / BN;
                const int cc = rows_fast2 ? e / BM : e % BN;
                const int row = m0 + r, col = n0 + cc;
                if (row >= p.m || col >= p.n) continue;
                const float v = value(r, cc);
                const int64_t off = (int64_t) z * p.c2_sz + (int64_t) row * p.c2_sm + (int64_t) col * p.c2_sn;
                reinterpret_cast<__nv_bfloat16*>(p.c2)[off] = __float2bfloat16_rn(v);
            }
        }
    }
    if (fail_sh && tid == 0) atomicOr(p.status, ST_WAIT);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ------------------------------------------------------------ small kernels

__global__ void mode_blocks_kernel(const float* wr, const float* wi, int modes, int width, __nv_bfloat16* blk)
{
    const int W2 = 2 * width;
    const int64_t total = (int64_t) modes * W2 * W2;
    for (int64_t t = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; t < total;
         t += (int64_t) gridDim.x * blockDim.x) {
        const int k = (int) (t % W2);              // input index: [Re x | Im x]
        const int j = (int) ((t / W2) % W2);       // output index: [Re y | Im y]
        const int m = (int) (t / ((int64_t) W2 * W2));
        const int c = k % width, o = j % width;
        const int64_t w = ((int64_t) m * width + c) * width + o;
        float v;
        if ((j < width) == (k < width))
            v = wr[w];                             // Re y <- Re x, Im y <- Im x
        else if (j < width)
            v = -wi[w];                            // Re y <- -wi Im x
        else
            v = wi[w];                             // Im y <- wi Re x
        blk[t] = __float2bfloat16_rn(v);
    }
}

__global__ void cast_kernel(const float* x, __nv_bfloat16* y, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

// img[z] = the K-major core-matrix image of the R x K matrix whose (r, c)
// entry is x[z zs + r ld + c] (zero outside rows x cols), as BF16
__global__ void image_kernel(const float* x, int batch, int rows, int cols, int64_t ld, int64_t zs, int R, int K,
                             __nv_bfloat16* img)
{
    const int64_t per = (int64_t) R * K, total = per * batch;
    for (int64_t t = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; t < total;
         t += (int64_t) gridDim.x * blockDim.x) {
        const int64_t z = t / per, e = t % per;
        const int blk = (int) (e >> 6), r = (blk / (K / 8)) * 8 + (int) ((e >> 3) & 7),
                  c = (blk % (K / 8)) * 8 + (int) (e & 7);
        img[t] = __float2bfloat16_rn(r < rows && c < cols ? x[z * zs + r * ld + c] : 0.0f);
    }
}

// one CTA per (column, row slice): strided partial sums, then atomics
__global__ void colsum_kernel(const float* x, int64_t rows, int cols, int64_t rs, float* out)
{
    const int col = blockIdx.x;
    float s = 0.0f;
    for (int64_t r = blockIdx.y * (int64_t) blockDim.x + threadIdx.x; r < rows; r += (int64_t) gridDim.y * blockDim.x)
        s += x[r * rs + col];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ float part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.0f;
        for (int w = 0; w < (int) (blockDim.x >> 5); w++) t += part[w];
        atomicAdd(out + col, t);
    }
}

__global__ void mse_kernel(const float* y, const float* t, int64_t n, float* grad, float* loss)
{
    float s = 0.0f;
    const float inv = 1.0f / (float) n;
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
        const float d = y[i] - t[i];
        grad[i] = 2.0f * d * inv;
        s += d * d * inv;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s);
}

__global__ void adam_kernel(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                            float eps, float wd, float c1, float c2)
{
    for (int64_t i = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; i < n; i += (int64_t) gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float mh = mi / c1, vh = vi / c2;
        w[i] -= lr * (mh / (sqrtf(vh) + eps) + wd * w[i]);
    }
}

__global__ void envelope_kernel(const double* e, int runs, int rows, int64_t rs, double t0, double dt, double f0,
                                int nout, double tout0, double dtout, float* out)
{
    const int64_t total = (int64_t) runs * nout;
    const double half = 0.5 / f0;
    const double w = 2.0 * 3.14159265358979323846 * f0;
    for (int64_t t = blockIdx.x * (int64_t) blockDim.x + threadIdx.x; t < total;
         t += (int64_t) gridDim.x * blockDim.x) {
        const int r = (int) (t / nout), j = (int) (t % nout);
        const double tc = tout0 + j * dtout;
        int i0 = (int) ceil((tc - half - t0) / dt);
        int i1 = (int) floor((tc + half - t0) / dt);
        i0 = max(i0, 0);
        i1 = min(i1, rows - 1);
        double re = 0.0, im = 0.0;
        int cnt = 0;
        for (int i = i0; i <= i1; i++) {
            const double ti = t0 + i * dt;
            double sn, cs;
            sincos(w * ti, &sn, &cs);
            const double x = e[(int64_t) r * rs + i];
            re += x * cs;
            im -= x * sn;
            cnt++;
        }
        out[t] = cnt > 0 ? (float) (2.0 * sqrt(re * re + im * im) / cnt) : 0.0f;
    }
}

// ------------------------------------------------------------ host side

struct status_slot {
    std::mutex mu;
    uint32_t* dev[64] = {};
};
status_slot g_status;

uint32_t* status_ptr()
{
    int d = 0;
    if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= 64) throw std::runtime_error("CUDA: no current device");
    std::lock_guard<std::mutex> lk(g_status.mu);
    if (!g_status.dev[d]) {
        uint32_t* p = nullptr;
        if (cudaMalloc(&p, sizeof(uint32_t)) != cudaSuccess) throw std::runtime_error("CUDA: status allocation failed");
        if (cudaMemset(p, 0, sizeof(uint32_t)) != cudaSuccess) throw std::runtime_error("CUDA: status memset failed");
        g_status.dev[d] = p;
    }
    return g_status.dev[d];
}

void check_launch(const char* what)
{
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + what + ": " + cudaGetErrorString(e));
}

int blocks_for(int64_t n, int per)
{
    int64_t b = (n + per - 1) / per;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int) b;
}

void require(bool c, const char* msg)
{
    if (!c) throw std::invalid_argument(msg);
}

void gemm(const mbg_gemm_desc* d, cudaStream_t s)
{
    require(d != nullptr, "gemm: null descriptor");
    require(d->m > 0 && d->n > 0 && d->batch > 0 && d->batch <= 65535, "gemm: bad m, n or batch");
    require(d->nseg >= 1 && d->nseg <= 3, "gemm: nseg must be 1..3");
    require(d->c != nullptr, "gemm: null C");
    require(d->c_type == MBG_F32 || d->c_type == MBG_BF16, "gemm: bad C type");
    require(d->mode >= MBG_GEMM_STORE && d->mode <= MBG_GEMM_ATOMIC, "gemm: bad mode");
    require(d->act >= MBG_ACT_NONE && d->act <= MBG_ACT_GELU_BWD, "gemm: bad activation");
    require(d->act != MBG_ACT_GELU_BWD || d->gate != nullptr, "gemm: GELU_BWD needs gate");
    if (d->mode == MBG_GEMM_ATOMIC)
        require(d->c_type == MBG_F32 && !d->bias && !d->pre && d->act == MBG_ACT_NONE,
                "gemm: ATOMIC mode takes an FP32 C and no epilogue");
    else
        require(d->split_k <= 1, "gemm: split_k needs ATOMIC mode");
    gemm_params p{};
    p.m = d->m;
    p.n = d->n;
    p.nseg = d->nseg;
    int kt = 0;
    for (int i = 0; i < d->nseg; i++) {
        const mbg_gemm_segment& g = d->seg[i];
        require(g.a && g.b && g.k > 0, "gemm: empty segment");
        require((g.a_type == MBG_F32 || g.a_type == MBG_BF16) && (g.b_type == MBG_F32 || g.b_type == MBG_BF16),
                "gemm: bad operand type");
        require(i == d->nseg - 1 || g.k % 8 == 0, "gemm: all segments but the last need k % 8 == 0");
        p.kstart[i] = kt;
        kt += g.k;
        p.seg[i] = seg_t{ g.a, g.b, g.a_sm, g.a_sk, g.a_sz, g.b_sn, g.b_sk, g.b_sz, g.k, g.a_type, g.b_type,
                          g.negate };
    }
    p.kstart[d->nseg] = kt;
    p.ktotal = kt;
    // asynchronous 16-byte copies need BF16 operands with K contiguous and
    // every row (and batch) start on a 16-byte boundary, and no negation
    bool async_ok = true;
    for (int i = 0; i < d->nseg; i++) {
        const mbg_gemm_segment& g = d->seg[i];
        const bool ok = g.a_type == MBG_BF16 && g.b_type == MBG_BF16 && g.a_sk == 1 && g.b_sk == 1 &&
            g.a_sm % 8 == 0 && g.b_sn % 8 == 0 && g.a_sz % 8 == 0 && g.b_sz % 8 == 0 &&
            (reinterpret_cast<uintptr_t>(g.a) & 15) == 0 && (reinterpret_cast<uintptr_t>(g.b) & 15) == 0 &&
            !g.negate && (i == d->nseg - 1 || g.k % 8 == 0);
        async_ok = async_ok && ok;
    }
    p.async_ok = async_ok ? 1 : 0;
    // STORE mode without pre-activation or gate: the finished values are
    // computed once, into the shared tile, and may be stored twice
    const bool plain_store = d->mode == MBG_GEMM_STORE && !d->pre && !d->gate && d->act != MBG_ACT_GELU_BWD;
    require(!d->c2 || plain_store, "gemm: a second output needs STORE mode without pre, gate or GELU_BWD");
    p.c2 = d->c2;
    p.c2_sm = d->c2_sm;
    p.c2_sn = d->c2_sn;
    p.c2_sz = d->c2_sz;
    // vectorised epilogues: the stored dimension contiguous, every 8-output
    // chunk 16-byte aligned
    const int64_t cw = d->c_type == MBG_BF16 ? 8 : 4;
    p.vec_c = plain_store && d->c_sn == 1 && d->c_sm % cw == 0 && d->c_sz % cw == 0 &&
        (reinterpret_cast<uintptr_t>(d->c) & 15) == 0;
    p.vec_c2 = d->c2 && d->c2_sm == 1 && d->c2_sn % 8 == 0 && d->c2_sz % 8 == 0 &&
        (reinterpret_cast<uintptr_t>(d->c2) & 15) == 0;
    require(!d->rowdot || (plain_store && !d->c2 && d->c_type == MBG_F32 && d->act != MBG_ACT_GELU_BWD),
            "gemm: rowdot needs STORE mode, an FP32 C and no second output");
    p.rowdot = d->rowdot;
    p.rowdot_bias = d->rowdot_bias;
    if (p.rowdot) p.vec_c = 0;
    p.fin = plain_store ? 1 : 0;
    p.c = d->c;
    p.c_sm = d->c_sm;
    p.c_sn = d->c_sn;
    p.c_sz = d->c_sz;
    p.c_type = d->c_type;
    p.mode = d->mode;
    p.act = d->act;
    p.alpha = d->alpha;
    p.bias = d->bias;
    p.pre = d->pre;
    p.gate = d->gate;
    p.status = status_ptr();
    const int kblocks = (kt + BK - 1) / BK;
    int split = d->split_k < 1 ? 1 : d->split_k;
    if (split > kblocks) split = kblocks;
    p.kblocks_per_split = (kblocks + split - 1) / split;
    const int ysplits = (kblocks + p.kblocks_per_split - 1) / p.kblocks_per_split;
    const int64_t tiles = (int64_t) ((d->m + BM - 1) / BM) * ((d->n + BN - 1) / BN);
    require(tiles <= 0x7fffffff, "gemm: too many tiles");
    static std::once_flag attr;
    std::call_once(attr, [] {
        cudaFuncSetAttribute(gemm_kernel<STAGES_ASYNC, AHEAD_ASYNC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_bytes(STAGES_ASYNC));
        cudaFuncSetAttribute(gemm_kernel<STAGES_GATHER, AHEAD_GATHER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_bytes(STAGES_GATHER));
        cudaFuncSetAttribute(gemm_kernel<STAGES_SHORT, AHEAD_SHORT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem_bytes(STAGES_SHORT));
    });
    const dim3 grid((unsigned) tiles, (unsigned) ysplits, (unsigned) d->batch);
    // (with at most AHEAD_SHORT = STAGES_SHORT blocks every block is staged
    // before the loop, so no stage is ever reused)
    if (p.async_ok && p.kblocks_per_split <= STAGES_SHORT)
        gemm_kernel<STAGES_SHORT, AHEAD_SHORT><<<grid, NTH, smem_bytes(STAGES_SHORT), s>>>(p);
    else if (p.async_ok)
        gemm_kernel<STAGES_ASYNC, AHEAD_ASYNC><<<grid, NTH, smem_bytes(STAGES_ASYNC), s>>>(p);
    else
        gemm_kernel<STAGES_GATHER, AHEAD_GATHER><<<grid, NTH, smem_bytes(STAGES_GATHER), s>>>(p);
    check_launch("gemm_kernel");
}

}  // namespace fno
}  // namespace mbg

using namespace mbg::fno;

extern "C" {

int mbg_fno_gemm(const mbg_gemm_desc* d, void* stream)
{
    return guard([&] { gemm(d, (cudaStream_t) stream); });
}

int mbg_fno_mode_blocks(const float* wr, const float* wi, int32_t modes, int32_t width, void* blk, void* stream)
{
    return guard([&] {
        require(wr && wi && blk && modes > 0 && width > 0, "mode_blocks: bad arguments");
        const int64_t n = (int64_t) modes * 4 * width * width;
        mode_blocks_kernel<<<blocks_for(n), 256, 0, (cudaStream_t) stream>>>(wr, wi, modes, width,
                                                                             (__nv_bfloat16*) blk);
        check_launch("mode_blocks_kernel");
    });
}

int mbg_fno_cast_bf16(const float* x, void* y, int64_t n, void* stream)
{
    return guard([&] {
        require(x && y && n > 0, "cast_bf16: bad arguments");
        cast_kernel<<<blocks_for(n), 256, 0, (cudaStream_t) stream>>>(x, (__nv_bfloat16*) y, n);
        check_launch("cast_kernel");
    });
}

int mbg_fno_image_bf16(const float* x, int32_t batch, int32_t rows, int32_t cols, int64_t ld, int64_t zs,
                       int32_t R, int32_t K, void* img, void* stream)
{
    return guard([&] {
        require(x && img && batch > 0 && rows > 0 && cols > 0, "image_bf16: bad arguments");
        require(R >= rows && K >= cols && R % 8 == 0 && K % 8 == 0, "image_bf16: R, K must cover rows, cols and be multiples of 8");
        require(ld >= cols && (batch == 1 || zs > 0), "image_bf16: bad strides");
        const int64_t n = (int64_t) batch * R * K;
        image_kernel<<<blocks_for(n), 256, 0, (cudaStream_t) stream>>>(x, batch, rows, cols, ld, zs, R, K,
                                                                       (__nv_bfloat16*) img);
        check_launch("image_kernel");
    });
}

int mbg_fno_colsum(const float* x, int64_t rows, int32_t cols, int64_t row_stride, float* out, void* stream)
{
    return guard([&] {
        require(x && out && rows > 0 && cols > 0 && cols <= 65535 && row_stride >= cols, "colsum: bad arguments");
        int ys = (int) ((rows + 255) / 256);
        if (ys > 64) ys = 64;
        colsum_kernel<<<dim3((unsigned) cols, (unsigned) ys), 256, 0, (cudaStream_t) stream>>>(x, rows, cols,
                                                                                            row_stride, out);
        check_launch("colsum_kernel");
    });
}

int mbg_fno_mse(const float* y, const float* t, int64_t n, float* grad, float* loss, void* stream)
{
    return guard([&] {
        require(y && t && grad && loss && n > 0, "mse: bad arguments");
        mse_kernel<<<blocks_for(n), 256, 0, (cudaStream_t) stream>>>(y, t, n, grad, loss);
        check_launch("mse_kernel");
    });
}

int mbg_fno_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float beta1, float beta2,
                 float eps, float weight_decay, int32_t step, void* stream)
{
    return guard([&] {
        require(w && g && m && v && n > 0 && step >= 1, "adam: bad arguments");
        const float c1 = 1.0f - powf(beta1, (float) step), c2 = 1.0f - powf(beta2, (float) step);
        adam_kernel<<<blocks_for(n), 256, 0, (cudaStream_t) stream>>>(w, g, m, v, n, lr, beta1, beta2, eps,
                                                                      weight_decay, c1, c2);
        check_launch("adam_kernel");
    });
}

int mbg_fno_envelope(const double* e, int32_t runs, int32_t rows, int64_t run_stride, double t0, double dt,
                     double f0, int32_t nout, double tout0, double dtout, float* out, void* stream)
{
    return guard([&] {
        require(e && out && runs > 0 && rows > 0 && nout > 0 && run_stride >= rows, "envelope: bad arguments");
        require(dt > 0 && f0 > 0 && dtout > 0, "envelope: dt, f0 and dtout must be positive");
        const int64_t n = (int64_t) runs * nout;
        envelope_kernel<<<blocks_for(n), 256, 0, (cudaStream_t) stream>>>(e, runs, rows, run_stride, t0, dt, f0,
                                                                          nout, tout0, dtout, out);
        check_launch("envelope_kernel");
    });
}

int mbg_fno_status(uint32_t* status)
{
    return guard([&] {
        require(status != nullptr, "status: null pointer");
        uint32_t* p = status_ptr();
        if (cudaMemcpy(status, p, sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
            throw std::runtime_error("CUDA: status read failed");
        if (cudaMemset(p, 0, sizeof(uint32_t)) != cudaSuccess) throw std::runtime_error("CUDA: status clear failed");
    });
}

}  // extern "C"
