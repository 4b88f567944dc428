// Tensor-core form of the coherence-vector step for 4 to 6 levels
// (FP32 kernels, uniform tiles, 128 points per CTA, one per thread).
//
// Each step's correction Bd v + k (after the field rotation; see
// cvr_layout) is, over the CTA's 128 points, the product
// D[128 x V] = U[128 x V] Bd^T: thread t's coherence vector is row
// t of U and row t of D lands in TMEM lane t, i.e. back in thread t's
// registers (tcgen05.ld 32x32b). The product runs as tcgen05.mma
// kind::tf32 (M = 128, N = V rounded up to 16, K = V rounded up to 8) with
// FP32 accumulation in TMEM, split into TF32 parts (rounded to nearest) for
// FP32 accuracy: Bd u ~ Bd_hi u_hi + Bd_lo u_hi + Bd_hi u_lo (the dropped
// Bd_lo u_lo is ~2^-22 of the product, and random); a second accumulator
// takes Bd_rest u_hi, the remainder of Bd + Bdl (Bdl = Bd - fl32(Bd), the
// low-word correction of the FP32 kernels) beyond Bd_hi + Bd_lo, so the
// propagator itself is represented to ~2^-33. Operands sit in shared memory
// in the no-swizzle K-major
// core-matrix layout (8 rows x 16 bytes per core matrix; 128 bytes between
// K-adjacent core matrices, K/4 x 128 bytes between 8-row groups).
//
// One thread issues the MMAs and commits them to an mbarrier; every wait is
// bounded and a time-out stops the tile (status flag) instead of hanging.
#pragma once

#include <cstdint>

#include "kernels.cuh"

namespace mbg {
namespace tc {

constexpr int M = 128;                     // points per CTA (TMEM lanes)
constexpr uint32_t WAIT_LIMIT = 1u << 22;
constexpr uint32_t TMEM_COLS = 128;        // D0 at column 0, D1 at column 64
constexpr uint32_t D1_COL = 64;

template<int V>
struct shape {
    static constexpr int K = (V + 7) / 8 * 8;      // TF32: 8 per MMA
    static constexpr int N = (V + 15) / 16 * 16;   // M = 128 needs N % 16 == 0
    static constexpr int KC = K / 4;               // 16-byte chunks per row
    static constexpr uint32_t SBO = (uint32_t) KC * 128u;
    static constexpr uint32_t A_BYTES = (uint32_t) M * K * 4u;
    static constexpr uint32_t B_BYTES = (uint32_t) N * K * 4u;
    // A_hi, A_lo, B_hi, B_lo, B_dl
    static constexpr uint32_t BYTES = 2u * A_BYTES + 3u * B_BYTES;
    static_assert(N <= 64, "two accumulators of N columns must fit 128 TMEM columns");
};

// byte offset of the 16-byte chunk (row, kc) in a K-major operand
template<int V>
__device__ __forceinline__ uint32_t chunk(int row, int kc)
{
    return (uint32_t) (((row >> 3) * shape<V>::KC + kc) * 128 + (row & 7) * 16);
}

template<int V>
__device__ __forceinline__ uint64_t desc(uint32_t addr)
{
    uint64_t d = 0;
    d |= (uint64_t) ((addr >> 4) & 0x3FFFu);
    d |= (uint64_t) ((128u >> 4) & 0x3FFFu) << 16;           // leading (K) offset
    d |= (uint64_t) ((shape<V>::SBO >> 4) & 0x3FFFu) << 32;  // stride (M/N) offset
    d |= (uint64_t) 1u << 46;                                // descriptor version
    return d;
}

// kind::tf32: FP32 accumulator (bits 4-5 = 1), A and B TF32 (bits 7-9 and
// 10-12 = 2), K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
template<int V>
constexpr uint32_t idesc()
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t) (shape<V>::N >> 3) << 17) |
        ((uint32_t) (M >> 4) << 24);
}

// x rounded to the nearest TF32 (10 explicit mantissa bits); x - hi is exact
__device__ __forceinline__ float tf32_hi(float x)
{
    const uint32_t u = __float_as_uint(x);
    return __uint_as_float((u + 0x1000u) & 0xFFFFE000u);
}

struct ctx {
    uint32_t a_hi, a_lo, b_hi, b_lo, b_dl;
    float* rows;  // the A_hi region as plain rows of V floats (mixed tiles)
    uint32_t tmem;
    uint32_t mbar;
    uint32_t phase;
    uint32_t wait_limit;  // polls of a completion wait
};

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc)
{
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint32_t limit)
{
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t ok;
        asm volatile(
            "{\n"
            ".reg .pred P;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n"
            "selp.b32 %0, 1, 0, P;\n"
            "}\n"
            : "=r"(ok)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void st16(uint32_t a, float x, float y, float z, float w)
{
    asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(x), "f"(y), "f"(z), "f"(w) : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Stage the B operands from the material block in global memory (layout of
// make_cvr_layout: Bd at FDTD_END, Bdl after it, both V x V row-major):
// Bd + Bdl = B_hi + B_lo + B_rest with B_hi and B_lo TF32 numbers (rounded
// to nearest) and B_rest the FP32 remainder. The tensor cores read only a
// TF32 number's bits, so a B_lo that was not itself a TF32 number would be
// truncated: a fixed error of ~2^-22 of Bd per material, larger than the
// Bdl correction. The second accumulator takes B_rest (D1 = A_hi B_rest).
// Rows n >= V and columns k >= V are zero. Called by all threads; a barrier
// must follow.
template<int V>
__device__ __forceinline__ void stage_b(const ctx& c, const float* mat)
{
    using S = shape<V>;
    const float* bd = mat + pre::FDTD_END;
    const float* bdl = bd + V * V;
    for (int e = threadIdx.x; e < S::N * S::KC; e += M) {
        const int n = e / S::KC, kc = e % S::KC;
        float h[4], l[4], dl[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int k = kc * 4 + q;
            const bool in = n < V && k < V;
            const float b = in ? bd[n * V + k] : 0.0f;
            h[q] = tf32_hi(b);
            const float r = b - h[q];           // exact
            l[q] = tf32_hi(r);
            dl[q] = (r - l[q]) + (in ? bdl[n * V + k] : 0.0f);
        }
        const uint32_t o = chunk<V>(n, kc);
        st16(c.b_hi + o, h[0], h[1], h[2], h[3]);
        st16(c.b_lo + o, l[0], l[1], l[2], l[3]);
        st16(c.b_dl + o, dl[0], dl[1], dl[2], dl[3]);
    }
}

// Write this thread's vector x (row threadIdx.x of A) as TF32 high and low
// parts; columns V..K-1 are zero.
template<int V>
__device__ __forceinline__ void write_row(const ctx& c, const float (&x)[V])
{
    using S = shape<V>;
    const int row = threadIdx.x;
    static_for<0, S::KC>([&](auto KCI) {
        constexpr int kc = decltype(KCI)::value;
        float h[4], l[4];
        static_for<0, 4>([&](auto QI) {
            constexpr int q = decltype(QI)::value;
            constexpr int k = kc * 4 + q;
            if constexpr (k < V) {
                h[q] = tf32_hi(x[k]);
                l[q] = tf32_hi(x[k] - h[q]);  // rounded, not truncated, by the MMA
            } else {
                h[q] = 0.0f;
                l[q] = 0.0f;
            }
        });
        const uint32_t o = chunk<V>(row, kc);
        st16(c.a_hi + o, h[0], h[1], h[2], h[3]);
        st16(c.a_lo + o, l[0], l[1], l[2], l[3]);
    });
}

// D0 = A_hi Bhi^T + A_hi Blo^T + A_lo Bhi^T, D1 = A_hi Bdl^T; returns false
// when the completion wait ran out. Called by all threads of the CTA after
// write_row.
template<int V>
__device__ __forceinline__ bool product(ctx& c)
{
    using S = shape<V>;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        fence_after();
        constexpr uint32_t id = idesc<V>();
#pragma unroll
        for (int ks = 0; ks < S::K / 8; ks++) {
            const uint32_t o = (uint32_t) ks * 256u;
            mma_tf32(c.tmem, desc<V>(c.a_hi + o), desc<V>(c.b_hi + o), id, ks > 0 ? 1u : 0u);
            mma_tf32(c.tmem, desc<V>(c.a_hi + o), desc<V>(c.b_lo + o), id, 1u);
            mma_tf32(c.tmem, desc<V>(c.a_lo + o), desc<V>(c.b_hi + o), id, 1u);
            mma_tf32(c.tmem + D1_COL, desc<V>(c.a_hi + o), desc<V>(c.b_dl + o), id, ks > 0 ? 1u : 0u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(c.mbar)
                     : "memory");
    }
    const bool ok = mbar_wait(c.mbar, c.phase, c.wait_limit);
    c.phase ^= 1u;
    fence_after();
    // the same answer in every thread, so that a time-out ends the tile in
    // all of them
    return __syncthreads_and(ok) != 0;
}

// Row threadIdx.x of D0 and D1, 16 columns at a time: f(i, D0[i], D1[i])
// for i < V (i a compile-time constant).
template<int V, class F>
__device__ __forceinline__ void consume_row(const ctx& c, F&& f)
{
    const uint32_t lane = (uint32_t) ((threadIdx.x >> 5) * 32) << 16;
    static_for<0, (V + 15) / 16>([&](auto BI) {
        constexpr int b = decltype(BI)::value;
        float v[16], w[16];
        tmem_ld16(c.tmem + lane + (uint32_t) (b * 16), v);
        tmem_ld16(c.tmem + lane + D1_COL + (uint32_t) (b * 16), w);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        static_for<0, 16>([&](auto QI) {
            constexpr int q = decltype(QI)::value;
            if constexpr (b * 16 + q < V) f(std::integral_constant<int, b * 16 + q>{}, v[q], w[q]);
        });
    });
}

// Per-material values the tensor-core update reads besides Bd (k, g,
// theta dt, p0): the FDTD head of the material block followed by its k, g
// and theta dt, staged in shared memory.
template<int V>
struct coef_small {
    static constexpr int len = pre::FDTD_END + 2 * V + (V / 2 > 0 ? V / 2 : 1);
    const float* base;
    __device__ __forceinline__ float k(int i) const { return base[pre::FDTD_END + i]; }
    __device__ __forceinline__ float g(int i) const { return base[pre::FDTD_END + V + i]; }
    __device__ __forceinline__ float th(int q) const { return base[pre::FDTD_END + 2 * V + q]; }
    __device__ __forceinline__ float p0() const { return base[5]; }
    // index in the material block (layout of make_cvr_layout) of entry i
    __device__ __forceinline__ static int source(int i)
    {
        return i < pre::FDTD_END ? i : pre::FDTD_END + 2 * V * V + (i - pre::FDTD_END);
    }
};

// Rotation of the planes of v = uh + ul by theta_k dt e (the first part of
// cvr_update_df).
template<int V, class CF>
__device__ __forceinline__ void rotate_df(float (&uh)[V], float (&ul)[V], float e, const CF& cf)
{
    static_for<0, V / 2>([&](auto KI) {
        constexpr int k = decltype(KI)::value;
        float sn, s2;
        rot_coeffs<float>(cf.th(k) * e, sn, s2);
        const float a = uh[2 * k], b = uh[2 * k + 1];
        const float da = -fmaf(s2, a, sn * b);
        const float db = fmaf(sn, a, -s2 * b);
        df_acc(uh[2 * k], ul[2 * k], da, 0.0f);
        df_acc(uh[2 * k + 1], ul[2 * k + 1], db, 0.0f);
    });
}

// The FP32 coherence-vector step of cvr_update_df with its matrix product
// on the tensor cores. The product reads its own copy of the vector
// (shared memory), so the registers are updated in place. All threads of
// the CTA call it (threads without a point pass zeros and discard the
// result).
template<int V, class CF>
__device__ __forceinline__ bool cvr_update_df_tc(
    ctx& c, float (&uh)[V], float (&ul)[V], float e, float& pout, const CF& cf)
{
    rotate_df<V>(uh, ul, e, cf);
    write_row<V>(c, uh);
    if (!product<V>(c)) return false;
    float pp = cf.p0();
    consume_row<V>(c, [&](auto I, float d, float dl) {
        constexpr int i = decltype(I)::value;
        df_acc(uh[i], ul[i], cf.k(i) + d, dl);
        df_renorm(uh[i], ul[i]);
        pp = fmaf(cf.g(i), uh[i], fmaf(cf.g(i), ul[i], pp));
    });
    pout = pp;
    fence_before();   // the reads of D above precede the next product's MMAs
    return true;
}

// The same step on the CUDA cores with the point's own coefficients
// (mixed-material tiles of the tensor-core kernel): the vector goes to this
// thread's row of shared memory so that the product can update the
// registers in place (the kernel's register budget has room for one
// vector of hi and lo words, not two).
template<int V, class CF>
__device__ __forceinline__ void cvr_update_df_row(
    float* row, float (&uh)[V], float (&ul)[V], float e, float& pout, const CF& cf)
{
    rotate_df<V>(uh, ul, e, cf);
    static_for<0, V>([&](auto J) {
        constexpr int j = decltype(J)::value;
        row[j] = uh[j];
    });
    float pp = cf.p0();
    static_for<0, V>([&](auto I) {
        constexpr int i = decltype(I)::value;
        float s = cf.k(i), sl = 0.0f;
        for (int j = 0; j < V; j++) {
            const float x = row[j];
            s = fmaf(cf.Bd(i, j), x, s);
            sl = fmaf(cf.Bdl(i, j), x, sl);
        }
        df_acc(uh[i], ul[i], s, sl);
        df_renorm(uh[i], ul[i]);
        pp = fmaf(cf.g(i), uh[i], fmaf(cf.g(i), ul[i], pp));
    });
    pout = pp;
}

}  // namespace tc
}  // namespace mbg
