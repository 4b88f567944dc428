// Device helpers shared by the surrogate's kernels (fno.cu, fno_layer.cu):
// inline-PTX wrappers for tcgen05 (MMA, commit, TMEM loads), mbarriers,
// asynchronous copies and shared-memory matrix descriptors, the GELU, and
// the host-side error plumbing of include/mbsolve_fno.h.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>

#include "../../include/mbsolve_fno.h"
#include "../../include/mbsolve_gb300.h"
#include "f32x2.cuh"

namespace mbg {
void set_last_error(const char* msg);

namespace fno {

constexpr uint32_t WAIT_LIMIT = 1u << 22;  // polls of a bounded mbarrier wait
constexpr uint32_t ST_WAIT = 1u;           // status bit: a wait ran out

// ------------------------------------------------------------ PTX wrappers

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t) __cvta_generic_to_shared(p);
}

// shared-memory matrix descriptor of a K-major operand without swizzle
// (layout type 0), version 1: 8-row x 16-byte core matrices, `lbo` bytes
// apart along K and `sbo` bytes apart along M/N (both multiples of 16)
__device__ __forceinline__ uint64_t smem_desc_nsw(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t) ((addr >> 4) & 0x3FFFu);
    d |= (uint64_t) ((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t) ((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t) 1u << 46;
    return d;
}

// instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// A and B BF16 (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bits 17-22,
// M >> 4 at bits 24-28
constexpr uint32_t idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t) (n >> 3) << 17) | ((uint32_t) (m >> 4) << 24);
}

// D (TMEM) = A B^T (+ D when acc != 0), issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "setp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n"
        "}\n" ::"r"(tmem),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}

// bounded wait for the completion of the phase with the given parity
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    for (uint32_t i = 0; i < WAIT_LIMIT; i++) {
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
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 16 bytes global -> shared, asynchronous, L2 only; src_bytes 0 fills zeros
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template<int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// bulk copies (TMA, no tensor map): 16-byte aligned addresses, sizes a
// multiple of 16. Global -> shared completes `bytes` of the mbarrier's
// expected transaction count.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(mbar)
        : "memory");
}
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template<int N>
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory"); }
template<int N>
__device__ __forceinline__ void bulk_wait() { asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory"); }

__device__ __forceinline__ void mbar_arrive(uint32_t mbar)
{
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(mbar) : "memory");
}
// one arrival that also raises the phase's expected transaction bytes
__device__ __forceinline__ void mbar_arrive_tx(uint32_t mbar, uint32_t bytes)
{
    asm volatile("{\n.reg .b64 st;\nmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}" ::"r"(mbar),
                 "r"(bytes)
                 : "memory");
}
// one poll of the phase with the given parity
__device__ __forceinline__ bool mbar_test(uint32_t mbar, uint32_t parity)
{
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
    return ok != 0;
}

// one non-blocking test of the phase with the given parity (try_wait may
// suspend the thread for a while; this never does)
__device__ __forceinline__ bool mbar_peek(uint32_t mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n"
        ".reg .pred P;\n"
        "mbarrier.test_wait.parity.shared::cta.b64 P, [%1], %2;\n"
        "selp.b32 %0, 1, 0, P;\n"
        "}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

// barrier among the `n` threads that name it (id 1..15; id 0 is __syncthreads)
__device__ __forceinline__ void named_sync(uint32_t id, uint32_t n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// ------------------------------------------------------------ arithmetic

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// GELU(x) = 0.5 x (1 + erf(x / sqrt 2)) with erf by Abramowitz and Stegun,
// Handbook of Mathematical Functions (1964), 7.1.26 (|error| <= 1.5e-7):
// erfc z = t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) exp(-z^2),
// t = 1 / (1 + p z), z = |x| / sqrt 2. Branch-free; x < 0 takes
// 0.5 x erfc z directly (no cancellation), x >= 0 takes x - 0.5 x erfc z.
__device__ __forceinline__ float gelu(float x)
{
    const float z = fabsf(x) * 0.70710678118654752f;
    const float t = __fdividef(1.0f, fmaf(0.3275911f, z, 1.0f));
    float q = fmaf(t, 1.061405429f, -1.453152027f);
    q = fmaf(t, q, 1.421413741f);
    q = fmaf(t, q, -0.284496736f);
    q = fmaf(t, q, 0.254829592f);
    const float h = 0.5f * x * (t * q * __expf(-z * z));
    return x < 0.0f ? h : x - h;
}

// gelu() on two values: lane by lane the same operations, the multiplies
// and fused multiply-adds as packed FP32 pairs (f32x2.cuh), the reciprocal
// and the exponential per lane
__device__ __forceinline__ float2 gelu2(float2 x)
{
    using namespace f2;
    const float2 z = mul(make_float2(fabsf(x.x), fabsf(x.y)), bc(0.70710678118654752f));
    const float2 d = fma(bc(0.3275911f), z, bc(1.0f));
    const float2 t = make_float2(__fdividef(1.0f, d.x), __fdividef(1.0f, d.y));
    float2 q = fma(t, bc(1.061405429f), bc(-1.453152027f));
    q = fma(t, q, bc(1.421413741f));
    q = fma(t, q, bc(-0.284496736f));
    q = fma(t, q, bc(0.254829592f));
    const float2 zz = mul(z, z);
    const float2 e = make_float2(__expf(-zz.x), __expf(-zz.y));
    const float2 h = mul(mul(bc(0.5f), x), mul(mul(t, q), e));
    const float2 xh = sub(x, h);
    return make_float2(x.x < 0.0f ? h.x : xh.x, x.y < 0.0f ? h.y : xh.y);
}

__device__ __forceinline__ float gelu_grad(float x)
{
    const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
    return cdf + x * pdf;
}

// ------------------------------------------------------------ host side

uint32_t* status_ptr();              // the device status word (per device)
void check_launch(const char* what);
void require(bool c, const char* msg);
int blocks_for(int64_t n, int per = 256);

template<typename F>
int guard(F&& f)
{
    try {
        f();
        return MBG_OK;
    } catch (const std::invalid_argument& e) {
        set_last_error(e.what());
        return MBG_ERR_INVALID_ARGUMENT;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return MBG_ERR_CUDA;
    }
}

}  // namespace fno
}  // namespace mbg
