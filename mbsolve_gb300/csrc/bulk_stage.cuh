// Bulk asynchronous (TMA) staging of a tile's state planes for the 2-level
// FP32 time-step kernels.
//
// At the start of a launch one thread copies the tile's input window of
// every plane (E, H, P, their low words, the coherence vector and its low
// words: 11 planes of NT*C floats) from global into shared memory with
// cp.async.bulk, completing on one mbarrier (expect_tx of the total bytes);
// every thread then takes its C consecutive cells of each plane with 16-byte
// shared loads. At the end every thread writes its cells back into the
// staged planes and, after an async-proxy fence and a barrier, one thread
// writes the tile's output range of every plane to global memory with
// cp.async.bulk (bulk group) and waits until they have read shared memory.
//
// Alignment: runs start on 8-cell boundaries, halos are multiples of 8 and
// the plane stride is a multiple of 8, so every copy starts on a 32-byte
// boundary; the output range is rounded up to 4 cells (16 bytes), which
// stays inside the run's padding to 8 cells (cells there hold zero state in
// every kernel). The input window may reach into the guards and neighbouring
// runs; those cells are masked to zero as in the register loads.
#pragma once

#include <cstdint>

#include "kernels.cuh"

namespace mbg {
namespace bulk {

constexpr uint32_t WAIT_LIMIT = 1u << 22;

template<typename T, int ALGO, int LEV, bool TC>
__device__ __host__ constexpr bool enabled()
{
    return sizeof(T) == 4 && ALGO == 1 && LEV == 2 && !TC;
}

// planes staged for a coherence-vector kernel with D density reals
template<int D>
__device__ __host__ constexpr int planes()
{
    return 5 + 2 * D;
}

// bytes of shared memory the staged planes of a tile of W cells need
template<int D>
__host__ __device__ constexpr size_t bytes(int W)
{
    return (size_t) planes<D>() * (size_t) W * sizeof(float);
}

template<int D>
__device__ __forceinline__ const float* plane_in(const kparams<float>& p, int k)
{
    switch (k) {
    case 0: return p.Ein;
    case 1: return p.Hin;
    case 2: return p.Pin;
    case 3: return p.Elin;
    case 4: return p.Hlin;
    default: return p.Din + (uint64_t) (k - 5) * p.plane;
    }
}

template<int D>
__device__ __forceinline__ float* plane_out(const kparams<float>& p, int k)
{
    switch (k) {
    case 0: return p.Eout;
    case 1: return p.Hout;
    case 2: return p.Pout;
    case 3: return p.Elout;
    case 4: return p.Hlout;
    default: return p.Dout + (uint64_t) (k - 5) * p.plane;
    }
}

// Copy the window [gt, gt + W) of every plane into shared memory at sdst;
// all threads call it, all return the same answer (false: the completion
// wait ran out).
template<int D, int W>
__device__ __forceinline__ bool load(const kparams<float>& p, uint64_t gt, uint32_t mbar, uint32_t sdst)
{
    constexpr uint32_t PB = (uint32_t) W * 4u;
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar),
                     "r"(PB * (uint32_t) planes<D>())
                     : "memory");
#pragma unroll 1
        for (int k = 0; k < planes<D>(); k++) {
            const float* src = plane_in<D>(p, k) + gt;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    sdst + (uint32_t) k * PB),
                "l"(src), "r"(PB), "r"(mbar)
                : "memory");
        }
    }
    __syncthreads();  // the barrier is initialised before anyone waits on it
    bool ok = false;
    const uint32_t limit = p.wait_limit ? p.wait_limit : WAIT_LIMIT;
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n"
            ".reg .pred P;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 P, [%1], 0;\n"
            "selp.b32 %0, 1, 0, P;\n"
            "}\n"
            : "=r"(done)
            : "r"(mbar)
            : "memory");
        if (done) {
            ok = true;
            break;
        }
    }
    return __syncthreads_and(ok) != 0;
}

// this thread's C cells of staged plane k (W cells per plane)
template<int C>
__device__ __forceinline__ void take(float (&r)[C], const float* mine, int k, int W)
{
    const float* s = mine + (size_t) k * W;
    if constexpr (C % 4 == 0) {
#pragma unroll
        for (int q = 0; q < C / 4; q++) {
            const float4 v = reinterpret_cast<const float4*>(s)[q];
            r[4 * q] = v.x;
            r[4 * q + 1] = v.y;
            r[4 * q + 2] = v.z;
            r[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < C; j++) r[j] = s[j];
    }
}

template<int C>
__device__ __forceinline__ void give(const float (&r)[C], float* mine, int k, int W)
{
    float* s = mine + (size_t) k * W;
    if constexpr (C % 4 == 0) {
#pragma unroll
        for (int q = 0; q < C / 4; q++)
            reinterpret_cast<float4*>(s)[q] = make_float4(r[4 * q], r[4 * q + 1], r[4 * q + 2], r[4 * q + 3]);
    } else {
#pragma unroll
        for (int j = 0; j < C; j++) s[j] = r[j];
    }
}

// Write cells [gout, gout + round4(len)) of every plane from shared memory
// at ssrc (the output range's first cell in staged plane 0).
template<int D, int W>
__device__ __forceinline__ void store(const kparams<float>& p, uint64_t gout, uint32_t len, uint32_t ssrc)
{
    constexpr uint32_t PB = (uint32_t) W * 4u;
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t nb = ((len + 3u) & ~3u) * 4u;
#pragma unroll 1
        for (int k = 0; k < planes<D>(); k++) {
            float* dst = plane_out<D>(p, k) + gout;
            asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                         "r"(ssrc + (uint32_t) k * PB), "r"(nb)
                         : "memory");
        }
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        // only until the copies have read shared memory: the CTA may then
        // exit while the writes drain (they complete with the grid)
        asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
    }
}

}  // namespace bulk
}  // namespace mbg
