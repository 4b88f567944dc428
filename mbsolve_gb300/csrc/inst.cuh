// Explicit instantiation helpers: each k_*.cu file registers the launch
// shapes (points per thread C, threads per CTA NT) it compiles.
#pragma once

#include "engine.hpp"
#include "tile_kernel.cuh"

namespace mbg {

template<typename T, int ALGO, int LEV, int C, int NT>
void launch_step(const kparams<T>& p, unsigned grid, size_t smem, cudaStream_t s)
{
    // 4 and more levels: uniform tiles stage the padded copy (cvr_pad)
    if constexpr (ALGO == 1 && density_len<ALGO, LEV>::value >= 15) {
        const size_t pad = (size_t) cvr_pad<T, density_len<ALGO, LEV>::value>::len * sizeof(T);
        if (smem < pad) smem = pad;
    }
    step_kernel<T, ALGO, LEV, C, NT><<<grid, NT, smem, s>>>(p);
}

// 2-level FP32 with bulk-copy staging: room for the staged planes after the
// coefficients
template<int C, int NT>
void launch_step_bulk(const kparams<float>& p, unsigned grid, size_t smem, cudaStream_t s)
{
    const size_t need = ((smem + 127) & ~(size_t) 127) + 128 + bulk::bytes<3>(C * NT);
    static const cudaError_t attr =
        cudaFuncSetAttribute(step_kernel_bulk<C, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) need);
    (void) attr;
    step_kernel_bulk<C, NT><<<grid, NT, need, s>>>(p);
}

// FP32 coherence-vector kernels for 4-6 levels with the density products
// of uniform tiles on the tensor cores (128 threads, one point each).
template<int LEV>
void launch_step_tc(const kparams<float>& p, unsigned grid, size_t smem, cudaStream_t s)
{
    constexpr int D = LEV * LEV - 1;
    const size_t need = ((tc::coef_small<D>::len * sizeof(float) + 127) & ~(size_t) 127) + 128 +
        tc::shape<D>::BYTES;
    if (smem < need) smem = need;
    static const cudaError_t attr = cudaFuncSetAttribute(
        step_kernel_tc<LEV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) need);
    (void) attr;
    step_kernel_tc<LEV><<<grid, tc::M, smem, s>>>(p);
}

// Persistent kernels: as many CTAs as fit the SMs at once. They need not
// all be resident: a CTA fetches work items only while it runs, and waits
// only for items fetched before its own (see step_kernel_persist), so the
// earliest unfinished item always has its dependencies done. An ordinary
// launch therefore suffices; the runtime's cooperative-launch limit
// allowed one tensor-core CTA per SM where three fit (measured).
// CTAs of `kernel` resident per SM from its registers and shared memory
// and the device's limits, and the runtime occupancy query's answer
template<typename K>
void persist_grid(K kernel, int threads, size_t smem, unsigned& by_limits, unsigned& by_query)
{
    int dev = 0, sms = 0, regs_sm = 0, smem_sm = 0, thr_sm = 0, per_sm = 0;
    MBG_CK(cudaGetDevice(&dev));
    MBG_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MBG_CK(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
    MBG_CK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    MBG_CK(cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
    MBG_CK(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int) cudaSharedmemCarveoutMaxShared));
    cudaFuncAttributes fa;
    MBG_CK(cudaFuncGetAttributes(&fa, kernel));
    const int warps = (threads + 31) / 32;
    const int regs_cta = ((fa.numRegs * 32 + 255) / 256) * 256 * warps;
    const size_t smem_cta = fa.sharedSizeBytes + smem + 1024;  // 1 KB reserved per CTA
    int n = std::min(regs_sm / std::max(1, regs_cta), thr_sm / (warps * 32));
    n = std::min<int>(n, (int) (smem_sm / smem_cta));
    n = std::min(n, 32);
    MBG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
    if (std::max(n, per_sm) < 1) throw std::runtime_error("CUDA: the persistent kernel does not fit an SM");
    by_limits = (unsigned) (std::max(n, 1) * sms);
    by_query = (unsigned) (std::max(per_sm, 1) * sms);
}

// the launch: one CTA per resident slot (device limits), at most one per
// work item
template<typename K, typename... A>
unsigned persist_launch(K kernel, int threads, size_t smem, unsigned items, cudaStream_t s, const A&... args)
{
    unsigned a = 0, b = 0;
    persist_grid(kernel, threads, smem, a, b);
    const unsigned slots = std::max(a, b);
    if (items == 0) return slots;
    kernel<<<std::min(slots, items), threads, smem, s>>>(args...);
    MBG_CK(cudaGetLastError());
    return std::min(slots, items);
}

template<typename T, int ALGO, int LEV, int C, int NT>
unsigned launch_persist(const kparams<T>& p, const persist_params& q, size_t smem, cudaStream_t s)
{
    if constexpr (ALGO == 1 && density_len<ALGO, LEV>::value >= 15) {
        const size_t pad = (size_t) cvr_pad<T, density_len<ALGO, LEV>::value>::len * sizeof(T);
        if (smem < pad) smem = pad;
    }
    return persist_launch(step_kernel_persist<T, ALGO, LEV, C, NT>, NT, smem, q.levels * q.n_tiles, s, p, q);
}

template<int LEV>
unsigned launch_persist_tc(const kparams<float>& p, const persist_params& q, size_t smem, cudaStream_t s)
{
    constexpr int D = LEV * LEV - 1;
    const size_t need = ((tc::coef_small<D>::len * sizeof(float) + 127) & ~(size_t) 127) + 128 +
        tc::shape<D>::BYTES;
    if (smem < need) smem = need;
    auto k = step_kernel_persist_tc<LEV>;
    static const cudaError_t attr = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) need);
    (void) attr;
    return persist_launch(k, tc::M, smem, q.levels * q.n_tiles, s, p, q);
}

}  // namespace mbg

// with a persistent kernel as well
#define MBG_REG_CVR_TC_P(LEV)                                                      \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<float>( \
        ::mbg::ALGO_CVR, LEV, 1, ::mbg::tc::M, &::mbg::launch_step_tc<LEV>, 0,      \
        &::mbg::launch_persist_tc<LEV>);
// only the persistent kernel of a shape registered elsewhere (a
// translation unit of its own, so that no kernel is compiled twice)
#define MBG_REG_CAY_PONLY(T, LEV, C, NT)                                       \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<T>( \
        ::mbg::ALGO_CAYLEY, LEV, C, NT, nullptr, 0, &::mbg::launch_persist<T, 2, LEV, C, NT>);
#define MBG_REG_CVR_P(T, LEV, C, NT)                                           \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<T>( \
        ::mbg::ALGO_CVR, LEV, C, NT, &::mbg::launch_step<T, 1, LEV, C, NT>, 0,  \
        &::mbg::launch_persist<T, 1, LEV, C, NT>);

#define MBG_REG_CVR_TC(LEV)                                                       \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<float>( \
        ::mbg::ALGO_CVR, LEV, 1, ::mbg::tc::M, &::mbg::launch_step_tc<LEV>);

#define MBG_REG_CVR2_BULK(C, NT)                                                  \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<float>( \
        ::mbg::ALGO_CVR, 2, C, NT, &::mbg::launch_step_bulk<C, NT>, 1);

#define MBG_CAT2(a, b) a##b
#define MBG_CAT(a, b) MBG_CAT2(a, b)
#define MBG_REG_CVR(T, LEV, C, NT)                                            \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<T>( \
        ::mbg::ALGO_CVR, LEV, C, NT, &::mbg::launch_step<T, 1, LEV, C, NT>);
#define MBG_REG_NOOP(T, C, NT)                                                \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<T>( \
        ::mbg::ALGO_NOOP, 0, C, NT, &::mbg::launch_step<T, 0, 0, C, NT>);
#define MBG_REG_CAY(T, LEV, C, NT)                                            \
    static const bool MBG_CAT(mbg_reg_, __LINE__) = ::mbg::register_kernel<T>( \
        ::mbg::ALGO_CAYLEY, LEV, C, NT, &::mbg::launch_step<T, 2, LEV, C, NT>);
