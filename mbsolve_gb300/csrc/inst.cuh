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

}  // namespace mbg

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
