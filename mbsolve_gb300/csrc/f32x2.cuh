// Packed FP32 pairs (Blackwell's two-lane fma/add/mul/sub.rn.f32x2): one
// instruction for two values, each lane rounded like the scalar operation.
#pragma once

#include <cuda_runtime.h>

namespace mbg {
namespace f2 {

__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 sub(float2 a, float2 b)
{
    float2 r;
    asm("{.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pd, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

}  // namespace f2
}  // namespace mbg
