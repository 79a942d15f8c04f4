// packed.cuh -- Blackwell packed-FP32 helpers: two FP32 lanes per 64-bit register pair in one
// `fma/mul/add/sub.rn.f32x2` instruction (sm_100 and later).
#pragma once
#include <cuda_runtime.h>

namespace mb {

typedef unsigned long long u64;
__device__ __forceinline__ u64 pk(float2 a) { return *reinterpret_cast<u64*>(&a); }
__device__ __forceinline__ float2 upk(u64 a) { return *reinterpret_cast<float2*>(&a); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    u64 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)), "l"(pk(c)));
    return upk(d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    u64 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    u64 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    u64 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk(a)), "l"(pk(b)));
    return upk(d);
}
__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }

}  // namespace mb
