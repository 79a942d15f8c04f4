// spai_apply.cuh -- row-gather application of the sparse approximate inverse M (ELL rows
// of MB_SPAI_WIDTH (local column, complex64 value) pairs, a row's pattern ends at the first
// negative column).  Shared by the preconditioner builder and the preconditioned solver.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/mesh_bem_gb300.h"

namespace mb {

// (M v)_i with v complex128, accumulated in FP32 (the input of an FP32 product)
__device__ __forceinline__ float2 spai_row_f32(const int32_t* __restrict__ cols, const float2* __restrict__ vals,
                                               int64_t i, const double2* __restrict__ v) {
    float sr = 0.f, si = 0.f;
    for (int q = 0; q < MB_SPAI_WIDTH; ++q) {
        const int32_t c = __ldg(cols + i * MB_SPAI_WIDTH + q);
        if (c < 0) break;
        const float2 m = __ldg(vals + i * MB_SPAI_WIDTH + q);
        const double2 x = __ldg(v + c);
        const float xr = (float)x.x, xi = (float)x.y;
        sr = fmaf(m.x, xr, fmaf(-m.y, xi, sr));
        si = fmaf(m.x, xi, fmaf(m.y, xr, si));
    }
    return make_float2(sr, si);
}

// (M v)_i in FP64 (the correction of the FP64 iterate, and the FP64 product path)
__device__ __forceinline__ double2 spai_row_f64(const int32_t* __restrict__ cols, const float2* __restrict__ vals,
                                                int64_t i, const double2* __restrict__ v) {
    double sr = 0.0, si = 0.0;
    for (int q = 0; q < MB_SPAI_WIDTH; ++q) {
        const int32_t c = __ldg(cols + i * MB_SPAI_WIDTH + q);
        if (c < 0) break;
        const float2 m = __ldg(vals + i * MB_SPAI_WIDTH + q);
        const double2 x = __ldg(v + c);
        sr = fma((double)m.x, x.x, fma(-(double)m.y, x.y, sr));
        si = fma((double)m.x, x.y, fma((double)m.y, x.x, si));
    }
    return make_double2(sr, si);
}

}  // namespace mb
