// common.cuh -- shared device helpers for the mesh-BEM sm_103a kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

#include "../../include/mesh_bem_gb300.h"

namespace mb {

constexpr double kPi = 3.14159265358979323846;
constexpr double kInv4Pi = 0.0795774715459476678844;  // 1 / (4 pi)
constexpr double kInv2Pi = 0.159154943091895335769;   // 1 / (2 pi)

// Records a message for mb_last_error(); returns `code`.
int set_error(int code, const char* fmt, ...);
// Checks cudaGetLastError() after a launch; returns MB_OK or MB_ERR_CUDA.
int check_launch(const char* what);

template <typename T>
struct V3 {
    T x, y, z;
};

template <typename T>
__device__ __forceinline__ V3<T> v3(T x, T y, T z) {
    return V3<T>{x, y, z};
}
template <typename T>
__device__ __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) {
    return V3<T>{a.x - b.x, a.y - b.y, a.z - b.z};
}
template <typename T>
__device__ __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) {
    return V3<T>{a.x + b.x, a.y + b.y, a.z + b.z};
}
template <typename T>
__device__ __forceinline__ V3<T> operator*(T s, V3<T> a) {
    return V3<T>{s * a.x, s * a.y, s * a.z};
}
template <typename T>
__device__ __forceinline__ T dot(V3<T> a, V3<T> b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <typename T>
__device__ __forceinline__ V3<T> cross(V3<T> a, V3<T> b) {
    return V3<T>{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <typename T>
__device__ __forceinline__ V3<T> load3(const T* p, int64_t i) {
    return V3<T>{__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2)};
}

// Reciprocal square root: MUFU approximation in float, correctly rounded path in double.
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float sqrt_t(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_t(double x) { return sqrt(x); }

// sin/cos of an angle given in turns-scaled form.  `turns` = angle / (2 pi).
// float: reduce to [-1/2, 1/2] turn (exact: t - rint(t)), then the SFU approximation on
// an angle in [-pi, pi], where its absolute error bound holds.  double: libdevice sincospi.
__device__ __forceinline__ void sincos_turns(float turns, float* s, float* c) {
    float r = turns - rintf(turns);
    __sincosf(r * 6.28318530717958647692f, s, c);
}
__device__ __forceinline__ void sincos_turns(double turns, double* s, double* c) {
    sincospi(2.0 * turns, s, c);
}

template <typename T>
__device__ __forceinline__ T ld(const T* p) {
    return __ldg(p);
}

}  // namespace mb
