/* ref_shim.h -- lets the reference's CUDA kernel bodies compile as host C++ (oracle
 * cross-check only; see build_oracle.py).  Each kernel "thread" becomes one iteration
 * of an OpenMP loop in ref_driver.inc, which sets blockIdx.x to the flat thread index. */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#define __device__ inline
#define __global__
struct RefDim3 { long x, y, z; };
static thread_local RefDim3 blockIdx = {0, 0, 0};
static thread_local RefDim3 threadIdx = {0, 0, 0};
static const RefDim3 blockDim = {1, 1, 1};
