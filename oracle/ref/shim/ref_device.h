/* Host stand-ins for the CUDA device built-ins used by the reference's
 * kernels, so that their source compiles with g++ and runs on the CPU.
 * TEST INFRASTRUCTURE ONLY: this is how oracle/ref compiles the reference's
 * own code into a checker of the oracle; nothing of the library uses it.
 *
 * A kernel runs one thread at a time: the harness sets threadIdx / blockIdx
 * / blockDim for each thread and calls the kernel body.  That is exact for
 * the kernels compiled here, whose threads never read what another thread
 * of their block wrote (the marching-cubes generator's __shared__ vertex list
 * is indexed by the thread's own id, and its __syncthreads() orders nothing
 * else), so __shared__ becomes a static and __syncthreads() nothing.
 *
 * Force-included before any reference header (g++ -include). */
#pragma once

#include <cuda_runtime.h> /* float3 / int3 / uint3 / dim3 and make_* (CUDA toolkit headers) */

#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>

/* CUDA's host_defines.h spells __forceinline__ as "inline + always_inline",
 * which g++ rejects after the reference's own "static inline"; the host
 * build does not need the forced inlining. */
#undef __forceinline__
#define __forceinline__
#undef __shared__
#define __shared__ static

/* the thread the harness is running */
extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;

inline void __syncthreads() {}

/* __float2int_rn: binary32 -> int32, rounded to nearest, ties to even,
 * saturated to the int32 range, NaN -> 0 (the PTX cvt.rni.s32.f32
 * semantics).  nearbyint rounds in the current mode, which is the default
 * to-nearest-even. */
inline int __float2int_rn(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT_MAX;
    if (f <= -2147483648.0f) return INT_MIN;
    return (int)std::nearbyint(f);
}

/* 1-D integer texture reference of the pre-CUDA-12 API (removed from the
 * toolkit headers): a bound texture is a plain table here. */
template <class T, int DIM = 1, int MODE = 0>
struct texture {
    const T *table = nullptr;
};
template <class T, int DIM, int MODE>
inline T tex1Dfetch(const texture<T, DIM, MODE> &t, int i) { return t.table[i]; }
