// Exact tsdf unpacking without a division.
//
// The reference unpacks a stored tsdf as (float)tsdf / 32766
// (cu_kinect_fusion_v1.h:253-256), an IEEE-rounded division.  Division by
// this one constant is replaced by q = RN(a * r) with r = RN(1/32766),
// followed by one correction step e = a - q*32766 (exact with an FMA) and
// q' = RN(q + e*r) -- Markstein's correction ("Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. R&D 34(1), 1990).
// tests/test_unpack_exact.py checks that q' equals the IEEE quotient for all
// 65536 int16 inputs, so kernels using it stay bit-exact with the division.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define MCG_HD __host__ __device__ __forceinline__
#else
#define MCG_HD inline
#endif

MCG_HD float mcg_unpack_tsdf(int t) {
    const float c = 32766.0f;
    const float r = 1.0f / 32766.0f;  // correctly rounded at compile time
    const float a = (float)t;
    const float q = a * r;
    const float e = fmaf(-q, c, a);
    return fmaf(e, r, q);
}
