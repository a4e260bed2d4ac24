/* Stand-in for the CUDA samples' helper_math.h: the reference's arithmetic
 * on the TSDF -> mesh path uses its own float3_* / vector3_* functions
 * (cu_vector_functions.h), not the samples' operators, so nothing is needed
 * from it.  TEST INFRASTRUCTURE ONLY. */
#pragma once
