// Pre-included when the LBVH/GJK prototypes (sandbox/testLBVH.cu,
// sandbox/testGJK.cu) are compiled for pinning the oracle: the unary minus on
// float3 that testGJK.cu:279 applies and the sandbox's helper_math.hpp does
// not declare (component-wise negation).  Test infrastructure only.
#pragma once
#include <vector_types.h>
#include <vector_functions.h>

inline __host__ __device__ float3 operator-(const float3& a) { return make_float3(-a.x, -a.y, -a.z); }
