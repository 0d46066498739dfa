/* Type stand-ins that let the reference's kernel sources compile without
 * its engine headers (which pull Eigen and OpenGL): the include guards of
 * src/engine/engine.hpp and src/engine/types.hpp are pre-defined on the
 * command line, and the few names the kernels use from them are declared
 * here (own declarations; their layouts follow types.hpp:33-43). */
#pragma once
#include <cuda_runtime.h>
namespace STARDUST {
using Scalar = float;
struct float9 {
    Scalar data[9];
    __forceinline__ __device__ Scalar& operator[](int i) { return data[i]; }
    __forceinline__ __device__ const Scalar& operator[](int i) const { return data[i]; }
};
}  // namespace STARDUST
