/*
 * Host stand-in for <cuda_runtime.h>, used ONLY to compile the reference's
 * unmodified tracing kernels (fastqslpy/cu/TraceBline*.cu) as host C++ so that
 * they can serve as the CPU oracle and the CPU baseline.  Test infrastructure:
 * nothing in the fastqsl_gb300 package links against it.
 *
 * It supplies what those files use from the CUDA runtime: the vector types
 * (float3, int3, dim3, ...), the make_* constructors, empty execution-space
 * qualifiers, per-thread blockIdx/threadIdx/blockDim/gridDim and the two
 * rounding intrinsics the kernels call (__float2int_rd, __int2float_rd).
 */
#ifndef QSL_REF_SHIM_CUDA_RUNTIME_H
#define QSL_REF_SHIM_CUDA_RUNTIME_H

#include <math.h>
#include <stdlib.h>
#include <vector_types.h>
#include <vector_functions.h>

#undef __global__
#undef __device__
#undef __host__
#undef __forceinline__
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

/* Launch coordinates of the "thread" currently executing a kernel body.  The
 * driver sets them before each call; one OpenMP thread runs one body. */
extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

/* Round toward -inf.  A NaN argument maps to 0, which is what the device
 * conversion instruction returns, so that a NaN position indexes the first
 * grid node instead of an arbitrary address; out-of-range values saturate as
 * they do on the device. */
static inline int __float2int_rd(float x)
{
    if (x != x) return 0;
    if (x >= 2147483647.0f) return 2147483647;
    if (x <= -2147483648.0f) return (-2147483647 - 1);
    return (int)floorf(x);
}
static inline float __int2float_rd(int x) { return (float)x; }

#endif
