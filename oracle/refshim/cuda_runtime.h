/* Host shim standing in for <cuda_runtime.h> when the reference's kernel
 * headers (brasstower/kernel/*.cuh) are compiled with g++ as plain host code.
 *
 * Test infrastructure only: this overlay lets oracle/ref_driver.cpp compile
 * the reference's own __global__/__device__ function bodies unmodified, so
 * that their outputs can pin the C restatement in oracle/oracle.c.
 *
 * What it provides:
 *   - the CUDA vector types (float3, int3, ...) and make_* constructors from
 *     the toolkit's vector_types.h / vector_functions.h;
 *   - empty __global__/__device__/__host__/__constant__ qualifiers, and
 *     __shared__ as `static` (blocks run one at a time, so a function-local
 *     static is shared by the block's threads exactly like shared memory);
 *   - thread-local threadIdx/blockIdx/blockDim set by the launch emulation;
 *   - atomicAdd as an OpenMP atomic, __mul24 as a plain product,
 *     __syncthreads as an OpenMP barrier;
 *   - cudaMemcpyToSymbol as memcpy into the (now host) symbol.
 */
#pragma once

#include <math.h>
#include <string.h>
#include <stddef.h>
#include <algorithm>
#include <vector_types.h>
#include <vector_functions.h>

#undef __global__
#undef __device__
#undef __host__
#undef __constant__
#undef __shared__
#undef __forceinline__
#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__ static
#define __forceinline__ inline

typedef unsigned int uint;

extern thread_local uint3 threadIdx;
extern thread_local uint3 blockIdx;
extern thread_local dim3 blockDim;
extern thread_local dim3 gridDim;

static inline int __mul24(int a, int b) { return a * b; }

static inline float atomicAdd(float *addr, float v)
{
    float old;
#pragma omp atomic capture
    { old = *addr; *addr += v; }
    return old;
}

static inline int atomicAdd(int *addr, int v)
{
    int old;
#pragma omp atomic capture
    { old = *addr; *addr += v; }
    return old;
}

#define __syncthreads() _Pragma("omp barrier")

/* CUDA's device min/max overloads for float (the kernels call them unqualified);
 * the int versions come from the reference's helper_math.h host section. */
static inline float min(float a, float b) { return a < b ? a : b; }
static inline float max(float a, float b) { return a > b ? a : b; }
static inline unsigned int min(unsigned int a, unsigned int b) { return a < b ? a : b; }
static inline unsigned int max(unsigned int a, unsigned int b) { return a > b ? a : b; }

/* kernel/util.cuh:154-160 (the float3 atomic add the constraint kernels call)
 * is declared here because util.cuh itself holds <<<>>> launches that a host
 * compiler cannot parse; it is the same per-component atomic add. */
static inline void atomicAdd(float3 *arr, int index, const float3 val)
{
    atomicAdd(&arr[index].x, val.x);
    atomicAdd(&arr[index].y, val.y);
    atomicAdd(&arr[index].z, val.z);
}

/* cudaError_t / cudaSuccess come from the toolkit's driver_types.h. */
template <class T>
static inline cudaError_t cudaMemcpyToSymbol(T &symbol, const void *src, size_t n)
{
    memcpy((void *)&symbol, src, n);
    return cudaSuccess;
}
