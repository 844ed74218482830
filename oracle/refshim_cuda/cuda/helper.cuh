/* CUDA-build shim: stand-in for the reference's cuda/helper.cuh.  The kernel
 * headers use only its error-check macro (SetKernelRadius, kernel/fluid.cuh:11-27);
 * here a failed call is recorded, and the replay driver reports it. */
#pragma once
#include <cuda_runtime.h>
extern cudaError_t g_ref_cuda_first_error;
#define checkCudaErrors(val)                                                        \
    do {                                                                            \
        cudaError_t e_ = (val);                                                     \
        if (e_ != cudaSuccess && g_ref_cuda_first_error == cudaSuccess)             \
            g_ref_cuda_first_error = e_;                                            \
    } while (0)
