/*
 * Forced-include stand-in for the one macro of the CUDA samples' helper
 * header that the reference's CPU path uses (checkCudaErrors, in
 * Utils/mem_manager.inl).  oracle/ref_build.py defines that header's include
 * guard, so the reference's copy (written for CUDA 10 device properties that
 * CUDA 13 removed) is skipped.  TEST INFRASTRUCTURE ONLY.
 */
#ifndef GLSU_REF_HELPER_CUDA_SHIM_H
#define GLSU_REF_HELPER_CUDA_SHIM_H
#include <cstdio>
#include <cstdlib>
#include <cuda_runtime.h>
#define checkCudaErrors(call)                                                             \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) std::fprintf(stderr, "CUDA error %d at %s:%d\n", (int)e_, __FILE__, __LINE__); \
    } while (0)
#endif
