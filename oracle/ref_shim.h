/*
 * ref_shim.h - force-included when the oracle recipe compiles the
 * reference's GPUGrossPitaevskii_BCC.cu (koodit/GrossPitaevskii).
 *
 * The reference includes a vendored CUDA-samples helper header that no longer
 * compiles against CUDA 13 (it reads cudaDeviceProp fields that were removed).
 * The recipe predefines that header's include guard (-DHELPER_CUDA_H) so the
 * vendored file contributes nothing, and this shim supplies the single macro the
 * reference uses from it, checkCudaErrors.  The reference's behaviour on a CUDA
 * error (print and exit) is kept.
 *
 * Test infrastructure only: used to build oracle/_ref/, never by the product.
 */
#pragma once
#include <cstdio>
#include <cstdlib>

#define checkCudaErrors(expr)                                                   \
    do {                                                                        \
        cudaError_t ref_shim_err_ = (expr);                                     \
        if (ref_shim_err_ != cudaSuccess) {                                     \
            std::fprintf(stderr, "CUDA error %d (%s) at %s:%d\n",               \
                         (int)ref_shim_err_, cudaGetErrorString(ref_shim_err_), \
                         __FILE__, __LINE__);                                   \
            std::exit(EXIT_FAILURE);                                            \
        }                                                                       \
    } while (0)
