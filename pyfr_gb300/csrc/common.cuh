// Shared helpers for the pyfrb200 CUDA library.
//
// Data layout (identical to the reference CUDA backend, SoA size 32,
// pyfr/backends/base/types.py:58-75 and pyfr/backends/cuda/base.py:55-59):
// a field of io-shape (nrow, nvars, neles) is stored row-major with
// `ld` scalars per row; inside a row, elements are grouped in blocks of 32
// and the variables of one block are contiguous:
//     a[row*ld + (e/32)*32*nvars + v*32 + e%32]
// so a warp that reads one variable of 32 consecutive elements touches one
// contiguous 256-byte (FP64) segment.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#define B200_SOASZ 32

namespace b200 {

// Record an error message for b200_get_last_error(); returns the code.
int set_error(int code, const char *fmt, ...);
int check_cuda(cudaError_t err, const char *what);

__host__ __device__ __forceinline__ int64_t soa_off(int64_t e, int v, int nv) {
    return (e / B200_SOASZ) * B200_SOASZ * nv + v * B200_SOASZ + (e % B200_SOASZ);
}

// Gather-index load from an int32 or int64 view mapping.
__device__ __forceinline__ int64_t load_ix(const void *map, int ix64, int64_t i) {
    return ix64 ? __ldg(static_cast<const long long *>(map) + i)
                : (int64_t)__ldg(static_cast<const int *>(map) + i);
}

inline unsigned ceil_div(int64_t a, int64_t b) { return (unsigned)((a + b - 1) / b); }

}  // namespace b200

// Status codes of the C ABI
#define B200_OK 0
#define B200_ERR_CUDA 1
#define B200_ERR_ARG 2
#define B200_ERR_UNSUPPORTED 3
#define B200_ERR_STATE 4

#define B200_CHECK_LAUNCH(what)                                              \
    do {                                                                     \
        cudaError_t e_ = cudaGetLastError();                                 \
        if (e_ != cudaSuccess) return b200::check_cuda(e_, what);            \
    } while (0)
