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

// FP32 <-> FP64 conversions on the integer pipes.  GB300's FP64 unit is
// narrow (about 2 operations per clock per SM) and executes the hardware
// conversions too, so a bandwidth-bound kernel that widens and narrows
// every element is FP64-bound.  These build the result from the IEEE 754
// binary32/binary64 encodings (1/8/23 and 1/11/52 bits, exponent biases 127
// and 1023) for the normal range and for signed zeros, which is where
// solution and RHS values live; subnormal, infinite and NaN operands take
// the hardware conversion.  Both are exact in the sense of IEEE 754: the
// widening is exact and the narrowing rounds to nearest, ties to even.
__device__ __forceinline__ double widen_f32(float f) {
    const uint32_t u = __float_as_uint(f);
    const uint32_t a = u & 0x7fffffffu;
    const uint64_t s = (uint64_t)(u & 0x80000000u) << 32;
    if (a - 0x00800000u < 0x7f000000u)  // biased exponent in [1, 254]
        return __longlong_as_double((long long)(s | ((uint64_t)a << 29) +
                                                         ((uint64_t)(1023 - 127) << 52)));
    if (a == 0) return __longlong_as_double((long long)s);
    return (double)f;
}

__device__ __forceinline__ float narrow_f64(double d) {
    const uint64_t u = (uint64_t)__double_as_longlong(d);
    const uint64_t a = u & 0x7fffffffffffffffull;
    const uint32_t s = (uint32_t)(u >> 32) & 0x80000000u;
    // Binary64 exponents 897..1150 are the binary32 normals 1..254
    if (a - (897ull << 52) < (254ull << 52)) {
        uint32_t r = (uint32_t)((a >> 29) - (896ull << 23));
        const uint32_t rem = (uint32_t)a & 0x1fffffffu;
        r += (uint32_t)(rem > 0x10000000u) | ((uint32_t)(rem == 0x10000000u) & r);
        return __uint_as_float(s | r);
    }
    if (a == 0) return __uint_as_float(s);
    return (float)d;
}

// 1/d in FP64 without an IEEE division.  A single-precision estimate
// (rcp.approx.ftz.f32, relative error about 2^-23) refined by two
// Newton-Raphson steps for f(r) = 1/r - d, r <- r + r*(1 - d*r), each of
// which squares the relative error (2^-46, then below the rounding of the
// last step): the result is within about one unit in the last place of
// the correctly rounded quotient, for 4 FP64 FMAs instead of the several
// FP64 operations, fix-up tests and slow path of an IEEE division on a GPU
// whose FP64 unit is narrow.  Operands with |d| outside [2^-100, 2^100]
// (where the estimate or its reciprocal could leave the binary32 normal
// range) take the IEEE division.
__device__ __forceinline__ double rcp_f64(double d) {
    const uint64_t a = (uint64_t)__double_as_longlong(d) & 0x7fffffffffffffffull;
    if (a - ((1023ull - 100) << 52) >= (200ull << 52)) return 1.0 / d;
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(narrow_f64(d)));
    double r = widen_f32(r0);
    r = fma(r, fma(-d, r, 1.0), r);
    r = fma(r, fma(-d, r, 1.0), r);
    return r;
}

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
