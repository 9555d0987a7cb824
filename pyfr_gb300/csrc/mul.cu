// Operator apply (the `mul` kernel of the backend API):
//     out[m, n] = alpha * sum_k A[m, k] * B[k, n] + beta * out[m, n]
// A is a small constant operator matrix, B and out are row-major with
// leading dimensions ldb/ldc and `ncol` active columns (nvars * padded
// neles for the AoSoA fields).  This replaces the GiMMiK and cuBLASLt
// providers of the reference (pyfr/backends/cuda/gimmik.py:23-121,
// pyfr/backends/cuda/cublaslt.py:169-280) with one sparsity-aware kernel.
//
// Each CTA stages a k x 64 column tile of B into shared memory with
// asynchronous 16-byte copies (cp.async: every copy of the tile is in
// flight at once, so staging costs one memory latency rather than one per
// row; with large K the tile limits residency to a few CTAs per SM, which
// then cannot hide a row-by-row staging behind each other's FMAs), or with
// coalesced loads when B is not 16-byte aligned; every warp then produces
// whole rows of the output tile,
// walking the nonzeros of A (CSR, read through the read-only cache and
// broadcast across the warp).  Structural zeros of A cost nothing, so the
// sparse tensor-product operators run at their nonzero count.
#include <stdlib.h>
#include <string.h>
#include <vector>

#include "common.cuh"
#include "../../include/pyfrb200.h"

namespace {

constexpr int MUL_NCOL = 64;     // columns per CTA
constexpr int MUL_WARPS = 8;     // warps per CTA

struct MulHandle {
    int m, k, nnz;
    int *rowptr;     // device, m + 1
    int *colidx;     // device, nnz
    double *val64;   // device, nnz
    float *val32;    // device, nnz
};

template <typename T>
__device__ __forceinline__ const T *vals(const MulHandle &h);
template <>
__device__ __forceinline__ const double *vals<double>(const MulHandle &h) { return h.val64; }
template <>
__device__ __forceinline__ const float *vals<float>(const MulHandle &h) { return h.val32; }

// Epilogue modes: FP64 arithmetic is the scarce resource on this GPU, so
// the common cases alpha = 1 with beta = 0 or beta = 1 issue no FP64 work
// beyond the FMAs of the product (beta = 1 accumulates onto the loaded C).
enum { EPI_SET = 0, EPI_ADD = 1, EPI_GENERAL = 2, EPI_SCALE = 3 };

// 16-byte global -> shared copy; bytes < 16 reads that many and zero-fills
// the rest
__device__ __forceinline__ void cp_async16(void *dst, const void *src, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16, %2;"
                 :: "r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src), "r"(bytes)
                 : "memory");
}

template <typename T, int EPI>
__global__ void __launch_bounds__(MUL_WARPS * 32)
mul_csr_kernel(MulHandle h, const T *__restrict__ b, int64_t ldb, T *__restrict__ c,
               int64_t ldc, int64_t ncol, T alpha, T beta, int vec) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *bs = reinterpret_cast<T *>(smem_raw);   // [k][MUL_NCOL]

    const int64_t col0 = (int64_t)blockIdx.x * MUL_NCOL;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    // Stage the B tile (zero-filled beyond ncol)
    if (vec) {
        constexpr int VEC = 16 / sizeof(T), NV = MUL_NCOL / VEC;
        for (int idx = threadIdx.x; idx < h.k * NV; idx += blockDim.x) {
            const int r = idx / NV, cv = (idx % NV) * VEC;
            const int64_t col = col0 + cv;
            const int64_t rem = ncol - col;
            const int bytes = rem >= VEC ? 16 : (rem > 0 ? (int)rem * (int)sizeof(T) : 0);
            // (with nothing to read the source is any valid address)
            cp_async16(bs + r * MUL_NCOL + cv, bytes ? b + r * ldb + col : b, bytes);
        }
        asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
    } else {
        for (int idx = threadIdx.x; idx < h.k * MUL_NCOL; idx += blockDim.x) {
            int r = idx / MUL_NCOL, cc = idx % MUL_NCOL;
            int64_t col = col0 + cc;
            bs[idx] = (col < ncol) ? b[r * ldb + col] : T(0);
        }
    }
    __syncthreads();

    const T *__restrict__ av = vals<T>(h);
    const int64_t ca = col0 + lane, cb = col0 + lane + 32;
    const bool oka = ca < ncol, okb = cb < ncol;

    for (int row = warp; row < h.m; row += MUL_WARPS) {
        T *crow = c + row * ldc;
        T acc0 = T(0), acc1 = T(0);
        if (EPI == EPI_ADD) {
            if (oka) acc0 = crow[ca];
            if (okb) acc1 = crow[cb];
        }
        const int p0 = __ldg(h.rowptr + row), p1 = __ldg(h.rowptr + row + 1);
        for (int p = p0; p < p1; p++) {
            const T a = __ldg(av + p);
            const int kk = __ldg(h.colidx + p);
            acc0 = fma(a, bs[kk * MUL_NCOL + lane], acc0);
            acc1 = fma(a, bs[kk * MUL_NCOL + lane + 32], acc1);
        }

        if (EPI == EPI_GENERAL) {
            if (oka) acc0 = alpha * acc0 + beta * crow[ca];
            if (okb) acc1 = alpha * acc1 + beta * crow[cb];
        } else if (EPI == EPI_SCALE) {
            acc0 *= alpha;
            acc1 *= alpha;
        }
        if (oka) crow[ca] = acc0;
        if (okb) crow[cb] = acc1;
    }
}

template <typename T>
int launch_mul(const MulHandle *h, const T *b, int64_t ldb, T *c, int64_t ldc, int64_t ncol,
               T alpha, T beta, cudaStream_t s) {
    if (!h) return b200::set_error(B200_ERR_ARG, "mul: null handle");
    if (ncol <= 0) return B200_OK;
    if (ldb < ncol || ldc < ncol)
        return b200::set_error(B200_ERR_ARG, "mul: leading dimension smaller than ncol");
    size_t smem = (size_t)h->k * MUL_NCOL * sizeof(T);
    if (smem > 227 * 1024)
        return b200::set_error(B200_ERR_UNSUPPORTED, "mul: k=%d too large for the tile", h->k);
    unsigned grid = b200::ceil_div(ncol, MUL_NCOL);
    // 16-byte copies need a 16-byte aligned base and row stride
    const int vec = !((uintptr_t)b & 15) && !((ldb * (int64_t)sizeof(T)) & 15);
    if (alpha == T(1) && beta == T(0))
        mul_csr_kernel<T, EPI_SET><<<grid, MUL_WARPS * 32, smem, s>>>(*h, b, ldb, c, ldc, ncol, alpha, beta, vec);
    else if (alpha == T(1) && beta == T(1))
        mul_csr_kernel<T, EPI_ADD><<<grid, MUL_WARPS * 32, smem, s>>>(*h, b, ldb, c, ldc, ncol, alpha, beta, vec);
    else if (beta == T(0))
        mul_csr_kernel<T, EPI_SCALE><<<grid, MUL_WARPS * 32, smem, s>>>(*h, b, ldb, c, ldc, ncol, alpha, beta, vec);
    else
        mul_csr_kernel<T, EPI_GENERAL><<<grid, MUL_WARPS * 32, smem, s>>>(*h, b, ldb, c, ldc, ncol, alpha, beta, vec);
    B200_CHECK_LAUNCH("mul_csr_kernel");
    return B200_OK;
}

// Opt every instantiation in to the largest tile.  Called from
// b200_mul_create, which never runs inside a stream capture: changing a
// function attribute while a capture is open invalidates the capture.
template <typename T>
int opt_in_smem() {
    void (*fns[4])(MulHandle, const T *, int64_t, T *, int64_t, int64_t, T, T, int) = {
        mul_csr_kernel<T, EPI_SET>, mul_csr_kernel<T, EPI_ADD>,
        mul_csr_kernel<T, EPI_GENERAL>, mul_csr_kernel<T, EPI_SCALE>};
    for (auto fn : fns) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             227 * 1024);
        if (e != cudaSuccess) return b200::check_cuda(e, "mul: smem attribute");
    }
    return B200_OK;
}

}  // namespace

extern "C" {

int b200_mul_create(const double *a, int m, int k, void **handle) {
    if (!a || !handle || m <= 0 || k <= 0)
        return b200::set_error(B200_ERR_ARG, "mul_create: bad arguments");
    int orc = opt_in_smem<double>();
    if (!orc) orc = opt_in_smem<float>();
    if (orc) return orc;

    std::vector<int> rowptr(m + 1, 0), colidx;
    std::vector<double> v64;
    std::vector<float> v32;
    for (int i = 0; i < m; i++) {
        for (int j = 0; j < k; j++) {
            double x = a[(size_t)i * k + j];
            if (x != 0.0) {
                colidx.push_back(j);
                v64.push_back(x);
                v32.push_back((float)x);
            }
        }
        rowptr[i + 1] = (int)colidx.size();
    }

    MulHandle *h = (MulHandle *)calloc(1, sizeof(MulHandle));
    if (!h) return b200::set_error(B200_ERR_STATE, "mul_create: out of host memory");
    h->m = m;
    h->k = k;
    h->nnz = (int)colidx.size();
    size_t nz = colidx.size() ? colidx.size() : 1;
    int rc = b200::check_cuda(cudaMalloc(&h->rowptr, sizeof(int) * (m + 1)), "mul_create");
    if (!rc) rc = b200::check_cuda(cudaMalloc(&h->colidx, sizeof(int) * nz), "mul_create");
    if (!rc) rc = b200::check_cuda(cudaMalloc(&h->val64, sizeof(double) * nz), "mul_create");
    if (!rc) rc = b200::check_cuda(cudaMalloc(&h->val32, sizeof(float) * nz), "mul_create");
    if (!rc) rc = b200::check_cuda(cudaMemcpy(h->rowptr, rowptr.data(), sizeof(int) * (m + 1),
                                              cudaMemcpyHostToDevice), "mul_create");
    if (!rc && h->nnz) {
        rc = b200::check_cuda(cudaMemcpy(h->colidx, colidx.data(), sizeof(int) * h->nnz,
                                         cudaMemcpyHostToDevice), "mul_create");
        if (!rc) rc = b200::check_cuda(cudaMemcpy(h->val64, v64.data(), sizeof(double) * h->nnz,
                                                  cudaMemcpyHostToDevice), "mul_create");
        if (!rc) rc = b200::check_cuda(cudaMemcpy(h->val32, v32.data(), sizeof(float) * h->nnz,
                                                  cudaMemcpyHostToDevice), "mul_create");
    }
    if (rc) {
        cudaFree(h->rowptr); cudaFree(h->colidx); cudaFree(h->val64); cudaFree(h->val32);
        free(h);
        return rc;
    }
    *handle = h;
    return B200_OK;
}

int b200_mul_nnz(void *handle, int *nnz) {
    if (!handle || !nnz) return b200::set_error(B200_ERR_ARG, "mul_nnz: bad arguments");
    *nnz = ((MulHandle *)handle)->nnz;
    return B200_OK;
}

int b200_mul_destroy(void *handle) {
    if (!handle) return B200_OK;
    MulHandle *h = (MulHandle *)handle;
    cudaFree(h->rowptr); cudaFree(h->colidx); cudaFree(h->val64); cudaFree(h->val32);
    free(h);
    return B200_OK;
}

int b200_mul_f64(void *handle, const double *b, int64_t ldb, double *c, int64_t ldc,
                 int64_t ncol, double alpha, double beta, void *stream) {
    return launch_mul<double>((const MulHandle *)handle, b, ldb, c, ldc, ncol, alpha, beta,
                              (cudaStream_t)stream);
}

int b200_mul_f32(void *handle, const float *b, int64_t ldb, float *c, int64_t ldc,
                 int64_t ncol, float alpha, float beta, void *stream) {
    return launch_mul<float>((const MulHandle *)handle, b, ldb, c, ldc, ncol, alpha, beta,
                             (cudaStream_t)stream);
}

}  // extern "C"
