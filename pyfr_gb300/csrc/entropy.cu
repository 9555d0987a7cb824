// Entropy filter (shock capturing) of the Euler and Navier-Stokes systems:
// the entry points, the tensor-product shapes (quadrilaterals of order 1-5,
// hexahedra of order 1-4) and the interface exchange.  The kernels are in
// entropy.cuh; the simplex shapes are instantiated in entropy_simplex.cu.
#include "entropy.cuh"

namespace {

#define EF_SHAPES(X)                                                               \
    X(2, 4) X(2, 9) X(2, 16) X(2, 25) X(2, 36) X(3, 8) X(3, 27) X(3, 64) X(3, 125)

template <typename T>
int entropyfilter(const b200_ef_t *p, int64_t neles, T *u, int64_t ldu, T *entmin, int64_t lde,
                  T *ef_filter, const T *vdm, int64_t ldv, const T *invvdm, int64_t ldi,
                  const T *m0, int64_t ldm, const T *mean_wts, int64_t ldw, const int *degs,
                  cudaStream_t st) {
    if (neles <= 0) return B200_OK;
    if (!p || !u || !entmin || !ef_filter || !vdm || !invvdm || !mean_wts || !degs ||
        (!p->fpts_in_upts && !m0))
        return b200::set_error(B200_ERR_ARG, "entropyfilter: null argument");
    if (p->order < 0 || p->order > EF_MAX_ORDER)
        return b200::set_error(B200_ERR_ARG, "entropyfilter: order out of range");
    const auto c = ef_consts<T>(*p);
#define X(nd, nu)                                                                  \
    if (p->ndims == nd && p->nupts == nu)                                          \
        return launch_filter<nd, nu, T>(p, c, neles, u, ldu, entmin, lde, ef_filter, vdm, \
                                        ldv, invvdm, ldi, m0, ldm, mean_wts, ldw, degs, st);
    EF_SHAPES(X)
#undef X
    return b200_ef::filter_simplex<T>(p, neles, u, ldu, entmin, lde, ef_filter, vdm, ldv,
                                      invvdm, ldi, m0, ldm, mean_wts, ldw, degs, st);
}

template <typename T>
int entropylocal(const b200_ef_t *p, int64_t neles, const T *u, int64_t ldu, T *entmin,
                 int64_t lde, const T *m0, int64_t ldm, cudaStream_t st) {
    if (neles <= 0) return B200_OK;
    if (!p || !u || !entmin || (!p->fpts_in_upts && !m0))
        return b200::set_error(B200_ERR_ARG, "entropylocal: null argument");
    const auto c = ef_consts<T>(*p);
#define X(nd, nu)                                                                  \
    if (p->ndims == nd && p->nupts == nu)                                          \
        return launch_local<nd, nu, T>(p, c, neles, u, ldu, entmin, lde, m0, ldm, st);
    EF_SHAPES(X)
#undef X
    return b200_ef::local_simplex<T>(p, neles, u, ldu, entmin, lde, m0, ldm, st);
}

template <typename T>
int intcent(int64_t n, T *lbase, const void *lmap, T *rbase, const void *rmap, int ix64,
            cudaStream_t st) {
    if (n <= 0) return B200_OK;
    intcent_kernel<T><<<b200::ceil_div(n, 128), 128, 0, st>>>(n, lbase, lmap, rbase, rmap, ix64);
    B200_CHECK_LAUNCH("intcent");
    return B200_OK;
}

// The chosen form keeps its solution in FP64 outside the system: the
// elements that the FP32 filter changed (strength below 1) replace their
// FP64 values by the filtered FP32 ones
__global__ void ef_merge_kernel(int nupts, int nvars, int64_t neles, const float *ef,
                                const float *u32, int64_t ldu, double *acc, int64_t lda) {
    const int64_t e = (int64_t)blockIdx.x * 128 + threadIdx.x;
    const int k = blockIdx.y;
    if (e >= neles || !(ef[e] < 1.0f)) return;
    for (int v = 0; v < nvars; v++) {
        const int64_t o = b200::soa_off(e, v, nvars);
        acc[k * lda + o] = (double)u32[k * ldu + o];
    }
}

}  // namespace

extern "C" {

int b200_ef_merge_f64f32(int nupts, int nvars, int64_t neles, const float *ef_filter,
                         const float *u32, int64_t ldu, double *acc, int64_t lda,
                         void *stream) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    if (!ef_filter || !u32 || !acc) return b200::set_error(B200_ERR_ARG, "ef_merge: null argument");
    dim3 grid(b200::ceil_div(neles, 128), nupts);
    ef_merge_kernel<<<grid, 128, 0, (cudaStream_t)stream>>>(nupts, nvars, neles, ef_filter, u32,
                                                             ldu, acc, lda);
    B200_CHECK_LAUNCH("ef_merge");
    return B200_OK;
}

int b200_entropyfilter_f64(const b200_ef_t *p, int64_t neles, double *u, int64_t ldu,
                           double *entmin, int64_t lde, double *ef_filter, const double *vdm,
                           int64_t ldv, const double *invvdm, int64_t ldi, const double *m0,
                           int64_t ldm, const double *mean_wts, int64_t ldw, const int *degs,
                           void *stream) {
    return entropyfilter<double>(p, neles, u, ldu, entmin, lde, ef_filter, vdm, ldv, invvdm, ldi,
                                 m0, ldm, mean_wts, ldw, degs, (cudaStream_t)stream);
}

int b200_entropyfilter_f32(const b200_ef_t *p, int64_t neles, float *u, int64_t ldu,
                           float *entmin, int64_t lde, float *ef_filter, const float *vdm,
                           int64_t ldv, const float *invvdm, int64_t ldi, const float *m0,
                           int64_t ldm, const float *mean_wts, int64_t ldw, const int *degs,
                           void *stream) {
    return entropyfilter<float>(p, neles, u, ldu, entmin, lde, ef_filter, vdm, ldv, invvdm, ldi,
                                 m0, ldm, mean_wts, ldw, degs, (cudaStream_t)stream);
}

int b200_entropylocal_f64(const b200_ef_t *p, int64_t neles, const double *u, int64_t ldu,
                          double *entmin, int64_t lde, const double *m0, int64_t ldm,
                          void *stream) {
    return entropylocal<double>(p, neles, u, ldu, entmin, lde, m0, ldm, (cudaStream_t)stream);
}

int b200_entropylocal_f32(const b200_ef_t *p, int64_t neles, const float *u, int64_t ldu,
                          float *entmin, int64_t lde, const float *m0, int64_t ldm,
                          void *stream) {
    return entropylocal<float>(p, neles, u, ldu, entmin, lde, m0, ldm, (cudaStream_t)stream);
}

int b200_intcent_f64(int64_t n, double *lbase, const void *lmap, double *rbase,
                     const void *rmap, int ix64, void *stream) {
    return intcent<double>(n, lbase, lmap, rbase, rmap, ix64, (cudaStream_t)stream);
}

int b200_intcent_f32(int64_t n, float *lbase, const void *lmap, float *rbase, const void *rmap,
                     int ix64, void *stream) {
    return intcent<float>(n, lbase, lmap, rbase, rmap, ix64, (cudaStream_t)stream);
}

}  // extern "C"
