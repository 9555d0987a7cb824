// Entropy filter kernels for triangles, tetrahedra, prisms and pyramids of
// orders 1-4 (a separate translation unit so that the library's parallel
// build stays short); the kernels are in entropy.cuh.
#include "entropy.cuh"

namespace b200_ef {

#define EF_SIMPLEX_SHAPES(X)                                                       \
    X(2, 3) X(2, 6) X(2, 10) X(2, 15) X(3, 4) X(3, 10) X(3, 20) X(3, 35)            \
    X(3, 6) X(3, 18) X(3, 40) X(3, 75) X(3, 5) X(3, 14) X(3, 30) X(3, 55)

template <typename T>
int filter_simplex(const b200_ef_t *p, int64_t neles, T *u, int64_t ldu, T *entmin,
                   int64_t lde, T *ef_filter, const T *vdm, int64_t ldv, const T *invvdm,
                   int64_t ldi, const T *m0, int64_t ldm, const T *mean_wts, int64_t ldw,
                   const int *degs, cudaStream_t st) {
    const auto c = ef_consts<T>(*p);
#define X(nd, nu)                                                                  \
    if (p->ndims == nd && p->nupts == nu)                                          \
        return launch_filter<nd, nu, T>(p, c, neles, u, ldu, entmin, lde, ef_filter, vdm, \
                                        ldv, invvdm, ldi, m0, ldm, mean_wts, ldw, degs, st);
    EF_SIMPLEX_SHAPES(X)
#undef X
    return b200::set_error(B200_ERR_UNSUPPORTED, "entropyfilter: no kernel for %d points in %dD",
                           p->nupts, p->ndims);
}

template <typename T>
int local_simplex(const b200_ef_t *p, int64_t neles, const T *u, int64_t ldu, T *entmin,
                  int64_t lde, const T *m0, int64_t ldm, cudaStream_t st) {
    const auto c = ef_consts<T>(*p);
#define X(nd, nu)                                                                  \
    if (p->ndims == nd && p->nupts == nu)                                          \
        return launch_local<nd, nu, T>(p, c, neles, u, ldu, entmin, lde, m0, ldm, st);
    EF_SIMPLEX_SHAPES(X)
#undef X
    return b200::set_error(B200_ERR_UNSUPPORTED, "entropylocal: no kernel for %d points in %dD",
                           p->nupts, p->ndims);
}

template int filter_simplex<double>(const b200_ef_t *, int64_t, double *, int64_t, double *,
                                    int64_t, double *, const double *, int64_t,
                                    const double *, int64_t, const double *, int64_t,
                                    const double *, int64_t, const int *, cudaStream_t);
template int filter_simplex<float>(const b200_ef_t *, int64_t, float *, int64_t, float *,
                                   int64_t, float *, const float *, int64_t, const float *,
                                   int64_t, const float *, int64_t, const float *, int64_t,
                                   const int *, cudaStream_t);
template int local_simplex<double>(const b200_ef_t *, int64_t, const double *, int64_t,
                                   double *, int64_t, const double *, int64_t, cudaStream_t);
template int local_simplex<float>(const b200_ef_t *, int64_t, const float *, int64_t, float *,
                                  int64_t, const float *, int64_t, cudaStream_t);

}  // namespace b200_ef
