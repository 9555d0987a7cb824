#pragma once
// Entropy filter (shock capturing) of the Euler and Navier-Stokes systems,
// kernel templates shared by entropy.cu (tensor-product shapes) and
// entropy_simplex.cu (triangles, tetrahedra, prisms):
// per-element minimum entropy, its exchange across interfaces, and the
// bounds-preserving modal filter.
//
//   compute_entropy   pyfr/solvers/euler/kernels/entropy.mako:3-13
//   entropylocal      pyfr/solvers/euler/kernels/entropylocal.mako:5-40
//   entropyfilter     pyfr/solvers/euler/kernels/entropyfilter.mako:5-221
//   intcent           pyfr/solvers/baseadvec/kernels/intcent.mako:4-8
//   bccent            pyfr/solvers/euler/kernels/bccent.mako:7-25
//   set-up            pyfr/solvers/baseadvec/entfilter.py:5-213
//
// One thread per element (per interface face, per boundary flux point).
// The element's solution is read and written in place in its AoSoA
// layout; the filter's modal coefficients live in thread-local arrays
// sized by the number of solution points, a template parameter.
#include <cfloat>
#include <cstdint>

#include "common.cuh"
#include "physics.cuh"
#include "pyfrb200.h"

namespace {

constexpr int EF_BLOCK = 64;
constexpr int EF_MAX_ORDER = 8;

template <typename T> __host__ __device__ constexpr T fp_max();
template <> __host__ __device__ constexpr double fp_max<double>() { return DBL_MAX; }
template <> __host__ __device__ constexpr float fp_max<float>() { return FLT_MAX; }

template <typename T>
struct EfConsts {
    T gamma, d_min, p_min, e_tol, f_tol;
    int niters, linearise, order, fpts_in_upts;
};

// Density, pressure and the entropy function p rho^-gamma (the largest
// value when density or pressure is not positive)
template <int NV, typename T>
__device__ __forceinline__ void entropy(const T *u, const EfConsts<T> &c, T &d, T &p, T &e) {
    d = u[0];
    const T rcpd = T(1) / d;
    T k2 = 0;
#pragma unroll
    for (int i = 1; i < NV - 1; i++) k2 += u[i] * u[i];
    p = (c.gamma - T(1)) * (u[NV - 1] - T(0.5) * rcpd * k2);
    e = (d > 0 && p > 0) ? p * pow(rcpd, c.gamma) : fp_max<T>();
}

template <int NV, typename T>
__device__ __forceinline__ bool violates(T d, T p, T e, T entmin, const EfConsts<T> &c) {
    return d < c.d_min || p < c.p_min || e < entmin - c.e_tol;
}

// Minima of density, pressure and entropy over the solution points and,
// when they are not among them, the flux points (m0 interpolation)
template <int NV, int NU, typename T>
__device__ void get_minima(const T *__restrict__ u, int64_t ldu, int64_t e, int nfpts,
                           const T *__restrict__ m0, int64_t ldm, const EfConsts<T> &c, T &dmin,
                           T &pmin, T &emin) {
    dmin = pmin = emin = fp_max<T>();
    T ui[NV], d, p, s;
    for (int i = 0; i < NU; i++) {
#pragma unroll
        for (int v = 0; v < NV; v++) ui[v] = u[i * ldu + b200::soa_off(e, v, NV)];
        entropy<NV, T>(ui, c, d, p, s);
        dmin = fmin(dmin, d);
        pmin = fmin(pmin, p);
        emin = fmin(emin, s);
    }
    if (!c.fpts_in_upts) {
        for (int f = 0; f < nfpts; f++) {
#pragma unroll
            for (int v = 0; v < NV; v++) ui[v] = 0;
            for (int k = 0; k < NU; k++) {
                const T w = m0[f * ldm + k];
#pragma unroll
                for (int v = 0; v < NV; v++) ui[v] += w * u[k * ldu + b200::soa_off(e, v, NV)];
            }
            entropy<NV, T>(ui, c, d, p, s);
            dmin = fmin(dmin, d);
            pmin = fmin(pmin, p);
            emin = fmin(emin, s);
        }
    }
}

// The filtered state at one point from its modal contributions grouped by
// degree, up[deg][var], for filter strength f (mode of degree k damped by
// f^(k^2)), and its density, pressure and entropy
template <int NV, typename T>
__device__ __forceinline__ void filter_point(const T up[][NV], int order, T f,
                                             const EfConsts<T> &c, T &d, T &p, T &e) {
    T ui[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) ui[v] = up[0][v];
    T fv = 1, fv2 = 1;
    for (int k = 1; k <= order; k++) {
        fv2 *= fv * fv * f;
        fv *= f;
#pragma unroll
        for (int v = 0; v < NV; v++) ui[v] += fv2 * up[k][v];
    }
    entropy<NV, T>(ui, c, d, p, e);
}

template <int ND, int NU, typename T>
__global__ void __launch_bounds__(EF_BLOCK)
entropyfilter_kernel(int64_t neles, EfConsts<T> c, int nfaces, int nfpts, int nefpts,
                     T *__restrict__ u, int64_t ldu, T *__restrict__ entmin_int, int64_t lde,
                     T *__restrict__ ef_filter, const T *__restrict__ vdm, int64_t ldv,
                     const T *__restrict__ invvdm, int64_t ldi, const T *__restrict__ m0,
                     int64_t ldm, const T *__restrict__ mean_wts, int64_t ldw,
                     const int *__restrict__ degs) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * EF_BLOCK + threadIdx.x;
    if (e >= neles) return;
    const int order = c.order;

    // Smallest entropy of the element and its neighbours
    T entmin = fp_max<T>();
    for (int f = 0; f < nfaces; f++) entmin = fmin(entmin, entmin_int[f * lde + e]);

    T dmin, pmin, emin;
    get_minima<NV, NU, T>(u, ldu, e, nfpts, m0, ldm, c, dmin, pmin, emin);

    // Element mean (Jacobian-weighted)
    T uavg[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uavg[v] = 0;
    for (int k = 0; k < NU; k++) {
        const T w = mean_wts[k * ldw + e];
#pragma unroll
        for (int v = 0; v < NV; v++) uavg[v] += w * u[k * ldu + b200::soa_off(e, v, NV)];
    }

    T f = 1;
    if (!c.linearise && violates<NV, T>(dmin, pmin, emin, entmin, c)) {
        // Modal coefficients
        T um[NU][NV];
        for (int m = 0; m < NU; m++) {
#pragma unroll
            for (int v = 0; v < NV; v++) um[m][v] = 0;
            for (int k = 0; k < NU; k++) {
                const T w = invvdm[m * ldi + k];
#pragma unroll
                for (int v = 0; v < NV; v++) um[m][v] += w * u[k * ldu + b200::soa_off(e, v, NV)];
            }
        }

        // Largest filter strength f = exp(-zeta) that keeps every point
        // within the bounds, by bisection point by point
        T up[EF_MAX_ORDER + 1][NV];
        for (int i = 0; i < nefpts; i++) {
            for (int k = 0; k <= order; k++)
#pragma unroll
                for (int v = 0; v < NV; v++) up[k][v] = 0;
            for (int m = 0; m < NU; m++) {
                const T w = vdm[i * ldv + m];
                const int dg = degs[m];
#pragma unroll
                for (int v = 0; v < NV; v++) up[dg][v] += w * um[m][v];
            }
            T d, p, s;
            filter_point<NV, T>(up, order, f, c, d, p, s);
            if (violates<NV, T>(d, p, s, entmin, c)) {
                T fhi = f, flo = 0;
                for (int it = 0; it < c.niters && fhi - flo > c.f_tol; it++) {
                    const T fnew = T(0.5) * (flo + fhi);
                    filter_point<NV, T>(up, order, fnew, c, d, p, s);
                    if (violates<NV, T>(d, p, s, entmin, c))
                        fhi = fnew;
                    else
                        flo = fnew;
                }
                f = flo;
            }
        }

        // Filter the whole solution with that strength
        T ffac[EF_MAX_ORDER + 1];
        T fv = ffac[0] = 1;
        for (int k = 1; k <= order; k++) {
            ffac[k] = ffac[k - 1] * fv * fv * f;
            fv *= f;
        }
        for (int i = 0; i < NU; i++) {
            T acc[NV];
#pragma unroll
            for (int v = 0; v < NV; v++) acc[v] = 0;
            for (int m = 0; m < NU; m++) {
                const T w = ffac[degs[m]] * vdm[i * ldv + m];
#pragma unroll
                for (int v = 0; v < NV; v++) acc[v] += w * um[m][v];
            }
#pragma unroll
            for (int v = 0; v < NV; v++) u[i * ldu + b200::soa_off(e, v, NV)] = acc[v];
        }

        // Restore the element mean (the filter acts in reference space)
        T dav[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) dav[v] = uavg[v];
        for (int k = 0; k < NU; k++) {
            const T w = mean_wts[k * ldw + e];
#pragma unroll
            for (int v = 0; v < NV; v++) dav[v] -= w * u[k * ldu + b200::soa_off(e, v, NV)];
        }
        for (int k = 0; k < NU; k++)
#pragma unroll
            for (int v = 0; v < NV; v++) u[k * ldu + b200::soa_off(e, v, NV)] += dav[v];

        get_minima<NV, NU, T>(u, ldu, e, nfpts, m0, ldm, c, dmin, pmin, emin);
    }

    // Linear limiting towards the mean: density, then pressure, then entropy
    if (violates<NV, T>(dmin, pmin, emin, entmin, c)) {
        T davg, pavg, eavg;
        entropy<NV, T>(uavg, c, davg, pavg, eavg);
        for (int q = 0; q < 3; q++) {
            const T vmin = q == 0 ? dmin : (q == 1 ? pmin : emin);
            const T vavg = q == 0 ? davg : (q == 1 ? pavg : eavg);
            const T bound = q == 0 ? c.d_min : (q == 1 ? c.p_min : entmin - c.e_tol);
            if (vmin < bound) {
                T alpha = (vmin - bound) / (vmin - vavg);
                alpha = fmin(fmax(alpha, T(0)), T(1));
                f = fmin(f, T(1) - alpha);
                const int nv = q == 0 ? 1 : NV;
                for (int k = 0; k < NU; k++)
                    for (int v = 0; v < nv; v++) {
                        T &x = u[k * ldu + b200::soa_off(e, v, NV)];
                        x += alpha * (uavg[v] - x);
                    }
                get_minima<NV, NU, T>(u, ldu, e, nfpts, m0, ldm, c, dmin, pmin, emin);
            }
        }
    }

    for (int fc = 0; fc < nfaces; fc++) entmin_int[fc * lde + e] = emin;
    ef_filter[e] = f;
}

template <int ND, int NU, typename T>
__global__ void __launch_bounds__(EF_BLOCK)
entropylocal_kernel(int64_t neles, EfConsts<T> c, int nfaces, int nfpts, const T *__restrict__ u,
                    int64_t ldu, T *__restrict__ entmin_int, int64_t lde,
                    const T *__restrict__ m0, int64_t ldm) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * EF_BLOCK + threadIdx.x;
    if (e >= neles) return;
    T dmin, pmin, emin;
    get_minima<NV, NU, T>(u, ldu, e, nfpts, m0, ldm, c, dmin, pmin, emin);
    for (int f = 0; f < nfaces; f++) entmin_int[f * lde + e] = emin;
}

template <typename T>
__global__ void intcent_kernel(int64_t n, T *lbase, const void *lmap, T *rbase, const void *rmap,
                               int ix64) {
    const int64_t i = (int64_t)blockIdx.x * 128 + threadIdx.x;
    if (i >= n) return;
    T *l = lbase + b200::load_ix(lmap, ix64, i);
    T *r = rbase + b200::load_ix(rmap, ix64, i);
    const T m = fmin(*l, *r);
    *l = m;
    *r = m;
}

template <typename T>
EfConsts<T> ef_consts(const b200_ef_t &p) {
    EfConsts<T> c;
    c.gamma = (T)p.gamma;
    c.d_min = (T)p.d_min;
    c.p_min = (T)p.p_min;
    c.e_tol = (T)p.e_tol;
    c.f_tol = (T)p.f_tol;
    c.niters = p.niters;
    c.linearise = p.linearise;
    c.order = p.order;
    c.fpts_in_upts = p.fpts_in_upts;
    return c;
}


// Launch the filter or the minima kernel for one (ndims, points) shape
template <int ND, int NU, typename T>
int launch_filter(const b200_ef_t *p, const EfConsts<T> &c, int64_t neles, T *u, int64_t ldu,
                  T *entmin, int64_t lde, T *ef_filter, const T *vdm, int64_t ldv,
                  const T *invvdm, int64_t ldi, const T *m0, int64_t ldm, const T *mean_wts,
                  int64_t ldw, const int *degs, cudaStream_t st) {
    entropyfilter_kernel<ND, NU, T><<<b200::ceil_div(neles, EF_BLOCK), EF_BLOCK, 0, st>>>(
        neles, c, p->nfaces, p->nfpts, p->nefpts, u, ldu, entmin, lde, ef_filter, vdm, ldv,
        invvdm, ldi, m0, ldm, mean_wts, ldw, degs);
    B200_CHECK_LAUNCH("entropyfilter");
    return B200_OK;
}

template <int ND, int NU, typename T>
int launch_local(const b200_ef_t *p, const EfConsts<T> &c, int64_t neles, const T *u,
                 int64_t ldu, T *entmin, int64_t lde, const T *m0, int64_t ldm,
                 cudaStream_t st) {
    entropylocal_kernel<ND, NU, T><<<b200::ceil_div(neles, EF_BLOCK), EF_BLOCK, 0, st>>>(
        neles, c, p->nfaces, p->nfpts, u, ldu, entmin, lde, m0, ldm);
    B200_CHECK_LAUNCH("entropylocal");
    return B200_OK;
}

}  // namespace

// Triangles, tetrahedra and prisms of orders 1-4 (entropy_simplex.cu);
// B200_ERR_UNSUPPORTED for any other shape
namespace b200_ef {
template <typename T>
int filter_simplex(const b200_ef_t *p, int64_t neles, T *u, int64_t ldu, T *entmin,
                   int64_t lde, T *ef_filter, const T *vdm, int64_t ldv, const T *invvdm,
                   int64_t ldi, const T *m0, int64_t ldm, const T *mean_wts, int64_t ldw,
                   const int *degs, cudaStream_t st);
template <typename T>
int local_simplex(const b200_ef_t *p, int64_t neles, const T *u, int64_t ldu, T *entmin,
                  int64_t lde, const T *m0, int64_t ldm, cudaStream_t st);
}  // namespace b200_ef
