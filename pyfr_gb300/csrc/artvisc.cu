// Artificial viscosity (shock capturing) of the Navier-Stokes system: the
// per-element shock sensor, its maximum over the mesh vertices, and the
// linear interpolation of the vertex values to the flux and solution
// points.
//
//   shocksensor   pyfr/solvers/baseadvecdiff/kernels/shocksensor.mako
//   avfill        pyfr/solvers/baseadvecdiff/kernels/avfill.mako
//   set-up        pyfr/solvers/baseadvecdiff/artvisc.py:24-200
//
// The sensor runs one thread per element: the modal coefficients of the
// sensed variable come from the inverse Vandermonde matrix (read through
// the L1 broadcast, every thread of a warp reading the same row), and the
// element's viscosity goes to each of its vertices with an integer
// atomicMax on the bit pattern of the non-negative value, which orders as
// the value does.  The vertex buffer is zeroed before the sensor runs.
#include <cstdint>

#include "common.cuh"
#include "pyfrb200.h"

namespace {

constexpr int AV_BLOCK = 128;
constexpr int AV_MAX_DEG = 16;

__device__ __forceinline__ void atomic_max_nonneg(double *a, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(a),
              (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_max_nonneg(float *a, float v) {
    atomicMax(reinterpret_cast<unsigned int *>(a), __float_as_uint(v));
}

template <typename T>
struct AvConsts {
    int nupts, nvars, svar, nverts, nmodes, ndeg, kwh;
    T kappa, max_av, se0;
    T w[AV_MAX_DEG], bd[AV_MAX_DEG];
};

template <typename T>
AvConsts<T> av_consts(const b200_av_t &p) {
    AvConsts<T> k;
    k.nupts = p.nupts;
    k.nvars = p.nvars;
    k.svar = p.svar;
    k.nverts = p.nverts;
    k.nmodes = p.nmodes;
    k.ndeg = p.ndeg;
    k.kwh = p.kwh;
    k.kappa = (T)p.kappa;
    k.max_av = (T)p.max_av;
    k.se0 = (T)p.se0;
    for (int i = 0; i < AV_MAX_DEG; i++) {
        k.w[i] = (T)p.s_weights[i];
        k.bd[i] = (T)p.baseline[i];
    }
    return k;
}

template <typename T>
__global__ void __launch_bounds__(AV_BLOCK)
shocksensor_kernel(AvConsts<T> c, int64_t neles, const T *__restrict__ u, int64_t ldu,
                   const T *__restrict__ invvdm, int64_t ldi, const int *__restrict__ degs,
                   const int *__restrict__ ind, const int *__restrict__ vnodes, int64_t ldn,
                   T *__restrict__ vtx) {
    const int64_t e = (int64_t)blockIdx.x * AV_BLOCK + threadIdx.x;
    if (e >= neles) return;
    const int64_t uoff = b200::soa_off(e, c.svar, c.nvars);
    const T pi = T(3.14159265358979323846);

    T mu;
    if (c.kwh) {
        // Klockner-Warburton-Hesthaven: energy per degree, a baseline decay
        // against noise, the skyline envelope, and the least-squares decay
        // rate of the energies of degrees 1..ndeg-1
        T en[AV_MAX_DEG];
        for (int d = 0; d < c.ndeg; d++) en[d] = 0;
        for (int k = 0; k < c.nmodes; k++) {
            T tmp = 0;
            for (int j = 0; j < c.nupts; j++) tmp += invvdm[k * ldi + j] * u[j * ldu + uoff];
            en[degs[k]] += tmp * tmp;
        }
        T tot = en[0];
        for (int d = 1; d < c.ndeg; d++) tot += en[d];
        for (int d = 1; d < c.ndeg; d++) en[d] += tot * c.bd[d - 1];
        for (int d = c.ndeg - 2; d >= 0; d--) en[d] = fmax(en[d], en[d + 1]);
        T s = 0;
        for (int d = 1; d < c.ndeg; d++) s += c.w[d - 1] * log(en[d]);
        s *= T(-0.5);
        mu = (s > T(2) + c.kappa)
                 ? T(0)
                 : T(0.5) * c.max_av * (T(1) - sin(T(0.5) * pi / c.kappa * (s - T(2))));
        mu = (s < T(2) - c.kappa) ? c.max_av : mu;
    } else {
        // Persson-Peraire: the share of the highest-degree modes
        T tot = 0, pn = T(1e-15);
        for (int k = 0; k < c.nmodes; k++) {
            T tmp = 0;
            for (int j = 0; j < c.nupts; j++) tmp += invvdm[k * ldi + j] * u[j * ldu + uoff];
            tot += tmp * tmp;
            if (ind[k]) pn += tmp * tmp;
        }
        const T se = T(1) / log(T(10)) * log(pn / tot);
        mu = (se < c.se0 - c.kappa)
                 ? T(0)
                 : T(0.5) * c.max_av * (T(1) + sin(T(0.5) * pi / c.kappa * (se - c.se0)));
        mu = (se < c.se0 + c.kappa) ? mu : c.max_av;
    }

    for (int i = 0; i < c.nverts; i++) atomic_max_nonneg(&vtx[vnodes[i * ldn + e]], mu);
}

template <typename T>
__global__ void __launch_bounds__(AV_BLOCK)
avfill_kernel(int nverts, int npts, int64_t neles, const T *__restrict__ vtx,
              const int *__restrict__ vnodes, int64_t ldn, const T *__restrict__ op,
              int64_t ldo, T *__restrict__ out, int64_t ldout) {
    const int64_t e = (int64_t)blockIdx.x * AV_BLOCK + threadIdx.x;
    const int p = blockIdx.y;
    if (e >= neles) return;
    T acc = 0;
    for (int i = 0; i < nverts; i++) acc += op[p * ldo + i] * vtx[vnodes[i * ldn + e]];
    out[p * ldout + e] = acc;
}

template <typename T>
int shocksensor(const b200_av_t *p, int64_t neles, const T *u, int64_t ldu, const T *invvdm,
                int64_t ldi, const int *degs, const int *ind, const int *vnodes, int64_t ldn,
                T *vtx, cudaStream_t st) {
    if (!p) return b200::set_error(B200_ERR_ARG, "shocksensor: null parameters");
    if (neles <= 0) return B200_OK;
    if (p->ndeg < 1 || p->ndeg > AV_MAX_DEG || p->nmodes <= 0 || p->nupts <= 0 ||
        p->nverts <= 0 || p->svar < 0 || p->svar >= p->nvars)
        return b200::set_error(B200_ERR_ARG, "shocksensor: bad sizes");
    const auto c = av_consts<T>(*p);
    shocksensor_kernel<T><<<b200::ceil_div(neles, AV_BLOCK), AV_BLOCK, 0, st>>>(
        c, neles, u, ldu, invvdm, ldi, degs, ind, vnodes, ldn, vtx);
    B200_CHECK_LAUNCH("shocksensor");
    return B200_OK;
}

template <typename T>
int avfill(int nverts, int npts, int64_t neles, const T *vtx, const int *vnodes, int64_t ldn,
           const T *op, int64_t ldo, T *out, int64_t ldout, cudaStream_t st) {
    if (neles <= 0 || npts <= 0) return B200_OK;
    if (nverts <= 0) return b200::set_error(B200_ERR_ARG, "avfill: bad sizes");
    dim3 grid(b200::ceil_div(neles, AV_BLOCK), npts);
    avfill_kernel<T><<<grid, AV_BLOCK, 0, st>>>(nverts, npts, neles, vtx, vnodes, ldn, op, ldo,
                                                out, ldout);
    B200_CHECK_LAUNCH("avfill");
    return B200_OK;
}

}  // namespace

extern "C" {

int b200_shocksensor_f64(const b200_av_t *p, int64_t neles, const double *u, int64_t ldu,
                         const double *invvdm, int64_t ldi, const int *degs, const int *ind,
                         const int *vnodes, int64_t ldn, double *vtx, void *stream) {
    return shocksensor<double>(p, neles, u, ldu, invvdm, ldi, degs, ind, vnodes, ldn, vtx,
                               (cudaStream_t)stream);
}

int b200_shocksensor_f32(const b200_av_t *p, int64_t neles, const float *u, int64_t ldu,
                         const float *invvdm, int64_t ldi, const int *degs, const int *ind,
                         const int *vnodes, int64_t ldn, float *vtx, void *stream) {
    return shocksensor<float>(p, neles, u, ldu, invvdm, ldi, degs, ind, vnodes, ldn, vtx,
                              (cudaStream_t)stream);
}

int b200_avfill_f64(int nverts, int npts, int64_t neles, const double *vtx, const int *vnodes,
                    int64_t ldn, const double *op, int64_t ldo, double *out, int64_t ldout,
                    void *stream) {
    return avfill<double>(nverts, npts, neles, vtx, vnodes, ldn, op, ldo, out, ldout,
                          (cudaStream_t)stream);
}

int b200_avfill_f32(int nverts, int npts, int64_t neles, const float *vtx, const int *vnodes,
                    int64_t ldn, const float *op, int64_t ldo, float *out, int64_t ldout,
                    void *stream) {
    return avfill<float>(nverts, npts, neles, vtx, vnodes, ldn, op, ldo, out, ldout,
                         (cudaStream_t)stream);
}

}  // extern "C"
