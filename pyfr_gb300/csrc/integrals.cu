// Field integrals for the kinetic-energy and enstrophy histories.
//
// Restates the reference's field reducer (pyfr/plugins/fieldeval.py:25-248
// with pyfr/plugins/kernels/fieldeval.mako:5-29) for its documented
// Taylor-Green integrands (doc/src/plugins/soln-plugin-integrate.rst):
//   int-E    = rho*(u*u + v*v [+ w*w])
//   int-enst = rho*|curl u|^2
// evaluated at the solution points with quadrature weights times |J|
// (the weights matrix of fieldeval.py:98-115), plus the volume.  Primitive
// gradients follow grad_con_to_pri (pyfr/solvers/euler/kernels/eos.mako:24-45).
// Sums are accumulated in FP64 whatever the storage precision, with fixed
// block partials and one ordered final pass (deterministic).
#include "common.cuh"
#include "../../include/pyfrb200.h"

namespace {

constexpr int IG_BLOCK = 256;
constexpr int IG_NOUT = 3;

// Constant per-variable offset added to the stored solution (a solution
// kept relative to a reference state); zero when there is none.
struct URef {
    double v[5];
};

template <int ND, typename TU, typename TG>
__global__ void __launch_bounds__(IG_BLOCK)
integrals_partial_kernel(int nupts, int64_t neles, const TU *__restrict__ u, int64_t ldu,
                         const TG *__restrict__ g, int64_t ldg, const double *__restrict__ wts,
                         int64_t ldw, URef uref, double *__restrict__ partial) {
    constexpr int NV = ND + 2;
    __shared__ double red[IG_NOUT][IG_BLOCK / 32];
    double acc[IG_NOUT] = {0, 0, 0};

    const int64_t npts = (int64_t)nupts * neles;
    for (int64_t p = (int64_t)blockIdx.x * IG_BLOCK + threadIdx.x; p < npts;
         p += (int64_t)gridDim.x * IG_BLOCK) {
        const int upt = (int)(p / neles);
        const int64_t e = p % neles;
        const double w = wts[upt * ldw + e];

        double s[NV];
#pragma unroll
        for (int v = 0; v < NV; v++)
            s[v] = (double)u[upt * ldu + b200::soa_off(e, v, NV)] + uref.v[v];
        const double rho = s[0], invrho = 1.0 / rho;
        double vel[ND], ke = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            vel[i] = invrho * s[i + 1];
            ke += vel[i] * vel[i];
        }

        // Velocity gradients: du_i/dx_d = (d(rho u_i)/dx_d - u_i drho/dx_d)/rho
        double du[ND][ND];
#pragma unroll
        for (int d = 0; d < ND; d++) {
            const double gr = (double)g[(int64_t)(d * nupts + upt) * ldg + b200::soa_off(e, 0, NV)];
#pragma unroll
            for (int i = 0; i < ND; i++) {
                const double gm = (double)g[(int64_t)(d * nupts + upt) * ldg +
                                            b200::soa_off(e, i + 1, NV)];
                du[i][d] = invrho * (gm - vel[i] * gr);
            }
        }

        double enst;
        if (ND == 3) {
            const double w1 = du[2][1] - du[1][2];
            const double w2 = du[0][2] - du[2][0];
            const double w3 = du[1][0] - du[0][1];
            enst = w1 * w1 + w2 * w2 + w3 * w3;
        } else {
            const double w3 = du[1][0] - du[0][1];
            enst = w3 * w3;
        }

        acc[0] += w * rho * ke;
        acc[1] += w * rho * enst;
        acc[2] += w;
    }

#pragma unroll
    for (int k = 0; k < IG_NOUT; k++) {
        double x = acc[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) red[k][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < IG_NOUT) {
        double x = 0;
        for (int w = 0; w < IG_BLOCK / 32; w++) x += red[threadIdx.x][w];
        partial[(int64_t)blockIdx.x * IG_NOUT + threadIdx.x] = x;
    }
}

__global__ void integrals_final_kernel(int nblk, const double *__restrict__ partial,
                                       double *__restrict__ out) {
    if (blockIdx.x == 0 && threadIdx.x < IG_NOUT) {
        double x = 0;
        for (int b = 0; b < nblk; b++) x += partial[(int64_t)b * IG_NOUT + threadIdx.x];
        out[threadIdx.x] = x;
    }
}

template <typename TU, typename TG>
int integrals(int ndims, int nupts, int64_t neles, const TU *u, int64_t ldu, const TG *g,
              int64_t ldg, const double *wts, int64_t ldw, const double *uref, double *scratch,
              int nscratch, double *out, cudaStream_t s) {
    if (nscratch < 1) return b200::set_error(B200_ERR_ARG, "integrals: no scratch");
    if (!u || !g || !wts || !out)
        return b200::set_error(B200_ERR_ARG, "integrals: null argument");
    const int64_t npts = (int64_t)nupts * neles;
    int64_t want = (npts + IG_BLOCK - 1) / IG_BLOCK;
    int nblk = (int)(want < 1 ? 1 : (want > nscratch ? nscratch : want));
    URef ur = {};
    if (uref)
        for (int v = 0; v < ndims + 2 && v < 5; v++) ur.v[v] = uref[v];
    if (ndims == 3)
        integrals_partial_kernel<3, TU, TG><<<nblk, IG_BLOCK, 0, s>>>(nupts, neles, u, ldu, g, ldg,
                                                                      wts, ldw, ur, scratch);
    else if (ndims == 2)
        integrals_partial_kernel<2, TU, TG><<<nblk, IG_BLOCK, 0, s>>>(nupts, neles, u, ldu, g, ldg,
                                                                      wts, ldw, ur, scratch);
    else
        return b200::set_error(B200_ERR_ARG, "integrals: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("integrals_partial");
    integrals_final_kernel<<<1, 32, 0, s>>>(nblk, scratch, out);
    B200_CHECK_LAUNCH("integrals_final");
    return B200_OK;
}

}  // namespace

extern "C" {

int b200_integrals_f64(int ndims, int nupts, int64_t neles, const double *u, int64_t ldu,
                       const double *gradu, int64_t ldg, const double *wts, int64_t ldw,
                       double *scratch, int nscratch, double *out, void *stream) {
    return integrals<double, double>(ndims, nupts, neles, u, ldu, gradu, ldg, wts, ldw, nullptr,
                                     scratch, nscratch, out, (cudaStream_t)stream);
}

int b200_integrals_f64f32(int ndims, int nupts, int64_t neles, const double *u, int64_t ldu,
                          const float *gradu, int64_t ldg, const double *wts, int64_t ldw,
                          const double *uref, double *scratch, int nscratch, double *out,
                          void *stream) {
    return integrals<double, float>(ndims, nupts, neles, u, ldu, gradu, ldg, wts, ldw, uref,
                                    scratch, nscratch, out, (cudaStream_t)stream);
}

}  // extern "C"
