// Pointwise and interface kernels of the right-hand side.
//
// Element kernels run over [nupts, neles] (one thread per solution point,
// consecutive threads on consecutive elements, so every access to an AoSoA
// field is a coalesced 32-element segment).  Interface kernels run over the
// interior flux-point pairs and reach both sides through the view gather
// maps (element offsets into the flux-point buffer, variable stride 32),
// the addressing of pyfr/backends/base/types.py:260-320.
//
//   tflux (Euler)      pyfr/solvers/euler/kernels/tflux.mako:8-30
//   tflux (NS, fused)  pyfr/solvers/navstokes/kernels/tflux.mako:13-50
//   gradcoru           pyfr/solvers/baseadvecdiff/kernels/gradcoru.mako:10-24
//   negdivconf         pyfr/solvers/baseadvec/kernels/negdivconf.mako:7-22
//   srcterms           negdivconf with source macros, evalsrcmacros.mako:7-22,
//                      pyfr/plugins/kernels/source.mako
//   intcflux (Euler)   pyfr/solvers/euler/kernels/intcflux.mako:6-22 (any of the
//                      six Riemann solvers, a template argument)
//   intcflux (NS)      pyfr/solvers/navstokes/kernels/intcflux.mako:10-54
//   intconu            pyfr/solvers/navstokes/kernels/intconu.mako:4-19
#include "common.cuh"
#include "exprprog.cuh"
#include "physics.cuh"
#include "../../include/pyfrb200.h"

using b200::Gas;
using b200::soa_off;

namespace {

constexpr int PW_BLOCK = 128;

template <typename T>
struct ElemGeom {
    const T *smats;  int64_t lds;
    const T *rcpdjac; int64_t ldr;
    const T *verts;  int64_t ldv;
    const T *upts;   int64_t ldup;
    int linear;
};

// Geometry modes (the `linear` argument of the element kernels)
enum { GEOM_STORED = 0, GEOM_VERTICES = 1, GEOM_PER_ELEMENT = 2 };

// Metric terms at solution point `upt` of element `e`: from the vertices
// (GEOM_VERTICES, multilinear elements), from the stored per-point smats
// and 1/|J| (GEOM_STORED), or from one stored set per element
// (GEOM_PER_ELEMENT: affine elements, whose Jacobian is constant, keep
// only the rows of their first point: io-shapes (ndims, 1, ndims, neles)
// and (1, neles)).
template <int ND, typename T>
__device__ __forceinline__ void elem_metrics(const ElemGeom<T> &g, int nupts, int upt,
                                             int64_t e, T s[ND][ND], T &rcpdjac,
                                             bool need_rcp) {
    if (g.linear == GEOM_PER_ELEMENT) {
        nupts = 1;
        upt = 0;
    }
    if (g.linear == GEOM_VERTICES) {
        T V[1 << ND][ND], x[ND], d;
#pragma unroll
        for (int v = 0; v < (1 << ND); v++)
#pragma unroll
            for (int k = 0; k < ND; k++) V[v][k] = g.verts[v * g.ldv + soa_off(e, k, ND)];
#pragma unroll
        for (int k = 0; k < ND; k++) x[k] = g.upts[upt * g.ldup + k];
        b200::linear_smats<ND, T>(V, x, s, d);
        rcpdjac = need_rcp ? T(1) / d : T(0);
    } else {
#pragma unroll
        for (int i = 0; i < ND; i++)
#pragma unroll
            for (int j = 0; j < ND; j++)
                s[i][j] = g.smats[(int64_t)(i * nupts + upt) * g.lds + soa_off(e, j, ND)];
        rcpdjac = need_rcp ? g.rcpdjac[(int64_t)upt * g.ldr + e] : T(0);
    }
}

template <int ND, typename T>
__global__ void __launch_bounds__(PW_BLOCK)
tflux_euler_kernel(int nupts, int64_t neles, T gamma, const T *__restrict__ u, int64_t ldu,
                   T *__restrict__ f, int64_t ldf, ElemGeom<T> geo) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    const int upt = blockIdx.y;
    if (e >= neles) return;

    T s[ND][ND], rcp;
    elem_metrics<ND, T>(geo, nupts, upt, e, s, rcp, false);

    T uu[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uu[v] = u[upt * ldu + soa_off(e, v, NV)];

    T ft[ND][NV], p, vel[ND];
    b200::inviscid_flux<ND, T>(uu, ft, p, vel, gamma);

#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int j = 0; j < NV; j++) {
            T acc = 0;
#pragma unroll
            for (int k = 0; k < ND; k++) acc += s[i][k] * ft[k][j];
            f[(int64_t)(i * nupts + upt) * ldf + soa_off(e, j, NV)] = acc;
        }
}

// Euler transformed flux on shifted inputs q = T(u - u_ref) (b200::Gas):
// the flux less the reference state's, formed from the perturbation
template <int ND, typename T, bool MOVING>
__global__ void __launch_bounds__(PW_BLOCK)
tflux_euler_shift_kernel(int nupts, int64_t neles, b200::GasK<T> gas, const T *__restrict__ u,
                         int64_t ldu, T *__restrict__ f, int64_t ldf, ElemGeom<T> geo) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    const int upt = blockIdx.y;
    if (e >= neles) return;

    T s[ND][ND], rcp;
    elem_metrics<ND, T>(geo, nupts, upt, e, s, rcp, false);

    T uu[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uu[v] = u[upt * ldu + soa_off(e, v, NV)];

    T ft[ND][NV], p, vel[ND], uf[NV];
    b200::inviscid_flux_shift<ND, T, MOVING>(uu, ft, p, vel, uf, gas);

#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int j = 0; j < NV; j++) {
            T acc = 0;
#pragma unroll
            for (int k = 0; k < ND; k++) acc += s[i][k] * ft[k][j];
            f[(int64_t)(i * nupts + upt) * ldf + soa_off(e, j, NV)] = acc;
        }
}

// Largest characteristic wave speed of each element in reference space,
// for the CFL controller (pyfr/solvers/euler/kernels/wavespeed.mako:9-44):
// max over the solution points of sum_i |sum_j (S_ij/|J|) v_j| +
// c sqrt(sum_j (S_ij/|J|)^2).  One thread per element walks the points.
template <int ND, typename T>
__global__ void __launch_bounds__(PW_BLOCK)
wavespeed_kernel(int nupts, int64_t neles, b200::GasK<T> gas, const T *__restrict__ u,
                 int64_t ldu, ElemGeom<T> geo, T *__restrict__ wspd) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    if (e >= neles) return;

    T lmax = 0;
    for (int upt = 0; upt < nupts; upt++) {
        T s[ND][ND], rcp;
        elem_metrics<ND, T>(geo, nupts, upt, e, s, rcp, true);

        T uu[NV];
#pragma unroll
        for (int v = 0; v < NV; v++) uu[v] = u[upt * ldu + soa_off(e, v, NV)];
        if (gas.shifted) {
            // q = T(u - u_ref): rho = rho_ref + q0, E = E_ref + qE + h_s q0
            uu[NV - 1] += gas.e_ref + gas.hs_ref * uu[0];
            uu[0] += gas.rho_ref;
#pragma unroll
            for (int d = 0; d < ND; d++) uu[d + 1] += gas.m_ref[d];
        }

        const T rho = uu[0], rcprho = T(1) / rho;
        T vel[ND], k2 = 0;
#pragma unroll
        for (int d = 0; d < ND; d++) {
            vel[d] = rcprho * uu[d + 1];
            k2 += uu[d + 1] * vel[d];
        }
        const T p = gas.gm1 * (uu[NV - 1] - T(0.5) * k2);
        const T csnd = sqrt(gas.gamma * p * rcprho);

        T lam = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            T vn = 0, nn = 0;
#pragma unroll
            for (int j = 0; j < ND; j++) {
                const T sij = s[i][j] * rcp;
                vn += sij * vel[j];
                nn += sij * sij;
            }
            lam += fabs(vn) + csnd * sqrt(nn);
        }
        lmax = fmax(lmax, lam);
    }
    wspd[e] = lmax;
}

template <int ND, typename T>
__global__ void __launch_bounds__(PW_BLOCK)
tflux_ns_kernel(int nupts, int64_t neles, b200::GasK<T> gas, const T *__restrict__ u, int64_t ldu,
                T *__restrict__ f, int64_t ldf, T *__restrict__ gradu, int64_t ldg,
                ElemGeom<T> geo, const T *__restrict__ av, int64_t lda, int gradwb) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    const int upt = blockIdx.y;
    if (e >= neles) return;

    // Fused form: the corrected reference gradient is in gradu and is
    // transformed here (and written back, unless gradwb is 0: then the
    // interface kernel transforms the face values); otherwise (flux
    // anti-aliasing) the physical gradient at the point is in f, which the
    // flux replaces
    const bool fused = gradu != nullptr;
    T s[ND][ND], rcp;
    elem_metrics<ND, T>(geo, nupts, upt, e, s, rcp, fused);

    T gr[ND][NV];
    if (fused) {
        T tg[ND][NV];
#pragma unroll
        for (int d = 0; d < ND; d++)
#pragma unroll
            for (int v = 0; v < NV; v++) tg[d][v] = gradu[(int64_t)(d * nupts + upt) * ldg + soa_off(e, v, NV)];
#pragma unroll
        for (int i = 0; i < ND; i++)
#pragma unroll
            for (int j = 0; j < NV; j++) {
                T acc = 0;
#pragma unroll
                for (int k = 0; k < ND; k++) acc += s[k][i] * tg[k][j];
                gr[i][j] = rcp * acc;
                if (gradwb) gradu[(int64_t)(i * nupts + upt) * ldg + soa_off(e, j, NV)] = gr[i][j];
            }
    } else {
#pragma unroll
        for (int d = 0; d < ND; d++)
#pragma unroll
            for (int v = 0; v < NV; v++) gr[d][v] = f[(int64_t)(d * nupts + upt) * ldf + soa_off(e, v, NV)];
    }

    T uu[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) uu[v] = u[upt * ldu + soa_off(e, v, NV)];

    T ft[ND][NV], p, vel[ND];
    if (gas.shifted) {
        T uf[NV], gu[ND][NV];
        b200::inviscid_flux_shift<ND, T>(uu, ft, p, vel, uf, gas);
        b200::unshift_grad<ND, T>(gr, gu, gas);
        b200::viscous_flux_add<ND, T>(uf, gu, ft, gas);
    } else {
        b200::inviscid_flux<ND, T>(uu, ft, p, vel, gas.gamma);
        b200::viscous_flux_add<ND, T>(uu, gr, ft, gas);
    }

    // Artificial viscosity (pyfr/solvers/baseadvecdiff/kernels/
    // artvisc.mako: F -= mu_av grad u)
    if (av) {
        const T a = av[(int64_t)upt * lda + e];
#pragma unroll
        for (int d = 0; d < ND; d++)
#pragma unroll
            for (int v = 0; v < NV; v++) ft[d][v] -= a * gr[d][v];
    }

#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int j = 0; j < NV; j++) {
            T acc = 0;
#pragma unroll
            for (int k = 0; k < ND; k++) acc += s[i][k] * ft[k][j];
            f[(int64_t)(i * nupts + upt) * ldf + soa_off(e, j, NV)] = acc;
        }
}

template <int ND, typename T>
__global__ void __launch_bounds__(PW_BLOCK)
gradcoru_kernel(int nupts, int64_t neles, T *__restrict__ gradu, int64_t ldg, ElemGeom<T> geo) {
    constexpr int NV = ND + 2;
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    const int upt = blockIdx.y;
    if (e >= neles) return;

    T s[ND][ND], rcp;
    elem_metrics<ND, T>(geo, nupts, upt, e, s, rcp, true);

    T tg[ND][NV];
#pragma unroll
    for (int d = 0; d < ND; d++)
#pragma unroll
        for (int v = 0; v < NV; v++) tg[d][v] = gradu[(int64_t)(d * nupts + upt) * ldg + soa_off(e, v, NV)];
#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int j = 0; j < NV; j++) {
            T acc = 0;
#pragma unroll
            for (int k = 0; k < ND; k++) acc += s[k][i] * tg[k][j];
            gradu[(int64_t)(i * nupts + upt) * ldg + soa_off(e, j, NV)] = rcp * acc;
        }
}

template <typename T>
__global__ void __launch_bounds__(PW_BLOCK)
negdivconf_kernel(int nvars, int64_t neles, T *__restrict__ r, int64_t ldr,
                  const T *__restrict__ rcpdjac, int64_t ldj) {
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    const int upt = blockIdx.y;
    if (e >= neles) return;
    const T rj = rcpdjac[(int64_t)upt * ldj + e];
    for (int v = 0; v < nvars; v++) {
        T *p = r + upt * ldr + soa_off(e, v, nvars);
        *p = -rj * *p;
    }
}

// Source terms at the solution points (b200_src_t in the kernels'
// precision)
constexpr int SRC_MAXV = 8;

template <typename T>
struct SrcK {
    const b200_bcop_t *prog;
    int estart[SRC_MAXV], elen[SRC_MAXV];
    const T *ploc;
    int64_t ldp;
    const T *u;
    int64_t ldu;
    T t;
    const double *t_dev;
};

// One thread per element of one solution point: the source of every
// variable, then (MODE) -R/|J| + src, R + src or src.  u may be R itself in
// the evaluation mode: every read of the point precedes its writes.
template <typename T, int MODE>
__global__ void __launch_bounds__(PW_BLOCK)
srcterms_kernel(int ndims, int nvars, int64_t neles, T *r, int64_t ldr,
                const T *__restrict__ rcpdjac, int64_t ldj, SrcK<T> s) {
    const int64_t e = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    const int upt = blockIdx.y;
    if (e >= neles) return;
    T x[3] = {0, 0, 0};
    if (s.ploc)
        for (int d = 0; d < ndims; d++) x[d] = s.ploc[upt * s.ldp + soa_off(e, d, ndims)];
    T u[SRC_MAXV];
    if (s.u)
        for (int v = 0; v < nvars; v++) u[v] = s.u[upt * s.ldu + soa_off(e, v, nvars)];
    const T t = s.t_dev ? (T)s.t_dev[0] : s.t;
    T src[SRC_MAXV];
    for (int v = 0; v < nvars; v++)
        src[v] = s.elen[v] ? b200::expr_program<T>(s.prog, s.estart[v], s.elen[v], x, t,
                                                    s.u ? u : nullptr, nvars)
                           : T(0);
    const T rj = MODE == B200_SRC_NEGDIVCONF ? rcpdjac[(int64_t)upt * ldj + e] : T(0);
    for (int v = 0; v < nvars; v++) {
        T *p = r + upt * ldr + soa_off(e, v, nvars);
        if (MODE == B200_SRC_NEGDIVCONF)
            *p = -rj * *p + src[v];
        else if (MODE == B200_SRC_ADD)
            *p += src[v];
        else
            *p = src[v];
    }
}

template <typename T>
int srcterms(int mode, int ndims, int nvars, int nupts, int64_t neles, T *r, int64_t ldr,
             const T *rcpdjac, int64_t ldj, const b200_src_t *src, cudaStream_t stream) {
    if (!src || nvars < 1 || nvars > SRC_MAXV || ndims < 1 || ndims > 3 || mode < 0 ||
        mode > 2 || (mode == B200_SRC_NEGDIVCONF && !rcpdjac))
        return B200_ERR_ARG;
    if (neles <= 0 || nupts <= 0) return B200_OK;
    SrcK<T> k;
    k.prog = src->prog;
    for (int v = 0; v < SRC_MAXV; v++) {
        k.estart[v] = src->expr_start[v];
        k.elen[v] = src->prog && v < nvars ? src->expr_len[v] : 0;
        if (k.elen[v] < 0 || k.estart[v] < 0) return B200_ERR_ARG;
    }
    k.ploc = static_cast<const T *>(src->ploc);
    k.ldp = src->ldp;
    k.u = static_cast<const T *>(src->u);
    k.ldu = src->ldu;
    k.t = (T)src->t;
    k.t_dev = src->t_dev;
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    if (mode == B200_SRC_NEGDIVCONF)
        srcterms_kernel<T, B200_SRC_NEGDIVCONF><<<grid, PW_BLOCK, 0, stream>>>(
            ndims, nvars, neles, r, ldr, rcpdjac, ldj, k);
    else if (mode == B200_SRC_ADD)
        srcterms_kernel<T, B200_SRC_ADD><<<grid, PW_BLOCK, 0, stream>>>(ndims, nvars, neles, r,
                                                                       ldr, rcpdjac, ldj, k);
    else
        srcterms_kernel<T, B200_SRC_EVAL><<<grid, PW_BLOCK, 0, stream>>>(ndims, nvars, neles, r,
                                                                        ldr, rcpdjac, ldj, k);
    B200_CHECK_LAUNCH("srcterms");
    return B200_OK;
}

// Pack a view into an AoSoA buffer: out[r*ldo + soa(i, c, ncol)] = the
// view's (r, c) value of point i (pyfr/backends/base/kernels/
// packing.mako:1-11, in this package's AoSoA exchange layout, which a view
// of identity map reads back directly).  One thread per point.
template <typename T>
__global__ void __launch_bounds__(PW_BLOCK)
pack_view_kernel(int64_t n, int nrow, int ncol, const T *__restrict__ base, const void *map,
                 const void *rstr, int ix64, T *__restrict__ out, int64_t ldo) {
    const int64_t i = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    if (i >= n) return;
    const T *p = base + b200::load_ix(map, ix64, i);
    const int64_t rs = rstr ? b200::load_ix(rstr, ix64, i) : 0;
    for (int r = 0; r < nrow; r++)
        for (int c = 0; c < ncol; c++)
            out[r * ldo + soa_off(i, c, ncol)] = p[r * rs + c * B200_SOASZ];
}

template <typename T>
int pack_view(int64_t n, int nrow, int ncol, const T *base, const void *map, const void *rstr,
              int ix64, T *out, int64_t ldo, cudaStream_t stream) {
    if (n <= 0) return B200_OK;
    if (!base || !map || !out || nrow < 1 || ncol < 1 || (nrow > 1 && !rstr) ||
        ldo < b200::ceil_div(n, B200_SOASZ) * (int64_t)B200_SOASZ * ncol)
        return b200::set_error(B200_ERR_ARG, "pack_view: bad arguments");
    pack_view_kernel<T><<<b200::ceil_div(n, PW_BLOCK), PW_BLOCK, 0, stream>>>(
        n, nrow, ncol, base, map, rstr, ix64, out, ldo);
    B200_CHECK_LAUNCH("pack_view");
    return B200_OK;
}

template <typename T>
struct ScalView {
    T *base;
    const void *map;
};

template <typename T>
struct VectView {
    const T *base;
    const void *map;
    const void *rstr;
};

// Unit normal and magnitude of pair i: stored (nl_unit: rows 0..ND-1 the
// unit normal, row ND its magnitude, formed once on the host as the
// reference forms them per call, mag = sqrt(n.n), n/mag = (1/mag) n) or
// formed here from the scaled normal
template <int ND, typename T>
__device__ __forceinline__ T pair_normal(const T *__restrict__ nl, int64_t ldn, int64_t i,
                                         int nl_unit, T nn[ND]) {
    if (nl_unit) {
#pragma unroll
        for (int d = 0; d < ND; d++) nn[d] = nl[d * ldn + i];
        return nl[ND * ldn + i];
    }
    T mag = 0;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        nn[d] = nl[d * ldn + i];
        mag += nn[d] * nn[d];
    }
    mag = sqrt(mag);
    const T inv = T(1) / mag;
#pragma unroll
    for (int d = 0; d < ND; d++) nn[d] = inv * nn[d];
    return mag;
}

template <int RS, int ND, typename T>
__global__ void __launch_bounds__(PW_BLOCK)
intcflux_euler_kernel(int64_t n, T gamma, T p_min, ScalView<T> vl, ScalView<T> vr, int ix64,
                      const T *__restrict__ nl, int64_t ldn, int nl_unit) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    if (i >= n) return;

    T *pl = vl.base + b200::load_ix(vl.map, ix64, i);
    T *pr = vr.base + b200::load_ix(vr.map, ix64, i);

    T ul[NV], ur[NV], nn[ND];
#pragma unroll
    for (int v = 0; v < NV; v++) {
        ul[v] = pl[v * B200_SOASZ];
        ur[v] = pr[v * B200_SOASZ];
    }
    const T mag = pair_normal<ND, T>(nl, ldn, i, nl_unit, nn);

    T fn[NV];
    b200::rsolve_t<RS, ND, T>(ul, ur, nn, fn, gamma, p_min);

#pragma unroll
    for (int v = 0; v < NV; v++) {
        pl[v * B200_SOASZ] = mag * fn[v];
        pr[v * B200_SOASZ] = -mag * fn[v];
    }
}

// Rusanov common flux on shifted inputs (the dissipation acts on
// differences of q, which are T times the differences of u)
template <int ND, typename T, bool MOVING>
__global__ void __launch_bounds__(PW_BLOCK)
intcflux_euler_shift_kernel(int64_t n, b200::GasK<T> gas, ScalView<T> vl, ScalView<T> vr,
                            int ix64, const T *__restrict__ nl, int64_t ldn, int nl_unit) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    if (i >= n) return;

    T *pl = vl.base + b200::load_ix(vl.map, ix64, i);
    T *pr = vr.base + b200::load_ix(vr.map, ix64, i);

    T ul[NV], ur[NV], nn[ND];
#pragma unroll
    for (int v = 0; v < NV; v++) {
        ul[v] = pl[v * B200_SOASZ];
        ur[v] = pr[v * B200_SOASZ];
    }
    const T mag = pair_normal<ND, T>(nl, ldn, i, nl_unit, nn);

    T fn[NV], ufl[NV], ufr[NV];
    b200::rsolve_rusanov_shift<ND, T, MOVING>(ul, ur, nn, fn, ufl, ufr, gas);

#pragma unroll
    for (int v = 0; v < NV; v++) {
        pl[v * B200_SOASZ] = mag * fn[v];
        pr[v * B200_SOASZ] = -mag * fn[v];
    }
}

// (FP32: 64 registers, so that eight blocks share an SM -- the kernel waits
// on its gathers, and occupancy hides them better than the spill-free 80
// registers do)
// Per-element metric terms of affine elements for the interface kernels
// that take face gradients in reference space (their elements' flux kernel
// left the solution-point gradient untransformed): rows i*ND + j hold
// S[i][j] and row ND*ND holds 1/|J| of element k in column k; il/ir give
// the column of each pair's left and right element.
template <typename T>
struct FaceMetrics {
    const T *m;
    int64_t ld;
    const int *il, *ir;
};

// grad <- (1/|J|) S^T grad at a face point of element column k
template <int ND, int NV, typename T>
__device__ __forceinline__ void face_grad_to_phys(const FaceMetrics<T> &fm, int k,
                                                  T gg[ND][NV]) {
    const T *m = fm.m + k;
    const T rcp = __ldg(m + (int64_t)(ND * ND) * fm.ld);
    // One output component at a time over every variable; the metric terms
    // are re-read rather than held (L1 hits: the pairs of one face share
    // their element), which keeps the kernel within its register bound
    T out[ND][NV];
#pragma unroll
    for (int i = 0; i < ND; i++) {
        T c[ND];
#pragma unroll
        for (int q = 0; q < ND; q++) c[q] = rcp * __ldg(m + (int64_t)(q * ND + i) * fm.ld);
#pragma unroll
        for (int v = 0; v < NV; v++) {
            T acc = 0;
#pragma unroll
            for (int q = 0; q < ND; q++) acc += c[q] * gg[q][v];
            out[i][v] = acc;
        }
    }
#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int v = 0; v < NV; v++) gg[i][v] = out[i][v];
}

template <int RS, int ND, typename T, bool FM>
__global__ void __launch_bounds__(PW_BLOCK, sizeof(T) == 4 ? 8 : 1)
intcflux_ns_kernel(int64_t n, b200::GasK<T> gas, T beta, T tau, ScalView<T> vl, ScalView<T> vr,
                   VectView<T> gl, VectView<T> gr, int ix64, const T *__restrict__ nl,
                   int64_t ldn, int nl_unit, ScalView<T> va, FaceMetrics<T> fm) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    if (i >= n) return;

    T *pl = vl.base + b200::load_ix(vl.map, ix64, i);
    T *pr = vr.base + b200::load_ix(vr.map, ix64, i);
    // (the element columns of the face metrics, loaded early)
    const int kl = FM && beta != T(-0.5) ? fm.il[i] : 0;
    const int kr = FM && beta != T(0.5) ? fm.ir[i] : 0;

    T ul[NV], ur[NV], nn[ND];
#pragma unroll
    for (int v = 0; v < NV; v++) {
        ul[v] = pl[v * B200_SOASZ];
        ur[v] = pr[v * B200_SOASZ];
    }
    const T mag = pair_normal<ND, T>(nl, ldn, i, nl_unit, nn);

    // Riemann flux; with a shifted input the viscous terms need the full
    // states, which the shifted flux reconstructs
    T fi[NV], ufl[NV], ufr[NV];
    if (RS == b200::RS_RUSANOV && gas.shifted) {
        b200::rsolve_rusanov_shift<ND, T>(ul, ur, nn, fi, ufl, ufr, gas);
    } else {
        b200::rsolve_t<RS, ND, T>(ul, ur, nn, fi, gas.gamma, gas.p_min);
#pragma unroll
        for (int v = 0; v < NV; v++) {
            ufl[v] = ul[v];
            ufr[v] = ur[v];
        }
    }

    // Artificial viscosity at the point (the left side's value)
    const T a = va.base ? va.base[b200::load_ix(va.map, ix64, i)] : T(0);

    // LDG viscous common flux from the left and/or right states, each
    // formed along the normal directly
    T nfl[NV], nfr[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) nfl[v] = nfr[v] = 0;

    if (beta != T(-0.5)) {
        const T *g = gl.base + b200::load_ix(gl.map, ix64, i);
        const int64_t rstr = b200::load_ix(gl.rstr, ix64, i);
        T gg[ND][NV];
#pragma unroll
        for (int d = 0; d < ND; d++)
#pragma unroll
            for (int v = 0; v < NV; v++) gg[d][v] = g[d * rstr + v * B200_SOASZ];
        if (FM) face_grad_to_phys<ND, NV, T>(fm, kl, gg);
        if (gas.shifted) {
            T gu[ND][NV];
            b200::unshift_grad<ND, T>(gg, gu, gas);
            b200::viscous_nflux_add<ND, T>(ufl, gu, nn, nfl, gas);
        } else {
            b200::viscous_nflux_add<ND, T>(ufl, gg, nn, nfl, gas);
            if (va.base) {
#pragma unroll
                for (int v = 0; v < NV; v++) {
                    T gn = 0;
#pragma unroll
                    for (int d = 0; d < ND; d++) gn += nn[d] * gg[d][v];
                    nfl[v] -= a * gn;
                }
            }
        }
    }
    if (beta != T(0.5)) {
        const T *g = gr.base + b200::load_ix(gr.map, ix64, i);
        const int64_t rstr = b200::load_ix(gr.rstr, ix64, i);
        T gg[ND][NV];
#pragma unroll
        for (int d = 0; d < ND; d++)
#pragma unroll
            for (int v = 0; v < NV; v++) gg[d][v] = g[d * rstr + v * B200_SOASZ];
        if (FM) face_grad_to_phys<ND, NV, T>(fm, kr, gg);
        if (gas.shifted) {
            T gu[ND][NV];
            b200::unshift_grad<ND, T>(gg, gu, gas);
            b200::viscous_nflux_add<ND, T>(ufr, gu, nn, nfr, gas);
        } else {
            b200::viscous_nflux_add<ND, T>(ufr, gg, nn, nfr, gas);
            if (va.base) {
#pragma unroll
                for (int v = 0; v < NV; v++) {
                    T gn = 0;
#pragma unroll
                    for (int d = 0; d < ND; d++) gn += nn[d] * gg[d][v];
                    nfr[v] -= a * gn;
                }
            }
        }
    }

#pragma unroll
    for (int v = 0; v < NV; v++) {
        T fvc;
        if (beta == T(-0.5))
            fvc = nfr[v];
        else if (beta == T(0.5))
            fvc = nfl[v];
        else
            fvc = (T(0.5) + beta) * nfl[v] + (T(0.5) - beta) * nfr[v];
        if (tau != T(0)) fvc += tau * (ul[v] - ur[v]);

        pl[v * B200_SOASZ] = mag * (fi[v] + fvc);
        pr[v * B200_SOASZ] = -mag * (fi[v] + fvc);
    }
}

template <typename T>
__global__ void __launch_bounds__(PW_BLOCK)
intconu_kernel(int64_t n, int nvars, T beta, ScalView<T> lin, ScalView<T> rin,
               ScalView<T> lout, ScalView<T> rout, int ix64, int both) {
    const int64_t i = (int64_t)blockIdx.x * PW_BLOCK + threadIdx.x;
    if (i >= n) return;

    const T *pli = lin.base + b200::load_ix(lin.map, ix64, i);
    const T *pri = rin.base + b200::load_ix(rin.map, ix64, i);
    T *plo = lout.base + b200::load_ix(lout.map, ix64, i);
    T *pro = rout.base + b200::load_ix(rout.map, ix64, i);

    // Every load before any store (the views may alias as far as the
    // compiler knows, so interleaving would serialise one round trip to
    // memory per variable)
    constexpr int NVMAX = 8;
    T c[NVMAX];
    if (beta == T(-0.5) || beta == T(0.5)) {
        const T *src = beta == T(-0.5) ? pli : pri;
        T *dst = beta == T(-0.5) ? pro : plo;
        T *other = beta == T(-0.5) ? plo : pro;
#pragma unroll
        for (int v = 0; v < NVMAX; v++)
            if (v < nvars) c[v] = src[v * B200_SOASZ];
#pragma unroll
        for (int v = 0; v < NVMAX; v++)
            if (v < nvars) {
                dst[v * B200_SOASZ] = c[v];
                if (both) other[v * B200_SOASZ] = c[v];
            }
    } else {
        T l[NVMAX];
#pragma unroll
        for (int v = 0; v < NVMAX; v++)
            if (v < nvars) {
                c[v] = pri[v * B200_SOASZ];
                l[v] = pli[v * B200_SOASZ];
            }
#pragma unroll
        for (int v = 0; v < NVMAX; v++)
            if (v < nvars) {
                const T x = c[v] * (T(0.5) + beta) + l[v] * (T(0.5) - beta);
                plo[v * B200_SOASZ] = x;
                pro[v * B200_SOASZ] = x;
            }
    }
}

template <typename T>
ElemGeom<T> make_geom(int linear, const T *smats, int64_t lds, const T *rcpdjac, int64_t ldr,
                      const T *verts, int64_t ldv, const T *upts, int64_t ldup) {
    ElemGeom<T> g;
    g.smats = smats; g.lds = lds;
    g.rcpdjac = rcpdjac; g.ldr = ldr;
    g.verts = verts; g.ldv = ldv;
    g.upts = upts; g.ldup = ldup;
    g.linear = linear;
    return g;
}

int check_geom(int linear, const void *smats, const void *rcpdjac, const void *verts,
               const void *upts, bool need_rcp) {
    if (linear < GEOM_STORED || linear > GEOM_PER_ELEMENT)
        return b200::set_error(B200_ERR_ARG, "unknown geometry mode %d", linear);
    if (linear == GEOM_VERTICES && (!verts || !upts))
        return b200::set_error(B200_ERR_ARG, "linear elements need verts and upts");
    if (linear != GEOM_VERTICES && (!smats || (need_rcp && !rcpdjac)))
        return b200::set_error(B200_ERR_ARG, "stored metrics need smats (and rcpdjac)");
    return B200_OK;
}

template <typename T>
int tflux_euler(int ndims, int nupts, int64_t neles, int linear, double gamma, const T *u,
                int64_t ldu, T *f, int64_t ldf, const T *smats, int64_t lds, const T *verts,
                int64_t ldv, const T *upts, int64_t ldup, cudaStream_t st) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    int rc = check_geom(linear, smats, nullptr, verts, upts, false);
    if (rc) return rc;
    auto geo = make_geom<T>(linear, smats, lds, nullptr, 0, verts, ldv, upts, ldup);
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    if (ndims == 2)
        tflux_euler_kernel<2, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, (T)gamma, u, ldu, f, ldf, geo);
    else if (ndims == 3)
        tflux_euler_kernel<3, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, (T)gamma, u, ldu, f, ldf, geo);
    else
        return b200::set_error(B200_ERR_ARG, "tflux: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("tflux_euler");
    return B200_OK;
}

template <typename T>
int wavespeed(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas, const T *u,
              int64_t ldu, const T *smats, int64_t lds, const T *rcpdjac, int64_t ldr,
              const T *verts, int64_t ldv, const T *upts, int64_t ldup, T *wspd,
              cudaStream_t st) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    if (!gas || !wspd) return b200::set_error(B200_ERR_ARG, "wavespeed: null argument");
    int rc = check_geom(linear, smats, rcpdjac, verts, upts, true);
    if (rc) return rc;
    auto geo = make_geom<T>(linear, smats, lds, rcpdjac, ldr, verts, ldv, upts, ldup);
    const auto g = b200::gas_consts<T>(*reinterpret_cast<const Gas *>(gas));
    const unsigned grid = (unsigned)b200::ceil_div(neles, PW_BLOCK);
    if (ndims == 2)
        wavespeed_kernel<2, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, geo, wspd);
    else if (ndims == 3)
        wavespeed_kernel<3, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, geo, wspd);
    else
        return b200::set_error(B200_ERR_ARG, "wavespeed: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("wavespeed");
    return B200_OK;
}

template <typename T>
int tflux_ns(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
             const T *u, int64_t ldu, T *f, int64_t ldf, T *gradu, int64_t ldg, const T *smats,
             int64_t lds, const T *rcpdjac, int64_t ldr, const T *verts, int64_t ldv,
             const T *upts, int64_t ldup, const T *av, int64_t lda, int gradwb, cudaStream_t st) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    if (!gas) return b200::set_error(B200_ERR_ARG, "tflux_ns: null gas constants");
    if (!gradwb && !gradu)
        return b200::set_error(B200_ERR_ARG, "tflux_ns: a reference gradient to leave needs gradu");
    if (av && reinterpret_cast<const Gas *>(gas)->shifted)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "tflux_ns: artificial viscosity takes unshifted states");
    int rc = check_geom(linear, smats, rcpdjac, verts, upts, gradu != nullptr);
    if (rc) return rc;
    auto geo = make_geom<T>(linear, smats, lds, rcpdjac, ldr, verts, ldv, upts, ldup);
    const auto g = b200::gas_consts<T>(*reinterpret_cast<const Gas *>(gas));
    if (g.moving)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "tflux_ns: the reference state must be at rest");
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    if (ndims == 2)
        tflux_ns_kernel<2, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, f, ldf, gradu, ldg, geo, av, lda, gradwb);
    else if (ndims == 3)
        tflux_ns_kernel<3, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, f, ldf, gradu, ldg, geo, av, lda, gradwb);
    else
        return b200::set_error(B200_ERR_ARG, "tflux_ns: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("tflux_ns");
    return B200_OK;
}

template <typename T>
int gradcoru(int ndims, int nupts, int64_t neles, int linear, T *gradu, int64_t ldg,
             const T *smats, int64_t lds, const T *rcpdjac, int64_t ldr, const T *verts,
             int64_t ldv, const T *upts, int64_t ldup, cudaStream_t st) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    int rc = check_geom(linear, smats, rcpdjac, verts, upts, true);
    if (rc) return rc;
    auto geo = make_geom<T>(linear, smats, lds, rcpdjac, ldr, verts, ldv, upts, ldup);
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    if (ndims == 2)
        gradcoru_kernel<2, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, gradu, ldg, geo);
    else if (ndims == 3)
        gradcoru_kernel<3, T><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, gradu, ldg, geo);
    else
        return b200::set_error(B200_ERR_ARG, "gradcoru: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("gradcoru");
    return B200_OK;
}

template <typename T>
int intcflux_euler(int ndims, int64_t n, int rsolver, double gamma, double p_min, T *ul_base,
                   const void *ul_map, T *ur_base, const void *ur_map, int ix64, const T *nl,
                   int64_t ldn, int nl_unit, cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (ndims != 2 && ndims != 3)
        return b200::set_error(B200_ERR_ARG, "intcflux: ndims must be 2 or 3");
    ScalView<T> l{ul_base, ul_map}, r{ur_base, ur_map};
    unsigned grid = b200::ceil_div(n, PW_BLOCK);
    const bool ok = b200::with_rsolver(rsolver, [&](auto rsc) {
        constexpr int RS = decltype(rsc)::value;
        if (ndims == 2)
            intcflux_euler_kernel<RS, 2, T><<<grid, PW_BLOCK, 0, st>>>(n, (T)gamma, (T)p_min, l, r, ix64, nl, ldn, nl_unit);
        else
            intcflux_euler_kernel<RS, 3, T><<<grid, PW_BLOCK, 0, st>>>(n, (T)gamma, (T)p_min, l, r, ix64, nl, ldn, nl_unit);
    });
    if (!ok) return b200::set_error(B200_ERR_ARG, "intcflux: unknown Riemann solver %d", rsolver);
    B200_CHECK_LAUNCH("intcflux_euler");
    return B200_OK;
}

template <typename T>
int tflux_euler_shift(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                      const T *u, int64_t ldu, T *f, int64_t ldf, const T *smats, int64_t lds,
                      const T *verts, int64_t ldv, const T *upts, int64_t ldup, cudaStream_t st) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    if (!gas) return b200::set_error(B200_ERR_ARG, "tflux_euler_shift: null gas constants");
    int rc = check_geom(linear, smats, nullptr, verts, upts, false);
    if (rc) return rc;
    auto geo = make_geom<T>(linear, smats, lds, nullptr, 0, verts, ldv, upts, ldup);
    const auto g = b200::gas_consts<T>(*reinterpret_cast<const Gas *>(gas));
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    if (ndims == 2 && g.moving)
        tflux_euler_shift_kernel<2, T, true><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, f, ldf, geo);
    else if (ndims == 2)
        tflux_euler_shift_kernel<2, T, false><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, f, ldf, geo);
    else if (ndims == 3 && g.moving)
        tflux_euler_shift_kernel<3, T, true><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, f, ldf, geo);
    else if (ndims == 3)
        tflux_euler_shift_kernel<3, T, false><<<grid, PW_BLOCK, 0, st>>>(nupts, neles, g, u, ldu, f, ldf, geo);
    else
        return b200::set_error(B200_ERR_ARG, "tflux: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("tflux_euler_shift");
    return B200_OK;
}

template <typename T>
int intcflux_euler_shift(int ndims, int64_t n, const b200_gas_t *gas, T *ul_base,
                         const void *ul_map, T *ur_base, const void *ur_map, int ix64,
                         const T *nl, int64_t ldn, int nl_unit, cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (!gas) return b200::set_error(B200_ERR_ARG, "intcflux_euler_shift: null gas constants");
    if (ndims != 2 && ndims != 3)
        return b200::set_error(B200_ERR_ARG, "intcflux: ndims must be 2 or 3");
    ScalView<T> l{ul_base, ul_map}, r{ur_base, ur_map};
    const auto g = b200::gas_consts<T>(*reinterpret_cast<const Gas *>(gas));
    unsigned grid = b200::ceil_div(n, PW_BLOCK);
    if (ndims == 2 && g.moving)
        intcflux_euler_shift_kernel<2, T, true><<<grid, PW_BLOCK, 0, st>>>(n, g, l, r, ix64, nl, ldn, nl_unit);
    else if (ndims == 2)
        intcflux_euler_shift_kernel<2, T, false><<<grid, PW_BLOCK, 0, st>>>(n, g, l, r, ix64, nl, ldn, nl_unit);
    else if (g.moving)
        intcflux_euler_shift_kernel<3, T, true><<<grid, PW_BLOCK, 0, st>>>(n, g, l, r, ix64, nl, ldn, nl_unit);
    else
        intcflux_euler_shift_kernel<3, T, false><<<grid, PW_BLOCK, 0, st>>>(n, g, l, r, ix64, nl, ldn, nl_unit);
    B200_CHECK_LAUNCH("intcflux_euler_shift");
    return B200_OK;
}

template <typename T>
int intcflux_ns(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double beta,
                double tau, T *ul_base, const void *ul_map, T *ur_base, const void *ur_map,
                const T *gl_base, const void *gl_map, const void *gl_rstr, const T *gr_base,
                const void *gr_map, const void *gr_rstr, int ix64, const T *nl, int64_t ldn,
                int nl_unit, const T *av_base, const void *av_map, FaceMetrics<T> fm,
                cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (!gas) return b200::set_error(B200_ERR_ARG, "intcflux_ns: null gas constants");
    if (fm.m && ((beta != -0.5 && !fm.il) || (beta != 0.5 && !fm.ir) || fm.ld <= 0))
        return b200::set_error(B200_ERR_ARG, "intcflux_ns: face metrics need the element columns");
    if (av_base && (!av_map || reinterpret_cast<const Gas *>(gas)->shifted))
        return b200::set_error(B200_ERR_ARG,
                               "intcflux_ns: artificial viscosity needs a view and unshifted states");
    ScalView<T> va{const_cast<T *>(av_base), av_map};
    ScalView<T> l{ul_base, ul_map}, r{ur_base, ur_map};
    VectView<T> gl{gl_base, gl_map, gl_rstr}, gr{gr_base, gr_map, gr_rstr};
    const auto g = b200::gas_consts<T>(*reinterpret_cast<const Gas *>(gas));
    if (g.shifted && rsolver != b200::RS_RUSANOV)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "intcflux_ns: shifted inputs need the Rusanov solver");
    if (g.moving)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "intcflux_ns: the reference state must be at rest");
    if (ndims != 2 && ndims != 3)
        return b200::set_error(B200_ERR_ARG, "intcflux_ns: ndims must be 2 or 3");
    unsigned grid = b200::ceil_div(n, PW_BLOCK);
    const bool ok = b200::with_rsolver(rsolver, [&](auto rsc) {
        constexpr int RS = decltype(rsc)::value;
        if (ndims == 2)
            intcflux_ns_kernel<RS, 2, T, false><<<grid, PW_BLOCK, 0, st>>>(n, g, (T)beta, (T)tau, l, r, gl, gr, ix64, nl, ldn, nl_unit, va, fm);
        else if (!fm.m)
            intcflux_ns_kernel<RS, 3, T, false><<<grid, PW_BLOCK, 0, st>>>(n, g, (T)beta, (T)tau, l, r, gl, gr, ix64, nl, ldn, nl_unit, va, fm);
        else
            intcflux_ns_kernel<RS, 3, T, true><<<grid, PW_BLOCK, 0, st>>>(n, g, (T)beta, (T)tau, l, r, gl, gr, ix64, nl, ldn, nl_unit, va, fm);
    });
    if (!ok) return b200::set_error(B200_ERR_ARG, "intcflux: unknown Riemann solver %d", rsolver);
    B200_CHECK_LAUNCH("intcflux_ns");
    return B200_OK;
}

template <typename T>
int intconu(int nvars, int64_t n, double beta, const T *lin_base, const void *lin_map,
            const T *rin_base, const void *rin_map, T *lout_base, const void *lout_map,
            T *rout_base, const void *rout_map, int ix64, int both, cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (nvars < 1 || nvars > 8) return b200::set_error(B200_ERR_ARG, "intconu: 1-8 variables");
    ScalView<T> li{const_cast<T *>(lin_base), lin_map};
    ScalView<T> ri{const_cast<T *>(rin_base), rin_map};
    ScalView<T> lo{lout_base, lout_map}, ro{rout_base, rout_map};
    intconu_kernel<T><<<b200::ceil_div(n, PW_BLOCK), PW_BLOCK, 0, st>>>(
        n, nvars, (T)beta, li, ri, lo, ro, ix64, both);
    B200_CHECK_LAUNCH("intconu");
    return B200_OK;
}

}  // namespace

extern "C" {

int b200_tflux_euler_f64(int ndims, int nupts, int64_t neles, int linear, double gamma,
                         const double *u, int64_t ldu, double *f, int64_t ldf,
                         const double *smats, int64_t lds, const double *verts, int64_t ldv,
                         const double *upts, int64_t ldup, void *stream) {
    return tflux_euler<double>(ndims, nupts, neles, linear, gamma, u, ldu, f, ldf, smats, lds,
                               verts, ldv, upts, ldup, (cudaStream_t)stream);
}

int b200_tflux_euler_f32(int ndims, int nupts, int64_t neles, int linear, double gamma,
                         const float *u, int64_t ldu, float *f, int64_t ldf,
                         const float *smats, int64_t lds, const float *verts, int64_t ldv,
                         const float *upts, int64_t ldup, void *stream) {
    return tflux_euler<float>(ndims, nupts, neles, linear, gamma, u, ldu, f, ldf, smats, lds,
                              verts, ldv, upts, ldup, (cudaStream_t)stream);
}

int b200_tflux_ns_f64(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                      const double *u, int64_t ldu, double *f, int64_t ldf, double *gradu,
                      int64_t ldg, const double *smats, int64_t lds, const double *rcpdjac,
                      int64_t ldr, const double *verts, int64_t ldv, const double *upts,
                      int64_t ldup, void *stream) {
    return tflux_ns<double>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, gradu, ldg, smats,
                            lds, rcpdjac, ldr, verts, ldv, upts, ldup, nullptr, 0, 1,
                            (cudaStream_t)stream);
}

int b200_tflux_ns_av_f64(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                         const double *u, int64_t ldu, double *f, int64_t ldf, double *gradu,
                         int64_t ldg, const double *smats, int64_t lds, const double *rcpdjac,
                         int64_t ldr, const double *verts, int64_t ldv, const double *upts,
                         int64_t ldup, const double *av, int64_t lda, void *stream) {
    if (!av) return b200::set_error(B200_ERR_ARG, "tflux_ns_av: null viscosity");
    return tflux_ns<double>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, gradu, ldg, smats,
                        lds, rcpdjac, ldr, verts, ldv, upts, ldup, av, lda, 1, (cudaStream_t)stream);
}

int b200_tflux_ns_f32(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                      const float *u, int64_t ldu, float *f, int64_t ldf, float *gradu,
                      int64_t ldg, const float *smats, int64_t lds, const float *rcpdjac,
                      int64_t ldr, const float *verts, int64_t ldv, const float *upts,
                      int64_t ldup, void *stream) {
    return tflux_ns<float>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, gradu, ldg, smats,
                           lds, rcpdjac, ldr, verts, ldv, upts, ldup, nullptr, 0, 1,
                            (cudaStream_t)stream);
}

int b200_tflux_ns_refgrad_f64(int ndims, int nupts, int64_t neles, int linear,
                              const b200_gas_t *gas, const double *u, int64_t ldu, double *f,
                              int64_t ldf, double *gradu, int64_t ldg, const double *smats,
                              int64_t lds, const double *rcpdjac, int64_t ldr,
                              const double *verts, int64_t ldv, const double *upts,
                              int64_t ldup, void *stream) {
    return tflux_ns<double>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, gradu, ldg, smats,
                            lds, rcpdjac, ldr, verts, ldv, upts, ldup, nullptr, 0, 0,
                            (cudaStream_t)stream);
}

int b200_tflux_ns_refgrad_f32(int ndims, int nupts, int64_t neles, int linear,
                              const b200_gas_t *gas, const float *u, int64_t ldu, float *f,
                              int64_t ldf, float *gradu, int64_t ldg, const float *smats,
                              int64_t lds, const float *rcpdjac, int64_t ldr, const float *verts,
                              int64_t ldv, const float *upts, int64_t ldup, void *stream) {
    return tflux_ns<float>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, gradu, ldg, smats,
                           lds, rcpdjac, ldr, verts, ldv, upts, ldup, nullptr, 0, 0,
                           (cudaStream_t)stream);
}

int b200_tflux_ns_av_f32(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                         const float *u, int64_t ldu, float *f, int64_t ldf, float *gradu,
                         int64_t ldg, const float *smats, int64_t lds, const float *rcpdjac,
                         int64_t ldr, const float *verts, int64_t ldv, const float *upts,
                         int64_t ldup, const float *av, int64_t lda, void *stream) {
    if (!av) return b200::set_error(B200_ERR_ARG, "tflux_ns_av: null viscosity");
    return tflux_ns<float>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, gradu, ldg, smats,
                        lds, rcpdjac, ldr, verts, ldv, upts, ldup, av, lda, 1, (cudaStream_t)stream);
}

int b200_gradcoru_f64(int ndims, int nupts, int64_t neles, int linear, double *gradu,
                      int64_t ldg, const double *smats, int64_t lds, const double *rcpdjac,
                      int64_t ldr, const double *verts, int64_t ldv, const double *upts,
                      int64_t ldup, void *stream) {
    return gradcoru<double>(ndims, nupts, neles, linear, gradu, ldg, smats, lds, rcpdjac, ldr,
                            verts, ldv, upts, ldup, (cudaStream_t)stream);
}

int b200_gradcoru_f32(int ndims, int nupts, int64_t neles, int linear, float *gradu,
                      int64_t ldg, const float *smats, int64_t lds, const float *rcpdjac,
                      int64_t ldr, const float *verts, int64_t ldv, const float *upts,
                      int64_t ldup, void *stream) {
    return gradcoru<float>(ndims, nupts, neles, linear, gradu, ldg, smats, lds, rcpdjac, ldr,
                           verts, ldv, upts, ldup, (cudaStream_t)stream);
}

int b200_negdivconf_f64(int nvars, int nupts, int64_t neles, double *r, int64_t ldr,
                        const double *rcpdjac, int64_t ldj, void *stream) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    negdivconf_kernel<double><<<grid, PW_BLOCK, 0, (cudaStream_t)stream>>>(nvars, neles, r, ldr, rcpdjac, ldj);
    B200_CHECK_LAUNCH("negdivconf");
    return B200_OK;
}

int b200_negdivconf_f32(int nvars, int nupts, int64_t neles, float *r, int64_t ldr,
                        const float *rcpdjac, int64_t ldj, void *stream) {
    if (neles <= 0 || nupts <= 0) return B200_OK;
    dim3 grid(b200::ceil_div(neles, PW_BLOCK), nupts);
    negdivconf_kernel<float><<<grid, PW_BLOCK, 0, (cudaStream_t)stream>>>(nvars, neles, r, ldr, rcpdjac, ldj);
    B200_CHECK_LAUNCH("negdivconf");
    return B200_OK;
}

int b200_pack_view_f64(int64_t n, int nrow, int ncol, const double *base, const void *map,
                       const void *rstr, int ix64, double *out, int64_t ldo, void *stream) {
    return pack_view<double>(n, nrow, ncol, base, map, rstr, ix64, out, ldo,
                             (cudaStream_t)stream);
}

int b200_pack_view_f32(int64_t n, int nrow, int ncol, const float *base, const void *map,
                       const void *rstr, int ix64, float *out, int64_t ldo, void *stream) {
    return pack_view<float>(n, nrow, ncol, base, map, rstr, ix64, out, ldo,
                            (cudaStream_t)stream);
}

int b200_srcterms_f64(int mode, int ndims, int nvars, int nupts, int64_t neles, double *r,
                      int64_t ldr, const double *rcpdjac, int64_t ldj, const b200_src_t *src,
                      void *stream) {
    return srcterms<double>(mode, ndims, nvars, nupts, neles, r, ldr, rcpdjac, ldj, src,
                            (cudaStream_t)stream);
}

int b200_srcterms_f32(int mode, int ndims, int nvars, int nupts, int64_t neles, float *r,
                      int64_t ldr, const float *rcpdjac, int64_t ldj, const b200_src_t *src,
                      void *stream) {
    return srcterms<float>(mode, ndims, nvars, nupts, neles, r, ldr, rcpdjac, ldj, src,
                           (cudaStream_t)stream);
}

int b200_intcflux_euler_f64(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                            double *ul_base,
                            const void *ul_map, double *ur_base, const void *ur_map, int ix64,
                            const double *nl, int64_t ldn, int nl_unit, void *stream) {
    return intcflux_euler<double>(ndims, n, rsolver, gamma, p_min, ul_base, ul_map, ur_base, ur_map,
                                  ix64, nl, ldn, nl_unit, (cudaStream_t)stream);
}

int b200_intcflux_euler_f32(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                            float *ul_base,
                            const void *ul_map, float *ur_base, const void *ur_map, int ix64,
                            const float *nl, int64_t ldn, int nl_unit, void *stream) {
    return intcflux_euler<float>(ndims, n, rsolver, gamma, p_min, ul_base, ul_map, ur_base, ur_map,
                                 ix64, nl, ldn, nl_unit, (cudaStream_t)stream);
}

int b200_tflux_euler_shift_f64(int ndims, int nupts, int64_t neles, int linear,
                               const b200_gas_t *gas, const double *u, int64_t ldu, double *f,
                               int64_t ldf, const double *smats, int64_t lds,
                               const double *verts, int64_t ldv, const double *upts,
                               int64_t ldup, void *stream) {
    return tflux_euler_shift<double>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, smats, lds,
                                     verts, ldv, upts, ldup, (cudaStream_t)stream);
}

int b200_tflux_euler_shift_f32(int ndims, int nupts, int64_t neles, int linear,
                               const b200_gas_t *gas, const float *u, int64_t ldu, float *f,
                               int64_t ldf, const float *smats, int64_t lds, const float *verts,
                               int64_t ldv, const float *upts, int64_t ldup, void *stream) {
    return tflux_euler_shift<float>(ndims, nupts, neles, linear, gas, u, ldu, f, ldf, smats, lds,
                                    verts, ldv, upts, ldup, (cudaStream_t)stream);
}

int b200_intcflux_euler_shift_f64(int ndims, int64_t n, const b200_gas_t *gas, double *ul_base,
                                  const void *ul_map, double *ur_base, const void *ur_map,
                                  int ix64, const double *nl, int64_t ldn, int nl_unit,
                                  void *stream) {
    return intcflux_euler_shift<double>(ndims, n, gas, ul_base, ul_map, ur_base, ur_map, ix64,
                                        nl, ldn, nl_unit, (cudaStream_t)stream);
}

int b200_intcflux_euler_shift_f32(int ndims, int64_t n, const b200_gas_t *gas, float *ul_base,
                                  const void *ul_map, float *ur_base, const void *ur_map,
                                  int ix64, const float *nl, int64_t ldn, int nl_unit,
                                  void *stream) {
    return intcflux_euler_shift<float>(ndims, n, gas, ul_base, ul_map, ur_base, ur_map, ix64, nl,
                                       ldn, nl_unit, (cudaStream_t)stream);
}

int b200_intcflux_ns_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double beta,
                         double tau, double *ul_base, const void *ul_map, double *ur_base,
                         const void *ur_map, const double *gl_base, const void *gl_map,
                         const void *gl_rstr, const double *gr_base, const void *gr_map,
                         const void *gr_rstr, int ix64, const double *nl, int64_t ldn, int nl_unit,
                         void *stream) {
    return intcflux_ns<double>(ndims, n, rsolver, gas, beta, tau, ul_base, ul_map, ur_base,
                               ur_map, gl_base, gl_map, gl_rstr, gr_base, gr_map, gr_rstr, ix64,
                               nl, ldn, nl_unit, nullptr, nullptr, FaceMetrics<double>{},
                               (cudaStream_t)stream);
}

int b200_intcflux_ns_av_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                            double beta, double tau, double *ul_base, const void *ul_map,
                            double *ur_base, const void *ur_map, const double *gl_base,
                            const void *gl_map, const void *gl_rstr, const double *gr_base,
                            const void *gr_map, const void *gr_rstr, int ix64, const double *nl,
                            int64_t ldn, int nl_unit, const double *av_base, const void *av_map, void *stream) {
    if (!av_base) return b200::set_error(B200_ERR_ARG, "intcflux_ns_av: null viscosity");
    return intcflux_ns<double>(ndims, n, rsolver, gas, beta, tau, ul_base, ul_map, ur_base, ur_map,
                           gl_base, gl_map, gl_rstr, gr_base, gr_map, gr_rstr, ix64, nl, ldn, nl_unit,
                           av_base, av_map, FaceMetrics<double>{}, (cudaStream_t)stream);
}

int b200_intcflux_ns_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double beta,
                         double tau, float *ul_base, const void *ul_map, float *ur_base,
                         const void *ur_map, const float *gl_base, const void *gl_map,
                         const void *gl_rstr, const float *gr_base, const void *gr_map,
                         const void *gr_rstr, int ix64, const float *nl, int64_t ldn, int nl_unit,
                         void *stream) {
    return intcflux_ns<float>(ndims, n, rsolver, gas, beta, tau, ul_base, ul_map, ur_base,
                              ur_map, gl_base, gl_map, gl_rstr, gr_base, gr_map, gr_rstr, ix64,
                              nl, ldn, nl_unit, nullptr, nullptr, FaceMetrics<float>{},
                              (cudaStream_t)stream);
}

int b200_intcflux_ns_refgrad_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                                 double beta, double tau, double *ul_base, const void *ul_map,
                                 double *ur_base, const void *ur_map, const double *gl_base,
                                 const void *gl_map, const void *gl_rstr, const double *gr_base,
                                 const void *gr_map, const void *gr_rstr, int ix64,
                                 const double *nl, int64_t ldn, int nl_unit, const double *emet,
                                 int64_t ldm, const int *eidx_l, const int *eidx_r, void *stream) {
    if (!emet) return b200::set_error(B200_ERR_ARG, "intcflux_ns_refgrad: null metrics");
    return intcflux_ns<double>(ndims, n, rsolver, gas, beta, tau, ul_base, ul_map, ur_base, ur_map,
                               gl_base, gl_map, gl_rstr, gr_base, gr_map, gr_rstr, ix64, nl, ldn,
                               nl_unit, nullptr, nullptr,
                               FaceMetrics<double>{emet, ldm, eidx_l, eidx_r},
                               (cudaStream_t)stream);
}

int b200_intcflux_ns_refgrad_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                                 double beta, double tau, float *ul_base, const void *ul_map,
                                 float *ur_base, const void *ur_map, const float *gl_base,
                                 const void *gl_map, const void *gl_rstr, const float *gr_base,
                                 const void *gr_map, const void *gr_rstr, int ix64,
                                 const float *nl, int64_t ldn, int nl_unit, const float *emet,
                                 int64_t ldm, const int *eidx_l, const int *eidx_r, void *stream) {
    if (!emet) return b200::set_error(B200_ERR_ARG, "intcflux_ns_refgrad: null metrics");
    return intcflux_ns<float>(ndims, n, rsolver, gas, beta, tau, ul_base, ul_map, ur_base, ur_map,
                              gl_base, gl_map, gl_rstr, gr_base, gr_map, gr_rstr, ix64, nl, ldn,
                              nl_unit, nullptr, nullptr,
                              FaceMetrics<float>{emet, ldm, eidx_l, eidx_r},
                              (cudaStream_t)stream);
}

int b200_intcflux_ns_av_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                            double beta, double tau, float *ul_base, const void *ul_map,
                            float *ur_base, const void *ur_map, const float *gl_base,
                            const void *gl_map, const void *gl_rstr, const float *gr_base,
                            const void *gr_map, const void *gr_rstr, int ix64, const float *nl,
                            int64_t ldn, int nl_unit, const float *av_base, const void *av_map, void *stream) {
    if (!av_base) return b200::set_error(B200_ERR_ARG, "intcflux_ns_av: null viscosity");
    return intcflux_ns<float>(ndims, n, rsolver, gas, beta, tau, ul_base, ul_map, ur_base, ur_map,
                           gl_base, gl_map, gl_rstr, gr_base, gr_map, gr_rstr, ix64, nl, ldn, nl_unit,
                           av_base, av_map, FaceMetrics<float>{}, (cudaStream_t)stream);
}

int b200_intconu_f64(int nvars, int64_t n, double beta, const double *lin_base,
                     const void *lin_map, const double *rin_base, const void *rin_map,
                     double *lout_base, const void *lout_map, double *rout_base,
                     const void *rout_map, int ix64, void *stream) {
    return intconu<double>(nvars, n, beta, lin_base, lin_map, rin_base, rin_map, lout_base,
                           lout_map, rout_base, rout_map, ix64, 0, (cudaStream_t)stream);
}

int b200_intconu_f32(int nvars, int64_t n, double beta, const float *lin_base,
                     const void *lin_map, const float *rin_base, const void *rin_map,
                     float *lout_base, const void *lout_map, float *rout_base,
                     const void *rout_map, int ix64, void *stream) {
    return intconu<float>(nvars, n, beta, lin_base, lin_map, rin_base, rin_map, lout_base,
                          lout_map, rout_base, rout_map, ix64, 0, (cudaStream_t)stream);
}

int b200_intconu_both_f64(int nvars, int64_t n, double beta, const double *lin_base,
                          const void *lin_map, const double *rin_base, const void *rin_map,
                          double *lout_base, const void *lout_map, double *rout_base,
                          const void *rout_map, int ix64, void *stream) {
    return intconu<double>(nvars, n, beta, lin_base, lin_map, rin_base, rin_map, lout_base,
                           lout_map, rout_base, rout_map, ix64, 1, (cudaStream_t)stream);
}

int b200_intconu_both_f32(int nvars, int64_t n, double beta, const float *lin_base,
                          const void *lin_map, const float *rin_base, const void *rin_map,
                          float *lout_base, const void *lout_map, float *rout_base,
                          const void *rout_map, int ix64, void *stream) {
    return intconu<float>(nvars, n, beta, lin_base, lin_map, rin_base, rin_map, lout_base,
                          lout_map, rout_base, rout_map, ix64, 1, (cudaStream_t)stream);
}

int b200_wavespeed_f64(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                       const double *u, int64_t ldu, const double *smats, int64_t lds,
                       const double *rcpdjac, int64_t ldr, const double *verts, int64_t ldv,
                       const double *upts, int64_t ldup, double *wspd, void *stream) {
    return wavespeed<double>(ndims, nupts, neles, linear, gas, u, ldu, smats, lds, rcpdjac, ldr,
                             verts, ldv, upts, ldup, wspd, (cudaStream_t)stream);
}

int b200_wavespeed_f32(int ndims, int nupts, int64_t neles, int linear, const b200_gas_t *gas,
                       const float *u, int64_t ldu, const float *smats, int64_t lds,
                       const float *rcpdjac, int64_t ldr, const float *verts, int64_t ldv,
                       const float *upts, int64_t ldup, float *wspd, void *stream) {
    return wavespeed<float>(ndims, nupts, neles, linear, gas, u, ldu, smats, lds, rcpdjac, ldr,
                            verts, ldv, upts, ldup, wspd, (cudaStream_t)stream);
}

}  // extern "C"
