// Boundary-condition interface kernels: the common normal flux at a
// boundary face point (Euler and Navier-Stokes) and the LDG common solution
// there (Navier-Stokes), from the interior state and a boundary ghost state.
//
//   bccflux (Euler)   pyfr/solvers/euler/kernels/bccflux.mako:7-26
//   bcconu            pyfr/solvers/navstokes/kernels/bcconu.mako:6-14
//   bccflux (NS)      pyfr/solvers/navstokes/kernels/bccflux.mako:10-20
//   ghost states      pyfr/solvers/euler/kernels/bcs/{sup-in-fa,sup-out-fn,
//                     slp-adia-wall,char-riem-inv}.mako,
//                     pyfr/solvers/navstokes/kernels/bcs/{no-slp-adia-wall,
//                     no-slp-isot-wall,slp-adia-wall,sub-in-frv,
//                     sub-in-ftpttang,sub-out-fp,common,ghost,
//                     ghost-imperm}.mako
//
// A boundary value is a constant or a postfix program of the point's
// coordinates and the time (compiled on the host, pyfr_gb300/bcexpr.py),
// evaluated by each thread for its point before the ghost state is formed.
// One thread per boundary flux point; the interior state is read through a
// view (element offsets into the flux-point field) and the flux written
// back in place.
#include <cstdint>

#include "common.cuh"
#include "exprprog.cuh"
#include "physics.cuh"
#include "pyfrb200.h"

namespace {

constexpr int BC_BLOCK = 128;

using b200::Gas;

template <typename T>
struct BcK {
    int type;
    T rho, p, u[3], cpTw_g;        // cpTw_g = cpTw / gamma
    // char-riem-inv: free-stream sound speed, entropy, 2 cs/(gamma - 1)
    T cs, s, ratio;
    // sub-in-ftpttang: cpTt, pt^-Rdcp, Rdcp = (gamma - 1)/gamma, direction
    T cpTt, ptfac, rdcp, vc[3];
    // Expressions: programs of rho, p, u, v, w, cpTw (length 0: constant)
    const b200_bcop_t *prog;
    int estart[6], elen[6], nexpr;
    const T *ploc;
    int64_t ldp;
    const double *t_dev;
    T t;
    // Controlled pressure p = ic + im*t (type B200_BC_CHAR_RIEM_INV_CTRL)
    T ic, im;
    const double *ctrl;
    // Values to form per point: programs or the controlled pressure
    int perpt;
};

// The boundary values at point i: the programs evaluated and the derived
// constants formed again from them
template <int ND, typename T>
__device__ __forceinline__ void bc_at_point(BcK<T> &b, int64_t i, T gamma) {
    T x[3] = {0, 0, 0};
    if (b.ploc)
#pragma unroll
        for (int d = 0; d < ND; d++) x[d] = b.ploc[d * b.ldp + i];
    const T t = b.t_dev ? (T)b.t_dev[0] : b.t;
    T *dst[6] = {&b.rho, &b.p, &b.u[0], &b.u[1], &b.u[2], &b.cpTw_g};
    for (int f = 0; f < 6; f++)
        if (b.elen[f]) *dst[f] = b200::expr_program<T>(b.prog, b.estart[f], b.elen[f], x, t);
    if (b.elen[5]) b.cpTw_g /= gamma;
    const bool ctrl = b.type == B200_BC_CHAR_RIEM_INV_CTRL;
    if (ctrl)
        b.p = b.ctrl ? (T)(b.ctrl[0] + b.ctrl[1] * (double)t) : b.ic + b.im * t;
    if (ctrl || b.elen[0] || b.elen[1]) {
        const T cs = b.rho > 0 && b.p > 0 ? sqrt(gamma * b.p / b.rho) : T(0);
        b.cs = cs;
        b.s = b.rho > 0 ? b.p * pow(b.rho, -gamma) : T(0);
        b.ratio = cs * T(2) / (gamma - T(1));
    }
}

template <typename T>
BcK<T> bc_consts(const b200_bc_t &b, double gamma) {
    BcK<T> k;
    k.type = b.type;
    k.rho = (T)b.rho;
    k.p = (T)b.p;
    for (int i = 0; i < 3; i++) k.u[i] = (T)b.u[i];
    k.cpTw_g = (T)(b.cpTw / gamma);
    const double cs = b.rho > 0 && b.p > 0 ? sqrt(gamma * b.p / b.rho) : 0.0;
    k.cs = (T)cs;
    k.s = (T)(b.rho > 0 ? b.p * pow(b.rho, -gamma) : 0.0);
    k.ratio = (T)(cs * 2.0 / (gamma - 1.0));
    const double rdcp = (gamma - 1.0) / gamma;
    k.cpTt = (T)b.cpTt;
    k.ptfac = (T)(b.pt > 0 ? pow(b.pt, -rdcp) : 0.0);
    k.rdcp = (T)rdcp;
    for (int i = 0; i < 3; i++) k.vc[i] = (T)b.vc[i];
    k.prog = b.prog;
    k.nexpr = 0;
    for (int f = 0; f < 6; f++) {
        k.estart[f] = b.expr_start[f];
        k.elen[f] = b.prog ? b.expr_len[f] : 0;
        k.nexpr += k.elen[f] > 0;
    }
    k.ploc = static_cast<const T *>(b.ploc);
    k.ldp = b.ldp;
    k.t_dev = b.t_dev;
    k.t = (T)b.t;
    k.ic = (T)b.ic;
    k.im = (T)b.im;
    k.ctrl = b.ctrl;
    k.perpt = k.nexpr > 0 || b.type == B200_BC_CHAR_RIEM_INV_CTRL;
    return k;
}

// Programs need the point coordinates
template <typename T>
bool bc_exprs_ok(const BcK<T> &k) {
    return !k.nexpr || k.ploc;
}

// Ghost state of the Riemann solve (bc_rsolve_state)
template <int ND, typename T>
__device__ __forceinline__ void bc_rsolve_state(const BcK<T> &bc, T gamma, const T *ul,
                                                const T *n, T *ur) {
    constexpr int NV = ND + 2;
    const T gm1 = gamma - T(1);
    switch (bc.type) {
    case B200_BC_SUP_IN_FA: {
        // Prescribed free-stream state
        ur[0] = bc.rho;
        T k2 = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            ur[i + 1] = bc.rho * bc.u[i];
            k2 += ur[i + 1] * ur[i + 1];
        }
        ur[NV - 1] = bc.p / gm1 + T(0.5) * (T(1) / ur[0]) * k2;
        break;
    }
    case B200_BC_SLP_ADIA_WALL: {
        // Momentum mirrored in the wall
        T nor = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) nor += ul[i + 1] * n[i];
        ur[0] = ul[0];
#pragma unroll
        for (int i = 0; i < ND; i++) ur[i + 1] = ul[i + 1] - 2 * nor * n[i];
        ur[NV - 1] = ul[NV - 1];
        break;
    }
    case B200_BC_CHAR_RIEM_INV:
    case B200_BC_CHAR_RIEM_INV_CTRL: {
        // Riemann invariants of the free stream and of the interior
        const T inv = T(1) / ul[0];
        T ve = 0, vi = 0, k2 = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            ve += bc.u[i] * n[i];
            vi += ul[i + 1] * n[i];
            k2 += ul[i + 1] * ul[i + 1];
        }
        vi *= inv;
        const T pi = gm1 * ul[NV - 1] - T(0.5) * gm1 * inv * k2;
        const T ci = sqrt(gamma * pi * inv);
        const T twogm1 = T(2) / gm1;
        const bool super = fabs(ve) >= bc.cs;
        const T re = super && vi >= 0 ? vi - ci * twogm1 : ve - bc.ratio;
        const T ri = super && vi < 0 ? ve + bc.ratio : vi + ci * twogm1;
        const T vb = T(0.5) * (re + ri);
        const T cb = T(0.25) * gm1 * (ri - re);
        const T rhob = vi < 0 ? pow((T(1) / (gamma * bc.s)) * cb * cb, T(1) / gm1)
                              : ul[0] * pow(ul[0] * cb * cb / (gamma * pi), T(1) / gm1);
        const T pb = (T(1) / gamma) * rhob * cb * cb;
        ur[0] = rhob;
        T kb = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            ur[i + 1] = vi >= 0 ? rhob * (ul[i + 1] * inv + (vb - vi) * n[i])
                                : rhob * (bc.u[i] + (vb - ve) * n[i]);
            kb += ur[i + 1] * ur[i + 1];
        }
        ur[NV - 1] = pb * (T(1) / gm1) + T(0.5) * (T(1) / ur[0]) * kb;
        break;
    }
    case B200_BC_NO_SLP_ADIA_WALL:
        // Momentum reversed
        ur[0] = ul[0];
#pragma unroll
        for (int i = 0; i < ND; i++) ur[i + 1] = -ul[i + 1];
        ur[NV - 1] = ul[NV - 1];
        break;
    case B200_BC_NO_SLP_ISOT_WALL: {
        // Wall velocity and temperature imposed
        ur[0] = ul[0];
        T k2 = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            ur[i + 1] = -ul[i + 1] + 2 * bc.u[i] * ul[0];
            k2 += ur[i + 1] * ur[i + 1];
        }
        ur[NV - 1] = bc.cpTw_g * ur[0] + T(0.5) * (T(1) / ur[0]) * k2;
        break;
    }
    case B200_BC_SUB_IN_FRV: {
        // Given density and velocity, the interior internal energy
        T kl = 0, kr = 0;
        ur[0] = bc.rho;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            ur[i + 1] = bc.rho * bc.u[i];
            kl += ul[i + 1] * ul[i + 1];
            kr += ur[i + 1] * ur[i + 1];
        }
        ur[NV - 1] = ul[NV - 1] - T(0.5) * (T(1) / ul[0]) * kl + T(0.5) * (T(1) / ur[0]) * kr;
        break;
    }
    case B200_BC_SUB_IN_FTPTTANG: {
        // Total enthalpy and pressure with the interior static pressure
        T kl = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) kl += ul[i + 1] * ul[i + 1];
        const T pl = gm1 * (ul[NV - 1] - (T(0.5) / ul[0]) * kl);
        T udotu = T(2) * bc.cpTt * (T(1) - bc.ptfac * pow(pl, bc.rdcp));
        udotu = fmax(T(0), udotu);
        ur[0] = (T(1) / bc.rdcp) * pl / (bc.cpTt - T(0.5) * udotu);
        const T speed = sqrt(udotu);
#pragma unroll
        for (int i = 0; i < ND; i++) ur[i + 1] = bc.vc[i] * ur[0] * speed;
        ur[NV - 1] = (T(1) / gm1) * pl + T(0.5) * ur[0] * udotu;
        break;
    }
    case B200_BC_SUB_OUT_FP: {
        // Given pressure, the interior density and momentum
        T kl = 0;
#pragma unroll
        for (int v = 0; v < NV - 1; v++) ur[v] = ul[v];
#pragma unroll
        for (int i = 0; i < ND; i++) kl += ul[i + 1] * ul[i + 1];
        ur[NV - 1] = bc.p / gm1 + T(0.5) * (T(1) / ul[0]) * kl;
        break;
    }
    default:  // B200_BC_SUP_OUT_FN: the interior state
#pragma unroll
        for (int v = 0; v < NV; v++) ur[v] = ul[v];
    }
}

// Boundary state of the LDG common solution (bc_ldg_state)
template <int ND, typename T>
__device__ __forceinline__ void bc_ldg_state(const BcK<T> &bc, T gamma, const T *ul,
                                             const T *n, T *ur) {
    constexpr int NV = ND + 2;
    if (bc.type == B200_BC_NO_SLP_ADIA_WALL) {
        // Zero velocity, the interior internal energy
        T k2 = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) k2 += ul[i + 1] * ul[i + 1];
        ur[0] = ul[0];
#pragma unroll
        for (int i = 0; i < ND; i++) ur[i + 1] = 0;
        ur[NV - 1] = ul[NV - 1] - (T(0.5) / ul[0]) * k2;
    } else if (bc.type == B200_BC_NO_SLP_ISOT_WALL) {
        ur[0] = ul[0];
        T k2 = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            ur[i + 1] = bc.u[i] * ul[0];
            k2 += ur[i + 1] * ur[i + 1];
        }
        ur[NV - 1] = bc.cpTw_g * ur[0] + T(0.5) * (T(1) / ur[0]) * k2;
    } else {
        bc_rsolve_state<ND, T>(bc, gamma, ul, n, ur);
    }
}

// Boundary gradient state (bc_ldg_grad_state): zero for prescribed inflow
// states, the interior gradient otherwise; at an adiabatic no-slip wall the
// normal temperature gradient is removed.  us is the state the reference
// passes as the macro's first argument (ghost: the interior state;
// ghost-imperm: the LDG boundary state).
template <int ND, typename T>
__device__ __forceinline__ void bc_ldg_grad_state(const BcK<T> &bc, const T *us, const T *n,
                                                  const T gl[ND][ND + 2], T gr[ND][ND + 2]) {
    constexpr int NV = ND + 2;
    const bool zero = bc.type == B200_BC_SUP_IN_FA || bc.type == B200_BC_CHAR_RIEM_INV ||
                      bc.type == B200_BC_CHAR_RIEM_INV_CTRL || bc.type == B200_BC_SUB_IN_FRV ||
                      bc.type == B200_BC_SUB_OUT_FP;
#pragma unroll
    for (int d = 0; d < ND; d++)
#pragma unroll
        for (int v = 0; v < NV; v++) gr[d][v] = zero ? T(0) : gl[d][v];

    if (bc.type == B200_BC_NO_SLP_ADIA_WALL) {
        const T rcprho = T(1) / us[0];
        T vel[ND];
#pragma unroll
        for (int i = 0; i < ND; i++) vel[i] = rcprho * us[i + 1];
        // c_v rho dT/dx_d of the interior
        T tl[ND];
#pragma unroll
        for (int d = 0; d < ND; d++) {
            T kd = 0;
#pragma unroll
            for (int i = 0; i < ND; i++) kd += vel[i] * (gl[d][i + 1] - vel[i] * gl[d][0]);
            tl[d] = gl[d][NV - 1] - (rcprho * gl[d][0] * us[NV - 1] + kd);
        }
#pragma unroll
        for (int d = 0; d < ND; d++) {
            T c = 0;
#pragma unroll
            for (int e = 0; e < ND; e++) c += n[d] * n[e] * tl[e];
            gr[d][NV - 1] -= c;
        }
    }
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

template <int ND, typename T>
__device__ __forceinline__ T unit_normal(const T *__restrict__ nl, int64_t ldn, int64_t i,
                                         T nn[ND]) {
    T mag = 0;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        nn[d] = nl[d * ldn + i];
        mag += nn[d] * nn[d];
    }
    mag = sqrt(mag);
    const T inv = T(1) / mag;
#pragma unroll
    for (int d = 0; d < ND; d++) nn[d] *= inv;
    return mag;
}

template <int RS, int ND, typename T>
__global__ void __launch_bounds__(BC_BLOCK)
bccflux_euler_kernel(int64_t n, T gamma, T p_min, BcK<T> bc0, ScalView<T> vl, int ix64,
                     const T *__restrict__ nl, int64_t ldn) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * BC_BLOCK + threadIdx.x;
    if (i >= n) return;
    BcK<T> bc = bc0;
    if (bc.perpt) bc_at_point<ND, T>(bc, i, gamma);
    T *pl = vl.base + b200::load_ix(vl.map, ix64, i);
    T ul[NV], ur[NV], nn[ND], fn[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) ul[v] = pl[v * B200_SOASZ];
    const T mag = unit_normal<ND, T>(nl, ldn, i, nn);
    bc_rsolve_state<ND, T>(bc, gamma, ul, nn, ur);
    b200::rsolve_t<RS, ND, T>(ul, ur, nn, fn, gamma, p_min);
#pragma unroll
    for (int v = 0; v < NV; v++) pl[v * B200_SOASZ] = mag * fn[v];
}

template <int ND, typename T>
__global__ void __launch_bounds__(BC_BLOCK)
bcconu_kernel(int64_t n, T gamma, BcK<T> bc0, ScalView<T> vin, ScalView<T> vout, int ix64,
              const T *__restrict__ nl, int64_t ldn) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * BC_BLOCK + threadIdx.x;
    if (i >= n) return;
    BcK<T> bc = bc0;
    if (bc.perpt) bc_at_point<ND, T>(bc, i, gamma);
    const T *pi = vin.base + b200::load_ix(vin.map, ix64, i);
    T *po = vout.base + b200::load_ix(vout.map, ix64, i);
    T ul[NV], ur[NV], nn[ND];
#pragma unroll
    for (int v = 0; v < NV; v++) ul[v] = pi[v * B200_SOASZ];
    unit_normal<ND, T>(nl, ldn, i, nn);
    bc_ldg_state<ND, T>(bc, gamma, ul, nn, ur);
#pragma unroll
    for (int v = 0; v < NV; v++) po[v * B200_SOASZ] = ur[v];
}

template <int RS, int ND, typename T>
__global__ void __launch_bounds__(BC_BLOCK)
bccflux_ns_kernel(int64_t n, b200::GasK<T> gas, T tau, BcK<T> bc0, ScalView<T> vl,
                  VectView<T> gl, int ix64, const T *__restrict__ nl, int64_t ldn,
                  ScalView<T> va) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * BC_BLOCK + threadIdx.x;
    if (i >= n) return;
    BcK<T> bc = bc0;
    if (bc.perpt) bc_at_point<ND, T>(bc, i, gas.gamma);
    T *pl = vl.base + b200::load_ix(vl.map, ix64, i);
    T ul[NV], ur[NV], nn[ND], fi[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) ul[v] = pl[v * B200_SOASZ];
    const T mag = unit_normal<ND, T>(nl, ldn, i, nn);

    // Viscous part: none at a slip wall; otherwise the flux of the LDG
    // boundary state and gradient ('ghost' or 'ghost-imperm' state)
    T fvr[ND][NV];
#pragma unroll
    for (int d = 0; d < ND; d++)
#pragma unroll
        for (int v = 0; v < NV; v++) fvr[d][v] = 0;
    const bool slip = bc.type == B200_BC_SLP_ADIA_WALL;
    const bool imperm = bc.type == B200_BC_NO_SLP_ADIA_WALL ||
                        bc.type == B200_BC_NO_SLP_ISOT_WALL;
    if (!slip) {
        const T *g = gl.base + b200::load_ix(gl.map, ix64, i);
        const int64_t rstr = b200::load_ix(gl.rstr, ix64, i);
        T gg[ND][NV], gr[ND][NV];
#pragma unroll
        for (int d = 0; d < ND; d++)
#pragma unroll
            for (int v = 0; v < NV; v++) gg[d][v] = g[d * rstr + v * B200_SOASZ];
        bc_ldg_state<ND, T>(bc, gas.gamma, ul, nn, ur);
        bc_ldg_grad_state<ND, T>(bc, imperm ? ur : ul, nn, gg, gr);
        b200::viscous_flux_add<ND, T>(ur, gr, fvr, gas);
        // Artificial viscosity of the boundary gradient
        if (va.base) {
            const T a = va.base[b200::load_ix(va.map, ix64, i)];
#pragma unroll
            for (int d = 0; d < ND; d++)
#pragma unroll
                for (int v = 0; v < NV; v++) fvr[d][v] -= a * gr[d][v];
        }
    }

    // Inviscid part: Riemann solve against the ghost state
    bc_rsolve_state<ND, T>(bc, gas.gamma, ul, nn, ur);
    b200::rsolve_t<RS, ND, T>(ul, ur, nn, fi, gas.gamma, gas.p_min);

#pragma unroll
    for (int v = 0; v < NV; v++) {
        T fv = 0;
#pragma unroll
        for (int d = 0; d < ND; d++) fv += nn[d] * fvr[d][v];
        if (!slip && !imperm) fv += tau * (ul[v] - ur[v]);
        pl[v * B200_SOASZ] = mag * (fi[v] + fv);
    }
}

// Order-preserving integer key of a non-negative value (its bit pattern)
__device__ __forceinline__ void atomic_min_nonneg(double *a, double v) {
    atomicMin(reinterpret_cast<unsigned long long *>(a),
              (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_min_nonneg(float *a, float v) {
    atomicMin(reinterpret_cast<unsigned int *>(a), __float_as_uint(v));
}

template <int ND, typename T>
__global__ void __launch_bounds__(BC_BLOCK)
bccent_kernel(int64_t n, T gamma, BcK<T> bc0, ScalView<T> vl, ScalView<T> ve, int ix64,
              const T *__restrict__ nl, int64_t ldn, T big) {
    constexpr int NV = ND + 2;
    const int64_t i = (int64_t)blockIdx.x * BC_BLOCK + threadIdx.x;
    if (i >= n) return;
    BcK<T> bc = bc0;
    if (bc.perpt) bc_at_point<ND, T>(bc, i, gamma);
    const T *pl = vl.base + b200::load_ix(vl.map, ix64, i);
    T *pe = ve.base + b200::load_ix(ve.map, ix64, i);
    T ul[NV], ur[NV], nn[ND];
#pragma unroll
    for (int v = 0; v < NV; v++) ul[v] = pl[v * B200_SOASZ];
    unit_normal<ND, T>(nl, ldn, i, nn);
    bc_rsolve_state<ND, T>(bc, gamma, ul, nn, ur);
    // Entropy p rho^-gamma of the ghost state (largest value when it has
    // no positive density and pressure)
    const T rcpd = T(1) / ur[0];
    T k2 = 0;
#pragma unroll
    for (int d = 0; d < ND; d++) k2 += ur[d + 1] * ur[d + 1];
    const T p = (gamma - T(1)) * (ur[NV - 1] - T(0.5) * rcpd * k2);
    const T e = (ur[0] > 0 && p > 0) ? p * pow(rcpd, gamma) : big;
    atomic_min_nonneg(pe, e);
}

bool bc_type_ok(int t) { return t >= B200_BC_SUP_IN_FA && t <= B200_BC_CHAR_RIEM_INV_CTRL; }

// The boundary types of the Euler system
bool bc_euler_type(int t) {
    return (t >= B200_BC_SUP_IN_FA && t <= B200_BC_CHAR_RIEM_INV) ||
           t == B200_BC_CHAR_RIEM_INV_CTRL;
}

template <typename T>
int bccflux_euler(int ndims, int64_t n, int rs, double gamma, double p_min, const b200_bc_t *bc,
                  T *ul_base, const void *ul_map, int ix64, const T *nl, int64_t ldn,
                  cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (!bc || !bc_euler_type(bc->type))
        return b200::set_error(B200_ERR_ARG, "bccflux_euler: bad boundary type");
    const auto k = bc_consts<T>(*bc, gamma);
    if (!bc_exprs_ok(k))
        return b200::set_error(B200_ERR_ARG, "boundary expressions need ploc");
    ScalView<T> l{ul_base, ul_map};
    const unsigned grid = b200::ceil_div(n, BC_BLOCK);
    if (ndims != 2 && ndims != 3)
        return b200::set_error(B200_ERR_ARG, "bccflux_euler: ndims must be 2 or 3");
    const bool ok = b200::with_rsolver(rs, [&](auto rsc) {
        constexpr int RS = decltype(rsc)::value;
        if (ndims == 2)
            bccflux_euler_kernel<RS, 2, T><<<grid, BC_BLOCK, 0, st>>>(n, (T)gamma, (T)p_min, k, l, ix64, nl, ldn);
        else
            bccflux_euler_kernel<RS, 3, T><<<grid, BC_BLOCK, 0, st>>>(n, (T)gamma, (T)p_min, k, l, ix64, nl, ldn);
    });
    if (!ok) return b200::set_error(B200_ERR_ARG, "bccflux_euler: unknown Riemann solver %d", rs);
    B200_CHECK_LAUNCH("bccflux_euler");
    return B200_OK;
}

template <typename T>
int bcconu(int ndims, int64_t n, double gamma, const b200_bc_t *bc, const T *in_base,
           const void *in_map, T *out_base, const void *out_map, int ix64, const T *nl,
           int64_t ldn, cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (!bc || !bc_type_ok(bc->type))
        return b200::set_error(B200_ERR_ARG, "bcconu: bad boundary type");
    const auto k = bc_consts<T>(*bc, gamma);
    if (!bc_exprs_ok(k))
        return b200::set_error(B200_ERR_ARG, "boundary expressions need ploc");
    ScalView<T> vi{const_cast<T *>(in_base), in_map}, vo{out_base, out_map};
    const unsigned grid = b200::ceil_div(n, BC_BLOCK);
    if (ndims == 2)
        bcconu_kernel<2, T><<<grid, BC_BLOCK, 0, st>>>(n, (T)gamma, k, vi, vo, ix64, nl, ldn);
    else if (ndims == 3)
        bcconu_kernel<3, T><<<grid, BC_BLOCK, 0, st>>>(n, (T)gamma, k, vi, vo, ix64, nl, ldn);
    else
        return b200::set_error(B200_ERR_ARG, "bcconu: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("bcconu");
    return B200_OK;
}

template <typename T>
int bccflux_ns(int ndims, int64_t n, int rs, const b200_gas_t *gas, double tau,
               const b200_bc_t *bc, T *ul_base, const void *ul_map, const T *gl_base,
               const void *gl_map, const void *gl_rstr, int ix64, const T *nl, int64_t ldn,
               const T *av_base, const void *av_map, cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (!gas || !bc || !bc_type_ok(bc->type) || (av_base && !av_map))
        return b200::set_error(B200_ERR_ARG, "bccflux_ns: bad arguments");
    ScalView<T> va{const_cast<T *>(av_base), av_map};
    const Gas &g0 = *reinterpret_cast<const Gas *>(gas);
    if (g0.shifted)
        return b200::set_error(B200_ERR_UNSUPPORTED,
                               "bccflux_ns: boundaries take unshifted states");
    const auto g = b200::gas_consts<T>(g0);
    const auto k = bc_consts<T>(*bc, g0.gamma);
    if (!bc_exprs_ok(k))
        return b200::set_error(B200_ERR_ARG, "boundary expressions need ploc");
    ScalView<T> l{ul_base, ul_map};
    VectView<T> gv{gl_base, gl_map, gl_rstr};
    const unsigned grid = b200::ceil_div(n, BC_BLOCK);
    if (ndims != 2 && ndims != 3)
        return b200::set_error(B200_ERR_ARG, "bccflux_ns: ndims must be 2 or 3");
    const bool ok = b200::with_rsolver(rs, [&](auto rsc) {
        constexpr int RS = decltype(rsc)::value;
        if (ndims == 2)
            bccflux_ns_kernel<RS, 2, T><<<grid, BC_BLOCK, 0, st>>>(n, g, (T)tau, k, l, gv, ix64, nl, ldn, va);
        else
            bccflux_ns_kernel<RS, 3, T><<<grid, BC_BLOCK, 0, st>>>(n, g, (T)tau, k, l, gv, ix64, nl, ldn, va);
    });
    if (!ok) return b200::set_error(B200_ERR_ARG, "bccflux_ns: unknown Riemann solver %d", rs);
    B200_CHECK_LAUNCH("bccflux_ns");
    return B200_OK;
}

template <typename T>
int bccent(int ndims, int64_t n, double gamma, const b200_bc_t *bc, const T *ul_base,
           const void *ul_map, T *ent_base, const void *ent_map, int ix64, const T *nl,
           int64_t ldn, cudaStream_t st) {
    if (n <= 0) return B200_OK;
    if (!bc || !bc_type_ok(bc->type))
        return b200::set_error(B200_ERR_ARG, "bccent: bad boundary type");
    const auto k = bc_consts<T>(*bc, gamma);
    if (!bc_exprs_ok(k))
        return b200::set_error(B200_ERR_ARG, "boundary expressions need ploc");
    ScalView<T> l{const_cast<T *>(ul_base), ul_map}, e{ent_base, ent_map};
    const T big = sizeof(T) == 8 ? (T)1.7976931348623157e308 : (T)3.4028234663852886e38;
    const unsigned grid = b200::ceil_div(n, BC_BLOCK);
    if (ndims == 2)
        bccent_kernel<2, T><<<grid, BC_BLOCK, 0, st>>>(n, (T)gamma, k, l, e, ix64, nl, ldn, big);
    else if (ndims == 3)
        bccent_kernel<3, T><<<grid, BC_BLOCK, 0, st>>>(n, (T)gamma, k, l, e, ix64, nl, ldn, big);
    else
        return b200::set_error(B200_ERR_ARG, "bccent: ndims must be 2 or 3");
    B200_CHECK_LAUNCH("bccent");
    return B200_OK;
}

__global__ void stage_time_kernel(double *t, const double *dt_dev, double dt, double c) {
    t[1] = t[0] + c * (dt_dev ? dt_dev[0] : dt);
}

}  // namespace

extern "C" {

int b200_stage_time(double *t, const double *dt_dev, double dt, double c, void *stream) {
    if (!t) return b200::set_error(B200_ERR_ARG, "stage_time: null time");
    stage_time_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(t, dt_dev, dt, c);
    B200_CHECK_LAUNCH("stage_time");
    return B200_OK;
}


int b200_bccent_f64(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const double *ul_base, const void *ul_map, double *ent_base,
                    const void *ent_map, int ix64, const double *nl, int64_t ldn, void *stream) {
    return bccent<double>(ndims, n, gamma, bc, ul_base, ul_map, ent_base, ent_map, ix64, nl, ldn,
                          (cudaStream_t)stream);
}

int b200_bccent_f32(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const float *ul_base, const void *ul_map, float *ent_base,
                    const void *ent_map, int ix64, const float *nl, int64_t ldn, void *stream) {
    return bccent<float>(ndims, n, gamma, bc, ul_base, ul_map, ent_base, ent_map, ix64, nl, ldn,
                         (cudaStream_t)stream);
}

int b200_bccflux_euler_f64(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                           const b200_bc_t *bc,
                           double *ul_base, const void *ul_map, int ix64, const double *nl,
                           int64_t ldn, void *stream) {
    return bccflux_euler<double>(ndims, n, rsolver, gamma, p_min, bc, ul_base, ul_map, ix64, nl, ldn,
                                 (cudaStream_t)stream);
}

int b200_bccflux_euler_f32(int ndims, int64_t n, int rsolver, double gamma, double p_min,
                           const b200_bc_t *bc,
                           float *ul_base, const void *ul_map, int ix64, const float *nl,
                           int64_t ldn, void *stream) {
    return bccflux_euler<float>(ndims, n, rsolver, gamma, p_min, bc, ul_base, ul_map, ix64, nl, ldn,
                                (cudaStream_t)stream);
}

int b200_bcconu_f64(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const double *ulin_base, const void *ulin_map, double *ulout_base,
                    const void *ulout_map, int ix64, const double *nl, int64_t ldn,
                    void *stream) {
    return bcconu<double>(ndims, n, gamma, bc, ulin_base, ulin_map, ulout_base, ulout_map, ix64,
                          nl, ldn, (cudaStream_t)stream);
}

int b200_bcconu_f32(int ndims, int64_t n, double gamma, const b200_bc_t *bc,
                    const float *ulin_base, const void *ulin_map, float *ulout_base,
                    const void *ulout_map, int ix64, const float *nl, int64_t ldn,
                    void *stream) {
    return bcconu<float>(ndims, n, gamma, bc, ulin_base, ulin_map, ulout_base, ulout_map, ix64,
                         nl, ldn, (cudaStream_t)stream);
}

int b200_bccflux_ns_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double tau,
                        const b200_bc_t *bc, double *ul_base, const void *ul_map,
                        const double *gl_base, const void *gl_map, const void *gl_rstr,
                        int ix64, const double *nl, int64_t ldn, void *stream) {
    return bccflux_ns<double>(ndims, n, rsolver, gas, tau, bc, ul_base, ul_map, gl_base, gl_map,
                              gl_rstr, ix64, nl, ldn, nullptr, nullptr, (cudaStream_t)stream);
}

int b200_bccflux_ns_av_f64(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                           double tau, const b200_bc_t *bc, double *ul_base, const void *ul_map,
                           const double *gl_base, const void *gl_map, const void *gl_rstr,
                           int ix64, const double *nl, int64_t ldn, const double *av_base,
                           const void *av_map, void *stream) {
    if (!av_base) return b200::set_error(B200_ERR_ARG, "bccflux_ns_av: null viscosity");
    return bccflux_ns<double>(ndims, n, rsolver, gas, tau, bc, ul_base, ul_map, gl_base, gl_map,
                          gl_rstr, ix64, nl, ldn, av_base, av_map, (cudaStream_t)stream);
}

int b200_bccflux_ns_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas, double tau,
                        const b200_bc_t *bc, float *ul_base, const void *ul_map,
                        const float *gl_base, const void *gl_map, const void *gl_rstr,
                        int ix64, const float *nl, int64_t ldn, void *stream) {
    return bccflux_ns<float>(ndims, n, rsolver, gas, tau, bc, ul_base, ul_map, gl_base, gl_map,
                             gl_rstr, ix64, nl, ldn, nullptr, nullptr, (cudaStream_t)stream);
}

int b200_bccflux_ns_av_f32(int ndims, int64_t n, int rsolver, const b200_gas_t *gas,
                           double tau, const b200_bc_t *bc, float *ul_base, const void *ul_map,
                           const float *gl_base, const void *gl_map, const void *gl_rstr,
                           int ix64, const float *nl, int64_t ldn, const float *av_base,
                           const void *av_map, void *stream) {
    if (!av_base) return b200::set_error(B200_ERR_ARG, "bccflux_ns_av: null viscosity");
    return bccflux_ns<float>(ndims, n, rsolver, gas, tau, bc, ul_base, ul_map, gl_base, gl_map,
                          gl_rstr, ix64, nl, ldn, av_base, av_map, (cudaStream_t)stream);
}

}  // extern "C"
