// Device functions for the compressible Euler / Navier-Stokes physics.
//
// Each function states the arithmetic of one reference kernel macro:
//   inviscid_flux      pyfr/solvers/euler/kernels/flux.mako:3-26
//   viscous_flux_add   pyfr/solvers/navstokes/kernels/flux.mako:3-105
//   rsolve (Rusanov)   pyfr/solvers/euler/kernels/rsolvers/rusanov.mako:4-26
//   rsolve (HLLC)      pyfr/solvers/euler/kernels/rsolvers/hllc.mako:4-77
//   calc_smats_detj    pyfr/solvers/baseadvec/kernels/smats.mako:3-25
//   transform_grad     pyfr/solvers/baseadvecdiff/kernels/transform_grad.mako:3-10
// NV = ND + 2 conserved variables: rho, rho*u_i, E.
#pragma once

#include "common.cuh"

namespace b200 {

// Gas / viscosity constants shared by all flux kernels (POD, matches the
// b200_gas_t struct of the C ABI).  When `shifted` is set the kernels'
// input is q = T(u - u_ref): the perturbation from a constant reference
// state (rho_ref, 0, E_ref = p_ref/(gamma - 1)) with the energy component
// replaced by dE - h_ref*drho, h_ref = gamma/(gamma - 1) p_ref/rho_ref the
// reference specific enthalpy.  T is linear and constant, so the system in
// q is the system in u multiplied by T: the mass and momentum equations are
// unchanged and the energy equation is the energy equation minus h_ref
// times the mass equation.  Its inviscid flux is (dE - h_ref*drho + dp) v
// instead of (H_ref + dE + dp) v, and the constant part p_ref*I of the
// momentum flux is dropped (the flux-reconstruction divergence of a
// constant flux field is exactly zero).  Every flux is then of the size of
// the perturbation, so FP32 rounding no longer scales with p_ref or H_ref.
struct Gas {
    double gamma, mu, pr, cpTref, cpTs;
    int sutherland;
    int shifted;
    double rho_ref, p_ref;
};

// The same constants in the kernel's arithmetic type, with every derived
// quantity formed once on the host: on this GPU a per-thread FP64
// division costs more than the whole FP32 flux evaluation.
template <typename T>
struct GasK {
    T gamma, gm1, mu, gamma_pr, rcp_cpTref, mu_ctt, cpTs, quarter_gamma;
    T rho_ref, p_ref, e_ref, h_ref, hs_ref;
    int sutherland, shifted;
};

template <typename T>
inline GasK<T> gas_consts(const Gas &g) {
    GasK<T> k;
    k.gamma = (T)g.gamma;
    k.gm1 = (T)(g.gamma - 1.0);
    k.mu = (T)g.mu;
    k.gamma_pr = (T)(g.gamma / g.pr);
    k.rcp_cpTref = (T)(1.0 / g.cpTref);
    k.mu_ctt = (T)(g.mu * (g.cpTref + g.cpTs));
    k.cpTs = (T)g.cpTs;
    k.quarter_gamma = (T)(0.25 * g.gamma);
    k.rho_ref = (T)g.rho_ref;
    k.p_ref = (T)g.p_ref;
    k.e_ref = (T)(g.p_ref / (g.gamma - 1.0));
    k.h_ref = (T)(g.gamma / (g.gamma - 1.0) * g.p_ref);
    k.hs_ref = (T)(g.rho_ref != 0.0 ? g.gamma / (g.gamma - 1.0) * g.p_ref / g.rho_ref : 0.0);
    k.sutherland = g.sutherland;
    k.shifted = g.shifted;
    return k;
}

enum RSolver { RS_RUSANOV = 0, RS_HLLC = 1 };

template <int ND, typename T>
__device__ __forceinline__ void inviscid_flux(const T *s, T f[ND][ND + 2], T &p, T v[ND],
                                              T gamma) {
    constexpr int NV = ND + 2;
    const T invrho = T(1) / s[0], E = s[NV - 1];
    T rhov[ND];
    T dot = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        rhov[i] = s[i + 1];
        v[i] = invrho * rhov[i];
        dot += rhov[i] * rhov[i];
    }
    p = (gamma - T(1)) * (E - T(0.5) * invrho * dot);
#pragma unroll
    for (int i = 0; i < ND; i++) {
        f[i][0] = rhov[i];
        f[i][NV - 1] = (E + p) * v[i];
#pragma unroll
        for (int j = 0; j < ND; j++) f[i][j + 1] = rhov[i] * v[j] + (i == j ? p : T(0));
    }
}

// Adds the (negated-stress) viscous flux to fout; grad[d][var] holds the
// physical gradient of the conserved variables.
template <int ND, typename T>
__device__ __forceinline__ void viscous_flux_add(const T *uin, const T grad[ND][ND + 2],
                                                 T fout[ND][ND + 2], const GasK<T> &g) {
    constexpr int NV = ND + 2;
    const T rho = uin[0], E = uin[NV - 1];
    const T rcprho = T(1) / rho;
    T vel[ND];
#pragma unroll
    for (int i = 0; i < ND; i++) vel[i] = rcprho * uin[i + 1];

    // Velocity derivatives times rho: dv[i][d] = rho * d(u_i)/dx_d
    T dv[ND][ND];
#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int d = 0; d < ND; d++) dv[i][d] = grad[d][i + 1] - vel[i] * grad[d][0];

    T mu_c;
    if (g.sutherland) {
        T ke = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) ke += vel[i] * vel[i];
        const T cpT = g.gamma * (rcprho * E - T(0.5) * ke);
        const T Trat = g.rcp_cpTref * cpT;
        mu_c = g.mu_ctt * Trat * sqrt(Trat) / (cpT + g.cpTs);
    } else {
        mu_c = g.mu;
    }

    // Temperature derivatives (c_v dT/dx_d)
    T dT[ND];
#pragma unroll
    for (int d = 0; d < ND; d++) {
        T t = rcprho * grad[d][0] * E;
#pragma unroll
        for (int i = 0; i < ND; i++) t += vel[i] * dv[i][d];
        dT[d] = rcprho * (grad[d][NV - 1] - t);
    }

    // Negated stress tensor
    T div = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) div += dv[i][i];
    T tau[ND][ND];
#pragma unroll
    for (int i = 0; i < ND; i++) {
        tau[i][i] = T(-2) * mu_c * rcprho * (dv[i][i] - T(1.0 / 3.0) * div);
#pragma unroll
        for (int j = i + 1; j < ND; j++) {
            tau[i][j] = tau[j][i] = -mu_c * rcprho * (dv[j][i] + dv[i][j]);
        }
    }

    const T kcoef = -mu_c * g.gamma_pr;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        T e = kcoef * dT[d];
#pragma unroll
        for (int i = 0; i < ND; i++) {
            fout[d][i + 1] += tau[i][d];
            e += vel[i] * tau[i][d];
        }
        fout[d][NV - 1] += e;
    }
}

template <int ND, typename T>
__device__ __forceinline__ void rsolve_rusanov(const T *ul, const T *ur, const T *n, T *nf,
                                               T gamma) {
    constexpr int NV = ND + 2;
    T fl[ND][NV], fr[ND][NV], vl[ND], vr[ND], pl, pr;
    inviscid_flux<ND, T>(ul, fl, pl, vl, gamma);
    inviscid_flux<ND, T>(ur, fr, pr, vr, gamma);

    T nv = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) nv += n[i] * (vl[i] + vr[i]);

    // Maximum wave speed estimate (halved)
    const T a = sqrt(T(0.25) * gamma * (pl + pr) / (ul[0] + ur[0])) + T(0.25) * fabs(nv);

#pragma unroll
    for (int i = 0; i < NV; i++) {
        T s = 0;
#pragma unroll
        for (int j = 0; j < ND; j++) s += n[j] * (fl[j][i] + fr[j][i]);
        nf[i] = T(0.5) * s + a * (ul[i] - ur[i]);
    }
}

// Inviscid flux from the transformed input s = q = T(u - u_ref) (see Gas):
// rho = rho_ref + s[0], m = s[1..ND], dE = s[E] + hs_ref*s[0], dp = p - p_ref
// from (gamma - 1)(dE - |m|^2/(2 rho)); mass flux m, momentum flux
// m v + dp I, energy flux (s[E] + dp) v.  Returns the full pressure in p and
// the full state in ufull (for the viscous terms).
template <int ND, typename T>
__device__ __forceinline__ void inviscid_flux_shift(const T *s, T f[ND][ND + 2], T &p, T v[ND],
                                                    T ufull[ND + 2], const GasK<T> &g) {
    constexpr int NV = ND + 2;
    const T gm1 = g.gm1;
    const T rho = g.rho_ref + s[0], invrho = T(1) / rho;
    const T dE = s[NV - 1] + g.hs_ref * s[0];
    T dot = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        v[i] = invrho * s[i + 1];
        dot += s[i + 1] * v[i];
    }
    const T dp = gm1 * (dE - T(0.5) * dot);
    p = g.p_ref + dp;
    const T hv = s[NV - 1] + dp;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        f[i][0] = s[i + 1];
        f[i][NV - 1] = hv * v[i];
#pragma unroll
        for (int j = 0; j < ND; j++) f[i][j + 1] = s[i + 1] * v[j] + (i == j ? dp : T(0));
    }
    ufull[0] = rho;
#pragma unroll
    for (int i = 0; i < ND; i++) ufull[i + 1] = s[i + 1];
    ufull[NV - 1] = g.e_ref + dE;
}

// Gradient of the full state from the gradient of q (the energy row of
// T^-1; the reference state itself is constant)
template <int ND, typename T>
__device__ __forceinline__ void unshift_grad(const T gq[ND][ND + 2], T gu[ND][ND + 2],
                                             const GasK<T> &g) {
    constexpr int NV = ND + 2;
#pragma unroll
    for (int d = 0; d < ND; d++) {
#pragma unroll
        for (int v = 0; v < NV - 1; v++) gu[d][v] = gq[d][v];
        gu[d][NV - 1] = gq[d][NV - 1] + g.hs_ref * gq[d][0];
    }
}

// Rusanov flux on transformed inputs: the dissipation acts on differences
// of q, which are T times the differences of u, so the flux is T times the
// Rusanov flux of the full states
template <int ND, typename T>
__device__ __forceinline__ void rsolve_rusanov_shift(const T *ul, const T *ur, const T *n, T *nf,
                                                     T ufl[ND + 2], T ufr[ND + 2],
                                                     const GasK<T> &g) {
    constexpr int NV = ND + 2;
    T fl[ND][NV], fr[ND][NV], vl[ND], vr[ND], pl, pr;
    inviscid_flux_shift<ND, T>(ul, fl, pl, vl, ufl, g);
    inviscid_flux_shift<ND, T>(ur, fr, pr, vr, ufr, g);

    T nv = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) nv += n[i] * (vl[i] + vr[i]);
    const T a = sqrt(g.quarter_gamma * (pl + pr) / (ufl[0] + ufr[0])) + T(0.25) * fabs(nv);

#pragma unroll
    for (int i = 0; i < NV; i++) {
        T s = 0;
#pragma unroll
        for (int j = 0; j < ND; j++) s += n[j] * (fl[j][i] + fr[j][i]);
        nf[i] = T(0.5) * s + a * (ul[i] - ur[i]);
    }
}

template <int ND, typename T>
__device__ __forceinline__ void rsolve_hllc(const T *ul, const T *ur, const T *n, T *nf,
                                            T gamma) {
    constexpr int NV = ND + 2;
    T fl[ND][NV], fr[ND][NV], vl[ND], vr[ND], pl, pr;
    inviscid_flux<ND, T>(ul, fl, pl, vl, gamma);
    inviscid_flux<ND, T>(ur, fr, pr, vr, gamma);

    T nvl = 0, nvr = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        nvl += n[i] * vl[i];
        nvr += n[i] * vr[i];
    }
    const T al = sqrt(gamma * pl / ul[0]), ar = sqrt(gamma * pr / ur[0]);
    const T sql = sqrt(ul[0]), sqr = sqrt(ur[0]);

    // Roe averages of the normal velocity, enthalpy and velocity
    const T nv = (sql * nvl + sqr * nvr) / (sql + sqr);
    const T H = (sql * (pr + ur[NV - 1]) + sqr * (pl + ul[NV - 1])) / (sql * ur[0] + sqr * ul[0]);
    const T inv_rar = T(1) / (sql + sqr);
    T qq = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        const T va = (vl[i] * sql + vr[i] * sqr) * inv_rar;
        qq += va * va;
    }
    const T a = sqrt((gamma - T(1)) * (H - T(0.5) * qq));

    // Wave speed estimates and the contact speed
    const T sl = fmin(nv - a, nvl - al);
    const T sr = fmax(nv + a, nvr + ar);
    const T sstar = (pr - pl + ul[0] * nvl * (sl - nvl) - ur[0] * nvr * (sr - nvr)) /
                    (ul[0] * (sl - nvl) - ur[0] * (sr - nvr));

    const T ul_com = (sl - nvl) / (sl - sstar);
    const T ur_com = (sr - nvr) / (sr - sstar);

    T usl[NV], usr[NV];
    usl[0] = ul_com * ul[0];
    usr[0] = ur_com * ur[0];
#pragma unroll
    for (int i = 0; i < ND; i++) {
        usl[i + 1] = usl[0] * (vl[i] + (sstar - nvl) * n[i]);
        usr[i + 1] = usr[0] * (vr[i] + (sstar - nvr) * n[i]);
    }
    usl[NV - 1] = ul_com * (ul[NV - 1] + (sstar - nvl) * (ul[0] * sstar + pl / (sl - nvl)));
    usr[NV - 1] = ur_com * (ur[NV - 1] + (sstar - nvr) * (ur[0] * sstar + pr / (sr - nvr)));

#pragma unroll
    for (int i = 0; i < NV; i++) {
        T nf_fl = 0, nf_fr = 0;
#pragma unroll
        for (int j = 0; j < ND; j++) {
            nf_fl += n[j] * fl[j][i];
            nf_fr += n[j] * fr[j][i];
        }
        const T nf_fsl = nf_fl + sl * (usl[i] - ul[i]);
        const T nf_fsr = nf_fr + sr * (usr[i] - ur[i]);
        nf[i] = (T(0) <= sl) ? nf_fl
              : (sl <= T(0) && T(0) <= sstar) ? nf_fsl
              : (sstar <= T(0) && T(0) <= sr) ? nf_fsr
              : nf_fr;
    }
}

template <int ND, typename T>
__device__ __forceinline__ void rsolve(int rs, const T *ul, const T *ur, const T *n, T *nf,
                                       T gamma) {
    if (rs == RS_HLLC)
        rsolve_hllc<ND, T>(ul, ur, n, nf, gamma);
    else
        rsolve_rusanov<ND, T>(ul, ur, n, nf, gamma);
}

// Metric terms of a linear (multilinear) element at reference point x from
// its vertices V (vertex order: first coordinate fastest).  s[i][j] is the
// adjugate of the Jacobian J[i][j] = dX_j/dxi_i, d = det J.
template <int ND, typename T>
__device__ __forceinline__ void linear_smats(const T V[1 << ND][ND], const T *x, T s[ND][ND],
                                             T &d) {
    constexpr int NVT = 1 << ND;
    T J[ND][ND];
#pragma unroll
    for (int i = 0; i < ND; i++)
#pragma unroll
        for (int j = 0; j < ND; j++) J[i][j] = 0;

#pragma unroll
    for (int v = 0; v < NVT; v++) {
#pragma unroll
        for (int i = 0; i < ND; i++) {
            // d(shape fn of vertex v)/d(xi_i)
            T w = ((v >> i) & 1) ? T(1) : T(-1);
#pragma unroll
            for (int k = 0; k < ND; k++)
                if (k != i) w *= ((v >> k) & 1) ? (T(1) + x[k]) : (T(1) - x[k]);
            w *= T(1.0 / NVT);
#pragma unroll
            for (int j = 0; j < ND; j++) J[i][j] += w * V[v][j];
        }
    }

    if (ND == 2) {
        s[0][0] = J[1][1];
        s[0][1] = -J[1][0];
        s[1][0] = -J[0][1];
        s[1][1] = J[0][0];
        d = s[0][0] * s[1][1] - s[0][1] * s[1][0];
    } else {
#pragma unroll
        for (int i = 0; i < ND; i++) {
            const int a = (i + 1) % 3, b = (i + 2) % 3;
            s[i][0] = J[a][1] * J[b][2] - J[a][2] * J[b][1];
            s[i][1] = J[a][2] * J[b][0] - J[a][0] * J[b][2];
            s[i][2] = J[a][0] * J[b][1] - J[a][1] * J[b][0];
        }
        d = J[0][0] * s[0][0] + J[0][1] * s[0][1] + J[0][2] * s[0][2];
    }
}

}  // namespace b200
