// Device functions for the compressible Euler / Navier-Stokes physics.
//
// Each function states the arithmetic of one reference kernel macro:
//   inviscid_flux      pyfr/solvers/euler/kernels/flux.mako:3-26
//   viscous_flux_add   pyfr/solvers/navstokes/kernels/flux.mako:3-105
//   rsolve (Rusanov)   pyfr/solvers/euler/kernels/rsolvers/rusanov.mako:4-26
//   rsolve (HLLC)      pyfr/solvers/euler/kernels/rsolvers/hllc.mako:4-77
//   rsolve (HLL)       pyfr/solvers/euler/kernels/rsolvers/hll.mako:4-53
//   rsolve (Roe)       pyfr/solvers/euler/kernels/rsolvers/roe.mako:6-84
//   rsolve (RoeM)      pyfr/solvers/euler/kernels/rsolvers/roem.mako:5-96
//   rsolve (exact)     pyfr/solvers/euler/kernels/rsolvers/exact.mako:14-185
//   normal frame       pyfr/solvers/baseadvec/kernels/transform.mako:5-75
//   calc_smats_detj    pyfr/solvers/baseadvec/kernels/smats.mako:3-25
//   transform_grad     pyfr/solvers/baseadvecdiff/kernels/transform_grad.mako:3-10
// NV = ND + 2 conserved variables: rho, rho*u_i, E.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace b200 {

// Gas / viscosity constants shared by all flux kernels (POD, matches the
// b200_gas_t struct of the C ABI).  When `shifted` is set the kernels'
// input is q = T(u - u_ref): the perturbation from a constant reference
// state (rho_ref, rho_ref V, E_ref = p_ref/(gamma - 1) + rho_ref |V|^2/2)
// with the energy component replaced by dE - h_t*drho, h_t = (E_ref +
// p_ref)/rho_ref the reference total enthalpy per unit mass.  T is linear
// and constant, so the system in q is the system in u multiplied by T: the
// mass and momentum equations are unchanged and the energy equation is the
// energy equation minus h_t times the mass equation.  The constant flux of
// the reference state is dropped (the flux-reconstruction divergence of a
// constant flux field is exactly zero), and what remains is formed from the
// perturbation: with v = V + w, w = (dm - V drho)/rho, the momentum flux is
// rho_ref V w + dm V + dm w + dp I and the energy flux (q_E + dp) v.  Every
// flux is then of the size of the perturbation, so FP32 rounding no longer
// scales with p_ref, the reference enthalpy or the mean flow.
struct Gas {
    double gamma, mu, pr, cpTref, cpTs;
    int sutherland;
    int shifted;
    double rho_ref, p_ref;
    double p_min;
    double v_ref[3];    // reference velocity V (zero: the fluid at rest)
};

// The same constants in the kernel's arithmetic type, with every derived
// quantity formed once on the host: on this GPU a per-thread FP64
// division costs more than the whole FP32 flux evaluation.
template <typename T>
struct GasK {
    T gamma, gm1, mu, gamma_pr, rcp_cpTref, mu_ctt, cpTs, quarter_gamma;
    T rho_ref, p_ref, e_ref, hs_ref, p_min;
    T v_ref[3], m_ref[3];
    int sutherland, shifted;
    int moving;     // v_ref is not zero
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
    double v2 = 0.0;
    for (int i = 0; i < 3; i++) {
        k.v_ref[i] = (T)g.v_ref[i];
        k.m_ref[i] = (T)(g.rho_ref * g.v_ref[i]);
        v2 += g.v_ref[i] * g.v_ref[i];
    }
    k.moving = v2 != 0.0;
    const double e_ref = g.p_ref / (g.gamma - 1.0) + 0.5 * g.rho_ref * v2;
    k.e_ref = (T)e_ref;
    k.hs_ref = (T)(g.rho_ref != 0.0 ? (e_ref + g.p_ref) / g.rho_ref : 0.0);
    k.p_min = (T)g.p_min;
    k.sutherland = g.sutherland;
    k.shifted = g.shifted;
    return k;
}

// Riemann solvers by the index the C ABI takes (rsolver argument)
enum RSolver { RS_RUSANOV = 0, RS_HLLC = 1, RS_HLL = 2, RS_ROE = 3, RS_ROEM = 4, RS_EXACT = 5 };

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

// The inviscid flux of state s along n, formed directly
// (pyfr/solvers/euler/kernels/flux.mako:3-26 contracted with n): mass
// rho v.n, momentum rho u_i v.n + p n_i, energy (E + p) v.n; returns the
// pressure and the normal velocity.  Fewer operations than the full flux
// followed by its projection, which matters where FP64 throughput bounds.
template <int ND, typename T>
__device__ __forceinline__ void inviscid_nflux(const T *s, const T *n, T *fn, T &p, T &vn,
                                               T gamma) {
    constexpr int NV = ND + 2;
    const T invrho = T(1) / s[0], E = s[NV - 1];
    T dot = 0, mn = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        dot += s[i + 1] * s[i + 1];
        mn += s[i + 1] * n[i];
    }
    p = (gamma - T(1)) * (E - T(0.5) * invrho * dot);
    vn = invrho * mn;
    fn[0] = mn;
#pragma unroll
    for (int i = 0; i < ND; i++) fn[i + 1] = s[i + 1] * vn + p * n[i];
    fn[NV - 1] = (E + p) * vn;
}

// The (negated-stress) viscous flux of uin along n, formed directly: the
// normal component of viscous_flux_add's flux, momentum tau.n and energy
// u.(tau.n) + kcoef dT.n, added to fn (mass untouched).
template <int ND, typename T>
__device__ __forceinline__ void viscous_nflux_add(const T *uin, const T grad[ND][ND + 2],
                                                  const T *n, T *fn, const GasK<T> &g) {
    constexpr int NV = ND + 2;
    const T rho = uin[0], E = uin[NV - 1];
    const T rcprho = T(1) / rho;
    T vel[ND];
#pragma unroll
    for (int i = 0; i < ND; i++) vel[i] = rcprho * uin[i + 1];

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

    // Normal temperature derivative (c_v dT/dn)
    T dTn = 0;
#pragma unroll
    for (int d = 0; d < ND; d++) {
        T t = rcprho * grad[d][0] * E;
#pragma unroll
        for (int i = 0; i < ND; i++) t += vel[i] * dv[i][d];
        dTn += n[d] * (rcprho * (grad[d][NV - 1] - t));
    }

    T div = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) div += dv[i][i];

    // (tau.n)_i with the negated stress tau_ij = -mu/rho (dv_ij + dv_ji -
    // 2/3 div delta_ij)
    const T mr = -mu_c * rcprho;
    T e = -mu_c * g.gamma_pr * dTn;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        T tn = T(-2.0 / 3.0) * div * n[i];
#pragma unroll
        for (int j = 0; j < ND; j++) tn += (dv[j][i] + dv[i][j]) * n[j];
        tn *= mr;
        fn[i + 1] += tn;
        e += vel[i] * tn;
    }
    fn[NV - 1] += e;
}

template <int ND, typename T>
__device__ __forceinline__ void rsolve_rusanov(const T *ul, const T *ur, const T *n, T *nf,
                                               T gamma) {
    constexpr int NV = ND + 2;
    T fl[NV], fr[NV], pl, pr, vnl, vnr;
    inviscid_nflux<ND, T>(ul, n, fl, pl, vnl, gamma);
    inviscid_nflux<ND, T>(ur, n, fr, pr, vnr, gamma);

    // Maximum wave speed estimate (halved)
    const T a = sqrt(T(0.25) * gamma * (pl + pr) / (ul[0] + ur[0])) + T(0.25) * fabs(vnl + vnr);

#pragma unroll
    for (int i = 0; i < NV; i++) nf[i] = T(0.5) * (fl[i] + fr[i]) + a * (ul[i] - ur[i]);
}

// Inviscid flux, less the reference state's, from the transformed input
// s = q = T(u - u_ref) (see Gas): rho = rho_ref + s[0], dm = s[1..ND],
// dE = s[E] + h_t s[0]; the velocity v = V + w with w = (dm - V s[0])/rho;
// dp = p - p_ref = (gamma - 1)(dE - (m.v - rho_ref |V|^2)/2) with
// m.v - rho_ref |V|^2 = rho_ref V.w + dm.V + dm.w; mass flux dm, momentum
// flux rho_ref V w + dm V + dm w + dp I, energy flux (s[E] + dp) v.  (With
// V = 0 these are m, m v + dp I and (s[E] + dp) v.)  Returns the full
// pressure in p, the full velocity in v and the full state in ufull (for
// the viscous terms and the wave speeds).
//
// MOVING false takes V = 0 at compile time (the reference state at rest:
// the Navier-Stokes kernels' case), which keeps those kernels as lean as
// before the moving form existed.
template <int ND, typename T, bool MOVING = false>
__device__ __forceinline__ void inviscid_flux_shift(const T *s, T f[ND][ND + 2], T &p, T v[ND],
                                                    T ufull[ND + 2], const GasK<T> &g) {
    constexpr int NV = ND + 2;
    const T gm1 = g.gm1;
    const T rho = g.rho_ref + s[0], invrho = T(1) / rho;
    const T dE = s[NV - 1] + g.hs_ref * s[0];
    if constexpr (MOVING) {
        T w[ND], dot = 0;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            w[i] = invrho * (s[i + 1] - g.v_ref[i] * s[0]);
            v[i] = g.v_ref[i] + w[i];
            dot += g.m_ref[i] * w[i] + s[i + 1] * v[i];
        }
        const T dp = gm1 * (dE - T(0.5) * dot);
        p = g.p_ref + dp;
        const T hv = s[NV - 1] + dp;
#pragma unroll
        for (int i = 0; i < ND; i++) {
            f[i][0] = s[i + 1];
            f[i][NV - 1] = hv * v[i];
#pragma unroll
            for (int j = 0; j < ND; j++)
                f[i][j + 1] = g.m_ref[i] * w[j] + s[i + 1] * v[j] + (i == j ? dp : T(0));
        }
#pragma unroll
        for (int i = 0; i < ND; i++) ufull[i + 1] = g.m_ref[i] + s[i + 1];
    } else {
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
#pragma unroll
        for (int i = 0; i < ND; i++) ufull[i + 1] = s[i + 1];
    }
    ufull[0] = rho;
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
template <int ND, typename T, bool MOVING = false>
__device__ __forceinline__ void rsolve_rusanov_shift(const T *ul, const T *ur, const T *n, T *nf,
                                                     T ufl[ND + 2], T ufr[ND + 2],
                                                     const GasK<T> &g) {
    constexpr int NV = ND + 2;
    T fl[ND][NV], fr[ND][NV], vl[ND], vr[ND], pl, pr;
    inviscid_flux_shift<ND, T, MOVING>(ul, fl, pl, vl, ufl, g);
    inviscid_flux_shift<ND, T, MOVING>(ur, fr, pr, vr, ufr, g);

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

// HLL (pyfr/solvers/euler/kernels/rsolvers/hll.mako:4-53): Roe-averaged
// wave-speed estimates; the reference takes the right state's sound speed
// in both the left and the right estimate, and so does this.
template <int ND, typename T>
__device__ __forceinline__ void rsolve_hll(const T *ul, const T *ur, const T *n, T *nf,
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
    const T ar = sqrt(gamma * pr / ur[0]);
    const T sql = sqrt(ul[0]), sqr = sqrt(ur[0]);
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
    const T sl = fmin(nv - a, nvl - ar);
    const T sr = fmax(nv + a, nvr + ar);
    const T rcpsrsl = T(1) / (sr - sl);

#pragma unroll
    for (int i = 0; i < NV; i++) {
        T nf_fl = 0, nf_fr = 0;
#pragma unroll
        for (int j = 0; j < ND; j++) {
            nf_fl += n[j] * fl[j][i];
            nf_fr += n[j] * fr[j][i];
        }
        const T sub = (sr * nf_fl - sl * nf_fr + sl * sr * (ur[i] - ul[i])) * rcpsrsl;
        nf[i] = (T(0) <= sl) ? nf_fl : (T(0) >= sr) ? nf_fr : sub;
    }
}

// Momentum components u[1..ND] expressed in the frame whose first axis is
// the unit normal n (Moler and Hughes 1999), and back:
// pyfr/solvers/baseadvec/kernels/transform.mako:5-75.  Density and energy
// are frame-independent.
template <int ND, typename T>
__device__ __forceinline__ void rot_to(const T *n, const T *u, T *t) {
    const T *m = u + 1;
    T *r = t + 1;
    if (ND == 2) {
        r[0] = n[0] * m[0] + n[1] * m[1];
        r[1] = n[0] * m[1] - n[1] * m[0];
    } else if (fabs(n[0]) < T(0.99)) {
        const T h = T(1) / (T(1) + n[0]);
        r[0] = n[0] * m[0] + n[1] * m[1] + n[2] * m[2];
        r[1] = (n[0] + h * n[2] * n[2]) * m[1] - n[1] * m[0] - h * n[1] * n[2] * m[2];
        r[2] = (n[0] + h * n[1] * n[1]) * m[2] - n[2] * m[0] - h * n[1] * n[2] * m[1];
    } else if (fabs(n[1]) < fabs(n[2])) {
        const T h = T(1) / (T(1) - n[1]);
        r[0] = n[0] * m[0] + n[1] * m[1] + n[2] * m[2];
        r[1] = (T(1) - h * n[0] * n[0]) * m[0] + n[0] * m[1] - h * n[0] * n[2] * m[2];
        r[2] = n[2] * m[1] - h * n[0] * n[2] * m[0] + (T(1) - h * n[2] * n[2]) * m[2];
    } else {
        const T h = T(1) / (T(1) - n[2]);
        r[0] = n[0] * m[0] + n[1] * m[1] + n[2] * m[2];
        r[1] = (T(1) - h * n[1] * n[1]) * m[1] - h * n[0] * n[1] * m[0] + n[1] * m[2];
        r[2] = (T(1) - h * n[0] * n[0]) * m[0] - h * n[0] * n[1] * m[1] + n[0] * m[2];
    }
}

template <int ND, typename T>
__device__ __forceinline__ void rot_from(const T *n, const T *t, T *u) {
    const T *m = t + 1;
    T *r = u + 1;
    if (ND == 2) {
        r[0] = n[0] * m[0] - n[1] * m[1];
        r[1] = n[1] * m[0] + n[0] * m[1];
    } else if (fabs(n[0]) < T(0.99)) {
        const T h = T(1) / (T(1) + n[0]);
        r[0] = n[0] * m[0] - n[1] * m[1] - n[2] * m[2];
        r[1] = n[1] * m[0] + (n[0] + h * n[2] * n[2]) * m[1] - h * n[1] * n[2] * m[2];
        r[2] = n[2] * m[0] - h * n[1] * n[2] * m[1] + (n[0] + h * n[1] * n[1]) * m[2];
    } else if (fabs(n[1]) < fabs(n[2])) {
        const T h = T(1) / (T(1) - n[1]);
        r[0] = n[0] * m[0] + (T(1) - h * n[0] * n[0]) * m[1] - h * n[0] * n[2] * m[2];
        r[1] = n[1] * m[0] + n[0] * m[1] + n[2] * m[2];
        r[2] = n[2] * m[0] - h * n[0] * n[2] * m[1] + (T(1) - h * n[2] * n[2]) * m[2];
    } else {
        const T h = T(1) / (T(1) - n[2]);
        r[0] = n[0] * m[0] - h * n[0] * n[1] * m[1] + (T(1) - h * n[0] * n[0]) * m[2];
        r[1] = n[1] * m[0] + (T(1) - h * n[1] * n[1]) * m[1] - h * n[0] * n[1] * m[2];
        r[2] = n[2] * m[0] + n[1] * m[1] + n[0] * m[2];
    }
}

// x-direction flux, pressure and velocity of a state in the normal frame
// (pyfr/solvers/euler/kernels/flux.mako:28-48)
template <int ND, typename T>
__device__ __forceinline__ void inviscid_flux_1d(const T *s, T *f, T &p, T *v, T gamma) {
    constexpr int NV = ND + 2;
    const T invrho = T(1) / s[0], E = s[NV - 1];
    T k2 = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        v[i] = invrho * s[i + 1];
        k2 += s[i + 1] * s[i + 1];
    }
    p = (gamma - T(1)) * (E - T(0.5) * invrho * k2);
    f[0] = s[1];
    f[NV - 1] = (E + p) * v[0];
    f[1] = s[1] * v[0] + p;
#pragma unroll
    for (int j = 1; j < ND; j++) f[j + 1] = s[1] * v[j];
}

// Roe flux with a parabolic entropy fix of width 1e-3 on the acoustic
// eigenvalues, in the normal frame
// (pyfr/solvers/euler/kernels/rsolvers/roe.mako:6-84)
template <int ND, typename T>
__device__ __forceinline__ void roe_1d(const T *ul, const T *ur, T *nf, T gamma) {
    constexpr int NV = ND + 2;
    constexpr double eps = 0.001;
    T fl[NV], fr[NV], vl[ND], vr[ND], pl, pr, va[ND], dv[ND];
    inviscid_flux_1d<ND, T>(ul, fl, pl, vl, gamma);
    inviscid_flux_1d<ND, T>(ur, fr, pr, vr, gamma);

    const T sql = sqrt(ul[0]), sqr = sqrt(ur[0]);
    const T roa = sql * sqr;
    const T ha = (sql * (pr + ur[NV - 1]) + sqr * (pl + ul[NV - 1])) / (sql * ur[0] + sqr * ul[0]);
    const T inv_rar = T(1) / (sql + sqr);
    T qq = 0, vdv = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        va[i] = (vl[i] * sql + vr[i] * sqr) * inv_rar;
        qq += va[i] * va[i];
    }
    const T a = sqrt((gamma - T(1)) * (ha - T(0.5) * qq));

    T l1 = fabs(va[0] - a);
    const T l2 = fabs(va[0]);
    T l3 = fabs(va[0] + a);
    l1 = (l1 < T(eps)) ? T(0.5 / eps) * (l1 * l1 + T(eps * eps)) : l1;
    l3 = (l3 < T(eps)) ? T(0.5 / eps) * (l3 * l3 + T(eps * eps)) : l3;

#pragma unroll
    for (int i = 0; i < ND; i++) {
        dv[i] = vr[i] - vl[i];
        vdv += va[i] * dv[i];
    }
    const T dro = ur[0] - ul[0];
    const T dp = pr - pl;
    const T inv_a2 = T(1) / (T(2) * a * a);

    // Wave strengths of the acoustic and entropy waves
    const T w1 = (dp - roa * a * dv[0]) * inv_a2;
    const T w2 = dro - dp * T(2) * inv_a2;
    const T w3 = (dp + roa * a * dv[0]) * inv_a2;

    nf[0] = T(0.5) * (fl[0] + fr[0]) - (l1 * w1 + l2 * w2 + l3 * w3);
#pragma unroll
    for (int i = 0; i < ND; i++) {
        T v1, v2, v3;
        if (i == 0) {
            v1 = w1 * (va[0] - a);
            v2 = w2 * va[0];
            v3 = w3 * (va[0] + a);
        } else {
            v1 = w1 * va[i];
            v2 = w2 * va[i] + roa * dv[i];
            v3 = w3 * va[i];
        }
        nf[i + 1] = T(0.5) * (fl[i + 1] + fr[i + 1]) - (l1 * v1 + l2 * v2 + l3 * v3);
    }
    const T v1 = w1 * (ha - a * va[0]);
    const T v2 = roa * (vdv - va[0] * dv[0]) + w2 * qq * T(0.5);
    const T v3 = w3 * (ha + a * va[0]);
    nf[NV - 1] = T(0.5) * (fl[NV - 1] + fr[NV - 1]) - (l1 * v1 + l2 * v2 + l3 * v3);
}

// RoeM (Kim, Kim and Rho, J. Comput. Phys. 185(2), 2003;
// pyfr/solvers/euler/kernels/rsolvers/roem.mako:5-96)
template <int ND, typename T>
__device__ __forceinline__ void rsolve_roem(const T *ul, const T *ur, const T *n, T *nf,
                                            T gamma) {
    constexpr int NV = ND + 2;
    T fl[ND][NV], fr[ND][NV], vl[ND], vr[ND], va[ND], dv[ND], du[NV], bdq[NV], pl, pr;
    inviscid_flux<ND, T>(ul, fl, pl, vl, gamma);
    inviscid_flux<ND, T>(ur, fr, pr, vr, gamma);

    const T hl = (ul[NV - 1] + pl) / ul[0];
    const T hr = (ur[NV - 1] + pr) / ur[0];
    T contral = 0, contrar = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        contral += n[i] * vl[i];
        contrar += n[i] * vr[i];
    }
    const T drho = ur[0] - ul[0];
    const T dp = pr - pl;
    const T dh = hr - hl;
    const T dcontra = contrar - contral;

    // Roe averages
    const T rrr = sqrt(ur[0] / ul[0]);
    const T ratl = T(1) / (T(1) + rrr);
    const T ratr = rrr * ratl;
    const T ra = rrr * ul[0];
    const T ha = hl * ratl + hr * ratr;
    T qq = 0, contraa = 0;
#pragma unroll
    for (int i = 0; i < ND; i++) {
        dv[i] = vr[i] - vl[i];
        va[i] = vl[i] * ratl + vr[i] * ratr;
        qq += va[i] * va[i];
        contraa += n[i] * va[i];
    }
    const T aa = sqrt((gamma - T(1)) * (ha - T(0.5) * qq));
    const T rcp_aa = T(1) / aa;
    const T abs_ma = fabs(contraa * rcp_aa) + T(1e-15);

    // Normalised wave speeds
    T b1 = fmax(T(0), fmax(contraa + aa, contrar + aa));
    T b2 = fmin(T(0), fmin(contraa - aa, contral - aa));
    T b1b2 = b1 * b2;
    const T rcp_b1_b2 = T(1) / (b1 - b2);
    b1 = b1 * rcp_b1_b2;
    b2 = b2 * rcp_b1_b2;
    b1b2 = b1b2 * rcp_b1_b2;

    // Shock sensing and the Mach-number functions f and g
    const T sdst = (pl < pr) ? pl / pr : pr / pl;
    const T h = T(1) - sdst;
    const T f = pow(abs_ma, h);
    const T g = f / (T(1) + abs_ma);

#pragma unroll
    for (int i = 0; i < NV - 1; i++) du[i] = ur[i] - ul[i];
    du[NV - 1] = ur[0] * hr - ul[0] * hl;

    bdq[0] = drho - f * dp * rcp_aa * rcp_aa;
    bdq[NV - 1] = bdq[0] * ha + ra * dh;
#pragma unroll
    for (int i = 0; i < ND; i++) bdq[i + 1] = bdq[0] * va[i] + ra * (dv[i] - n[i] * dcontra);

#pragma unroll
    for (int i = 0; i < NV; i++) {
        T s = 0;
#pragma unroll
        for (int j = 0; j < ND; j++) s += n[j] * (b1 * fl[j][i] - b2 * fr[j][i]);
        nf[i] = s + b1b2 * (du[i] - g * bdq[i]);
    }
}

// Flux f(p) of the pressure function and its derivative for one side of
// the exact Riemann problem, covolume zero (Toro 2009, eqs. 4.86-4.87;
// pyfr/solvers/euler/kernels/rsolvers/exact.mako:14-30)
template <typename T>
__device__ __forceinline__ void exact_star_flux(T p, T ps, T rs, T cs, T gamma, T &f, T &fd) {
    const double g = (double)gamma;
    if (p <= ps) {
        const T pr = p / ps;
        const T pr_g = pow(pr, T(-(g + 1) / (2 * g)));
        fd = pr_g / (rs * cs);
        f = T(2 / (g - 1)) * cs * (pr_g * pr - T(1));
    } else {
        const T pbs_inv = T(1) / (p + T((g - 1) / (g + 1)) * ps);
        const T sapb = sqrt(T(2 / (g + 1)) * pbs_inv / rs);
        f = (p - ps) * sapb;
        fd = sapb - T(0.5) * f * pbs_inv;
    }
}

// Exact Riemann solution sampled at x/t = 0 in the normal frame: adaptive
// initial guess (primitive-variable, two-rarefaction or two-shock), three
// Newton iterations on the star pressure, then the sampling decision tree
// (Toro 2009, ch. 4 and 9; pyfr/solvers/euler/kernels/rsolvers/exact.mako)
template <int ND, typename T>
__device__ __forceinline__ void exact_1d(const T *ul, const T *ur, T *nf, T gamma, T p_min) {
    constexpr int NV = ND + 2;
    const double g = (double)gamma;
    const T hgm = T(0.5 * (g - 1)), grgm = T(g / (g - 1)), trgm = T(2 / (g - 1));
    const T trgp = T(2 / (g + 1)), gmrtg = T((g - 1) / (2 * g)), gprtg = T((g + 1) / (2 * g));
    const T tgrgm = T((2 * g) / (g - 1)), gmrgp = T((g - 1) / (g + 1)), rg = T(1 / g);

    T vl[ND], vr[ND], w0[NV];
    T pl, pr, cl, cr;
    {
        T k2 = 0;
        const T inv = T(1) / ul[0];
#pragma unroll
        for (int i = 0; i < ND; i++) {
            vl[i] = inv * ul[i + 1];
            k2 += ul[i + 1] * ul[i + 1];
        }
        pl = (gamma - T(1)) * (ul[NV - 1] - T(0.5) * inv * k2);
        cl = sqrt(gamma * pl * inv);
    }
    {
        T k2 = 0;
        const T inv = T(1) / ur[0];
#pragma unroll
        for (int i = 0; i < ND; i++) {
            vr[i] = inv * ur[i + 1];
            k2 += ur[i + 1] * ur[i + 1];
        }
        pr = (gamma - T(1)) * (ur[NV - 1] - T(0.5) * inv * k2);
        cr = sqrt(gamma * pr * inv);
    }

    const T rl = ul[0], rr = ur[0];
    const T bpv = fmax(T(0), T(0.125) * (vl[0] - vr[0]) * (rl + rr) * (cl + cr) +
                                 T(0.5) * (pl + pr));
    const T pmin = fmin(pl, pr), pmax = fmax(pl, pr);
    T p0;
    if (pmax <= T(2) * pmin && pmin <= bpv && bpv <= pmax) {
        p0 = bpv;
    } else if (bpv < pmin) {
        // Two-rarefaction guess
        const T pre = pow(pl / pr, gmrtg);
        const T um = (pre * vl[0] * cr + vr[0] * cl + trgm * (pre - T(1)) * cl * cr) /
                     (pre * cr + cl);
        const T ptl = T(1) - hgm * (um - vl[0]) / cl;
        const T ptr = T(1) + hgm * (um - vr[0]) / cr;
        p0 = T(0.5) * (pl * pow(ptl, tgrgm) + pr * pow(ptr, tgrgm));
    } else {
        // Two-shock guess
        const T gl = sqrt(trgp / (rl * (gmrgp * pl + bpv)));
        const T gr = sqrt(trgp / (rr * (gmrgp * pr + bpv)));
        p0 = (gl * pl + gr * pr - vr[0] + vl[0]) / (gl + gr);
    }

    T fsl, fdl, fsr, fdr;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        exact_star_flux<T>(p0, pl, rl, cl, gamma, fsl, fdl);
        exact_star_flux<T>(p0, pr, rr, cr, gamma, fsr, fdr);
        const T p1 = p0 - (fsl + fsr + vr[0] - vl[0]) / (fdl + fdr);
        p0 = (p1 < T(0)) ? p_min : p1;
    }
    const T us = T(0.5) * (vl[0] + vr[0] + fsr - fsl);

    if (T(0) <= us) {
#pragma unroll
        for (int i = 1; i < ND; i++) w0[i + 1] = vl[i];
        if (p0 <= pl) {
            if (vl[0] >= cl) {
                w0[0] = rl; w0[1] = vl[0]; w0[NV - 1] = pl;
            } else if (us < cl * pow(p0 / pl, gmrtg)) {
                w0[0] = rl * pow(p0 / pl, rg); w0[1] = us; w0[NV - 1] = p0;
            } else {
                const T c = trgp + gmrgp * vl[0] / cl;
                w0[0] = rl * pow(c, trgm);
                w0[1] = trgp * cl + gmrgp * vl[0];
                w0[NV - 1] = pl * pow(c, tgrgm);
            }
        } else {
            const T p0p = p0 / pl;
            const T sl = vl[0] - cl * sqrt(gprtg * p0p + gmrtg);
            if (T(0) <= sl) {
                w0[0] = rl; w0[1] = vl[0]; w0[NV - 1] = pl;
            } else {
                w0[0] = rl * (p0p + gmrgp) / (p0p * gmrgp + T(1)); w0[1] = us; w0[NV - 1] = p0;
            }
        }
    } else {
#pragma unroll
        for (int i = 1; i < ND; i++) w0[i + 1] = vr[i];
        if (p0 > pr) {
            const T p0p = p0 / pr;
            const T sr = vr[0] + cr * sqrt(gprtg * p0p + gmrtg);
            if (sr <= T(0)) {
                w0[0] = rr; w0[1] = vr[0]; w0[NV - 1] = pr;
            } else {
                w0[0] = rr * (p0p + gmrgp) / (p0p * gmrgp + T(1)); w0[1] = us; w0[NV - 1] = p0;
            }
        } else if (vr[0] + cr <= T(0)) {
            w0[0] = rr; w0[1] = vr[0]; w0[NV - 1] = pr;
        } else {
            const T p0p = p0 / pr;
            if (us + cr * pow(p0p, gmrtg) >= T(0)) {
                w0[0] = rr * pow(p0p, rg); w0[1] = us; w0[NV - 1] = p0;
            } else {
                const T c = trgp - gmrgp * vr[0] / cr;
                w0[0] = rr * pow(c, trgm);
                w0[1] = gmrgp * vr[0] - trgp * cr;
                w0[NV - 1] = pr * pow(c, tgrgm);
            }
        }
    }

    // Primitive state to the x-direction flux
    nf[0] = w0[0] * w0[1];
    nf[1] = nf[0] * w0[1] + w0[NV - 1];
    T k2 = 0;
#pragma unroll
    for (int i = 1; i < ND + 1; i++) k2 += w0[i] * w0[i];
#pragma unroll
    for (int i = 2; i < ND + 1; i++) nf[i] = nf[0] * w0[i];
    nf[NV - 1] = (grgm * w0[NV - 1] + T(0.5) * w0[0] * k2) * w0[1];
}

// A one-dimensional solver applied in the normal frame
// (pyfr/solvers/euler/kernels/rsolvers/rsolve1d.mako:5-22)
template <int RS, int ND, typename T>
__device__ __forceinline__ void rsolve_rotated(const T *ul, const T *ur, const T *n, T *nf,
                                               T gamma, T p_min) {
    constexpr int NV = ND + 2;
    T utl[NV], utr[NV], ntf[NV];
    utl[0] = ul[0];
    utr[0] = ur[0];
    utl[NV - 1] = ul[NV - 1];
    utr[NV - 1] = ur[NV - 1];
    rot_to<ND, T>(n, ul, utl);
    rot_to<ND, T>(n, ur, utr);
    if (RS == RS_ROE)
        roe_1d<ND, T>(utl, utr, ntf, gamma);
    else
        exact_1d<ND, T>(utl, utr, ntf, gamma, p_min);
    nf[0] = ntf[0];
    nf[NV - 1] = ntf[NV - 1];
    rot_from<ND, T>(n, ntf, nf);
}

// The Riemann solver as a compile-time choice: each interface kernel is
// instantiated per solver, so it carries the registers of its own solver
// only.  p_min: the floor of the exact solver's Newton iterations
// (pyfr/solvers/euler/inters.py:12-25).
template <int RS, int ND, typename T>
__device__ __forceinline__ void rsolve_t(const T *ul, const T *ur, const T *n, T *nf, T gamma,
                                         T p_min) {
    if constexpr (RS == RS_HLLC)
        rsolve_hllc<ND, T>(ul, ur, n, nf, gamma);
    else if constexpr (RS == RS_HLL)
        rsolve_hll<ND, T>(ul, ur, n, nf, gamma);
    else if constexpr (RS == RS_ROEM)
        rsolve_roem<ND, T>(ul, ur, n, nf, gamma);
    else if constexpr (RS == RS_ROE || RS == RS_EXACT)
        rsolve_rotated<RS, ND, T>(ul, ur, n, nf, gamma, p_min);
    else
        rsolve_rusanov<ND, T>(ul, ur, n, nf, gamma);
}

// Host-side dispatch of a launch over the solvers: fn(integral_constant<RS>)
template <typename F>
inline bool with_rsolver(int rs, F &&fn) {
    switch (rs) {
    case RS_RUSANOV: fn(std::integral_constant<int, RS_RUSANOV>()); return true;
    case RS_HLLC: fn(std::integral_constant<int, RS_HLLC>()); return true;
    case RS_HLL: fn(std::integral_constant<int, RS_HLL>()); return true;
    case RS_ROE: fn(std::integral_constant<int, RS_ROE>()); return true;
    case RS_ROEM: fn(std::integral_constant<int, RS_ROEM>()); return true;
    case RS_EXACT: fn(std::integral_constant<int, RS_EXACT>()); return true;
    default: return false;
    }
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
