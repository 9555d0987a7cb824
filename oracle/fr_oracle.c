/*
 * C/OpenMP restatement of the flux-reconstruction right-hand side.
 *
 * TEST INFRASTRUCTURE AND CPU BASELINE ONLY.  It is the multi-core CPU
 * counterpart of oracle/fr_oracle.py and stands in for the reference's
 * OpenMP backend (pyfr/backends/openmp), which cannot be built here or on
 * the GPU hosts: its runtime dependencies (mako, libxsmm) are absent.  It
 * follows the same kernel arithmetic (see the citations in fr_oracle.py):
 *
 *   Euler: disu (M0) -> intcflux -> tflux -> M1-M3*M2 -> M3 -> negdivconf
 *          (pyfr/solvers/baseadvec/system.py:58-136)
 *   NS:    disu -> intconu -> M4-M6*M0 + M6 -> transform + flux ->
 *          M0 (gradients to flux points) -> intcflux -> M1-M3*M2 -> M3 ->
 *          negdivconf (pyfr/solvers/baseadvecdiff/system.py:54-231)
 *
 * Data layout is element-major: u[e][pt][var].  Operators are CSR (their
 * structural zeros cost nothing, as with the reference's sparse kernels).
 * Element phases and interface phases are each one OpenMP loop.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int m, k;
    const int *rowptr, *colidx;
    const double *val;
} fro_csr;

typedef struct {
    int ndims, nvars, nupts, nfpts, neles;
    fro_csr M0, M132, M3, M460, M6;
    const double *smats;      /* [e][upt][i][j] */
    const double *rcpdjac;    /* [e][upt] */
    int64_t npairs;
    const int64_t *lpt, *le, *rpt, *re;   /* flux point / element of each side */
    const double *nl;         /* [pair][d], scaled left normals */
    double gamma, mu, pr, beta, tau;
    int rsolver;              /* 0 rusanov, 1 hllc */
} fro_disc;

#define MAXV 5
#define MAXD 3

/* out[e] (m x nv) = A (m x k) @ in[e] (k x nv), element by element */
static void csr_apply(const fro_csr *A, const double *in, double *out, int nv, int accumulate) {
    for (int i = 0; i < A->m; i++) {
        double acc[MAXV];
        for (int v = 0; v < nv; v++) acc[v] = accumulate ? out[i * nv + v] : 0.0;
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
            const double a = A->val[p];
            const double *x = in + (int64_t)A->colidx[p] * nv;
            for (int v = 0; v < nv; v++) acc[v] += a * x[v];
        }
        for (int v = 0; v < nv; v++) out[i * nv + v] = acc[v];
    }
}

static void inviscid_flux(int nd, const double *s, double f[MAXD][MAXV], double *p, double *v,
                          double gamma) {
    const int nv = nd + 2;
    const double invrho = 1.0 / s[0], E = s[nv - 1];
    double dot = 0;
    for (int i = 0; i < nd; i++) {
        v[i] = invrho * s[i + 1];
        dot += s[i + 1] * s[i + 1];
    }
    *p = (gamma - 1) * (E - 0.5 * invrho * dot);
    for (int i = 0; i < nd; i++) {
        f[i][0] = s[i + 1];
        f[i][nv - 1] = (E + *p) * v[i];
        for (int j = 0; j < nd; j++) f[i][j + 1] = s[i + 1] * v[j] + (i == j ? *p : 0.0);
    }
}

static void viscous_flux_add(int nd, const double *u, double g[MAXD][MAXV],
                             double f[MAXD][MAXV], const fro_disc *d) {
    const int nv = nd + 2;
    const double rho = u[0], E = u[nv - 1], rcprho = 1.0 / rho;
    double vel[MAXD], dv[MAXD][MAXD], dT[MAXD], tau[MAXD][MAXD], div = 0;
    for (int i = 0; i < nd; i++) vel[i] = rcprho * u[i + 1];
    for (int i = 0; i < nd; i++)
        for (int k = 0; k < nd; k++) dv[i][k] = g[k][i + 1] - vel[i] * g[k][0];
    for (int k = 0; k < nd; k++) {
        double t = rcprho * g[k][0] * E;
        for (int i = 0; i < nd; i++) t += vel[i] * dv[i][k];
        dT[k] = rcprho * (g[k][nv - 1] - t);
    }
    for (int i = 0; i < nd; i++) div += dv[i][i];
    const double mu = d->mu;
    for (int i = 0; i < nd; i++) {
        tau[i][i] = -2 * mu * rcprho * (dv[i][i] - div / 3.0);
        for (int j = i + 1; j < nd; j++) tau[i][j] = tau[j][i] = -mu * rcprho * (dv[j][i] + dv[i][j]);
    }
    for (int k = 0; k < nd; k++) {
        double e = -mu * (d->gamma / d->pr) * dT[k];
        for (int i = 0; i < nd; i++) {
            f[k][i + 1] += tau[i][k];
            e += vel[i] * tau[i][k];
        }
        f[k][nv - 1] += e;
    }
}

static void rsolve(int nd, const double *ul, const double *ur, const double *n, double *nf,
                   const fro_disc *d) {
    const int nv = nd + 2;
    const double gamma = d->gamma;
    double fl[MAXD][MAXV], fr[MAXD][MAXV], vl[MAXD], vr[MAXD], pl, pr;
    inviscid_flux(nd, ul, fl, &pl, vl, gamma);
    inviscid_flux(nd, ur, fr, &pr, vr, gamma);

    if (d->rsolver == 0) {
        double nvs = 0;
        for (int i = 0; i < nd; i++) nvs += n[i] * (vl[i] + vr[i]);
        const double a = sqrt(0.25 * gamma * (pl + pr) / (ul[0] + ur[0])) + 0.25 * fabs(nvs);
        for (int v = 0; v < nv; v++) {
            double s = 0;
            for (int j = 0; j < nd; j++) s += n[j] * (fl[j][v] + fr[j][v]);
            nf[v] = 0.5 * s + a * (ul[v] - ur[v]);
        }
        return;
    }

    double nvl = 0, nvr = 0, qq = 0;
    for (int i = 0; i < nd; i++) {
        nvl += n[i] * vl[i];
        nvr += n[i] * vr[i];
    }
    const double al = sqrt(gamma * pl / ul[0]), ar = sqrt(gamma * pr / ur[0]);
    const double sql = sqrt(ul[0]), sqr = sqrt(ur[0]);
    const double nvroe = (sql * nvl + sqr * nvr) / (sql + sqr);
    const double H = (sql * (pr + ur[nv - 1]) + sqr * (pl + ul[nv - 1])) / (sql * ur[0] + sqr * ul[0]);
    for (int i = 0; i < nd; i++) {
        const double va = (vl[i] * sql + vr[i] * sqr) / (sql + sqr);
        qq += va * va;
    }
    const double a = sqrt((gamma - 1) * (H - 0.5 * qq));
    const double sl = fmin(nvroe - a, nvl - al), sr = fmax(nvroe + a, nvr + ar);
    const double ss = (pr - pl + ul[0] * nvl * (sl - nvl) - ur[0] * nvr * (sr - nvr)) /
                      (ul[0] * (sl - nvl) - ur[0] * (sr - nvr));
    const double lc = (sl - nvl) / (sl - ss), rc = (sr - nvr) / (sr - ss);
    double usl[MAXV], usr[MAXV];
    usl[0] = lc * ul[0];
    usr[0] = rc * ur[0];
    for (int i = 0; i < nd; i++) {
        usl[i + 1] = usl[0] * (vl[i] + (ss - nvl) * n[i]);
        usr[i + 1] = usr[0] * (vr[i] + (ss - nvr) * n[i]);
    }
    usl[nv - 1] = lc * (ul[nv - 1] + (ss - nvl) * (ul[0] * ss + pl / (sl - nvl)));
    usr[nv - 1] = rc * (ur[nv - 1] + (ss - nvr) * (ur[0] * ss + pr / (sr - nvr)));
    for (int v = 0; v < nv; v++) {
        double nfl = 0, nfr = 0;
        for (int j = 0; j < nd; j++) {
            nfl += n[j] * fl[j][v];
            nfr += n[j] * fr[j][v];
        }
        const double nfsl = nfl + sl * (usl[v] - ul[v]), nfsr = nfr + sr * (usr[v] - ur[v]);
        nf[v] = (0 <= sl) ? nfl : (sl <= 0 && 0 <= ss) ? nfsl : (ss <= 0 && 0 <= sr) ? nfsr : nfr;
    }
}

/* Scratch sizes (doubles) */
int64_t fro_scratch_size(const fro_disc *d) {
    const int64_t ne = d->neles, nv = d->nvars, nd = d->ndims;
    /* uf, comm, gradf (nd*nfpts), F/g per element in-loop */
    return ne * nv * (d->nfpts * (2 + nd));
}

static void unit_normal(const fro_disc *d, int64_t i, double *n, double *mag) {
    double m = 0;
    for (int k = 0; k < d->ndims; k++) m += d->nl[i * d->ndims + k] * d->nl[i * d->ndims + k];
    m = sqrt(m);
    for (int k = 0; k < d->ndims; k++) n[k] = d->nl[i * d->ndims + k] / m;
    *mag = m;
}

/* Transformed flux (from physical flux f) into F[d][upt][v] of one element */
static void transform_store(const fro_disc *d, const double *S, double f[MAXD][MAXV], double *F,
                            int upt) {
    const int nd = d->ndims, nv = d->nvars, nupts = d->nupts;
    for (int i = 0; i < nd; i++)
        for (int v = 0; v < nv; v++) {
            double acc = 0;
            for (int k = 0; k < nd; k++) acc += S[i * nd + k] * f[k][v];
            F[((int64_t)i * nupts + upt) * nv + v] = acc;
        }
}

/* Solution at the flux points and, for Navier-Stokes, the LDG common
 * solution (intconu) into comm */
static void flux_point_states(const fro_disc *d, int navier_stokes, const double *u, double *uf,
                              double *comm) {
    const int nv = d->nvars, nupts = d->nupts, nfpts = d->nfpts;
    const int64_t ne = d->neles;

    #pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < ne; e++) {
        csr_apply(&d->M0, u + e * nupts * nv, uf + e * nfpts * nv, nv, 0);
        if (navier_stokes) memcpy(comm + e * nfpts * nv, uf + e * nfpts * nv, sizeof(double) * nfpts * nv);
    }

    if (navier_stokes) {
        #pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < d->npairs; i++) {
            const double *ul = uf + (d->le[i] * nfpts + d->lpt[i]) * nv;
            const double *ur = uf + (d->re[i] * nfpts + d->rpt[i]) * nv;
            double *cl = comm + (d->le[i] * nfpts + d->lpt[i]) * nv;
            double *cr = comm + (d->re[i] * nfpts + d->rpt[i]) * nv;
            for (int v = 0; v < nv; v++) {
                if (d->beta == -0.5) cr[v] = ul[v];
                else if (d->beta == 0.5) cl[v] = ur[v];
                else cl[v] = cr[v] = ur[v] * (0.5 + d->beta) + ul[v] * (0.5 - d->beta);
            }
        }
    }
}

/* Physical corrected gradient of element e at its solution points into
 * g[d][upt][v] (tgradpcoru + tgradcoru + gradcoru) */
static void element_gradient(const fro_disc *d, const double *u, const double *comm, int64_t e,
                             double *g) {
    const int nd = d->ndims, nv = d->nvars, nupts = d->nupts, nfpts = d->nfpts;
    csr_apply(&d->M460, u + e * nupts * nv, g, nv, 0);
    csr_apply(&d->M6, comm + e * nfpts * nv, g, nv, 1);
    for (int p = 0; p < nupts; p++) {
        const double *S = d->smats + (e * nupts + p) * nd * nd;
        const double rj = d->rcpdjac[e * nupts + p];
        double tg[MAXD][MAXV];
        for (int k = 0; k < nd; k++)
            for (int v = 0; v < nv; v++) tg[k][v] = g[((int64_t)k * nupts + p) * nv + v];
        for (int i = 0; i < nd; i++)
            for (int v = 0; v < nv; v++) {
                double acc = 0;
                for (int k = 0; k < nd; k++) acc += S[k * nd + i] * tg[k][v];
                g[((int64_t)i * nupts + p) * nv + v] = rj * acc;
            }
    }
}

/* Kinetic energy, enstrophy and volume integrals of a 3-D Navier-Stokes
 * solution with solution-point quadrature weights qw (per point; times
 * |J|): out = {sum w rho |v|^2, sum w rho |curl v|^2, sum w}
 * (pyfr/plugins/integrate.py:58-77 with the expressions of the
 * Taylor-Green diagnostics). */
int fro_integrals(const fro_disc *d, const double *u, const double *qw, double *scratch,
                  double *out) {
    const int nd = d->ndims, nv = d->nvars, nupts = d->nupts, nfpts = d->nfpts;
    const int64_t ne = d->neles;
    if (nd != 3) return 1;
    double *uf = scratch, *comm = uf + ne * nfpts * nv;
    flux_point_states(d, 1, u, uf, comm);
    double ke = 0, en = 0, vol = 0;
    #pragma omp parallel reduction(+:ke, en, vol)
    {
        double *g = malloc(sizeof(double) * nd * nupts * nv);
        #pragma omp for schedule(static)
        for (int64_t e = 0; e < ne; e++) {
            element_gradient(d, u, comm, e, g);
            for (int p = 0; p < nupts; p++) {
                const double *up = u + (e * nupts + p) * nv;
                const double w = qw[p] / d->rcpdjac[e * nupts + p];
                const double rho = up[0];
                double vel[3], du[3][3];
                for (int i = 0; i < 3; i++) vel[i] = up[i + 1] / rho;
                for (int k = 0; k < 3; k++)
                    for (int i = 0; i < 3; i++)
                        du[k][i] = (g[((int64_t)k * nupts + p) * nv + i + 1] -
                                    vel[i] * g[((int64_t)k * nupts + p) * nv]) / rho;
                const double w1 = du[1][2] - du[2][1], w2 = du[2][0] - du[0][2],
                             w3 = du[0][1] - du[1][0];
                ke += w * rho * (vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2]);
                en += w * rho * (w1 * w1 + w2 * w2 + w3 * w3);
                vol += w;
            }
        }
        free(g);
    }
    out[0] = ke;
    out[1] = en;
    out[2] = vol;
    return 0;
}

int fro_rhs(const fro_disc *d, int navier_stokes, const double *u, double *r, double *scratch) {
    const int nd = d->ndims, nv = d->nvars, nupts = d->nupts, nfpts = d->nfpts;
    const int64_t ne = d->neles;
    double *uf = scratch;                                   /* [e][nfpts][nv] */
    double *comm = uf + ne * nfpts * nv;                    /* [e][nfpts][nv] */
    double *gf = comm + ne * nfpts * nv;                    /* [e][nd*nfpts][nv] */

    flux_point_states(d, navier_stokes, u, uf, comm);

    if (navier_stokes) {

        /* Corrected gradient, flux, gradients at the flux points, divergence */
        #pragma omp parallel
        {
            double *g = malloc(sizeof(double) * nd * nupts * nv);
            double *F = malloc(sizeof(double) * nd * nupts * nv);
            #pragma omp for schedule(static)
            for (int64_t e = 0; e < ne; e++) {
                const double *ue = u + e * nupts * nv;
                csr_apply(&d->M460, ue, g, nv, 0);
                csr_apply(&d->M6, comm + e * nfpts * nv, g, nv, 1);
                for (int p = 0; p < nupts; p++) {
                    const double *S = d->smats + (e * nupts + p) * nd * nd;
                    const double rj = d->rcpdjac[e * nupts + p];
                    double tg[MAXD][MAXV], pg[MAXD][MAXV], f[MAXD][MAXV], pp, vel[MAXD];
                    for (int k = 0; k < nd; k++)
                        for (int v = 0; v < nv; v++) tg[k][v] = g[((int64_t)k * nupts + p) * nv + v];
                    for (int i = 0; i < nd; i++)
                        for (int v = 0; v < nv; v++) {
                            double acc = 0;
                            for (int k = 0; k < nd; k++) acc += S[k * nd + i] * tg[k][v];
                            pg[i][v] = rj * acc;
                            g[((int64_t)i * nupts + p) * nv + v] = pg[i][v];
                        }
                    inviscid_flux(nd, ue + p * nv, f, &pp, vel, d->gamma);
                    viscous_flux_add(nd, ue + p * nv, pg, f, d);
                    transform_store(d, S, f, F, p);
                }
                for (int k = 0; k < nd; k++)
                    csr_apply(&d->M0, g + (int64_t)k * nupts * nv,
                              gf + (e * nd * nfpts + (int64_t)k * nfpts) * nv, nv, 0);
                csr_apply(&d->M132, F, r + e * nupts * nv, nv, 0);
            }
            free(g);
            free(F);
        }

        /* Common flux (Riemann + LDG viscous) */
        #pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < d->npairs; i++) {
            double *ul = uf + (d->le[i] * nfpts + d->lpt[i]) * nv;
            double *ur = uf + (d->re[i] * nfpts + d->rpt[i]) * nv;
            double n[MAXD], mag, fi[MAXV], fvl[MAXD][MAXV] = {{0}}, fvr[MAXD][MAXV] = {{0}};
            double gl[MAXD][MAXV], gr[MAXD][MAXV];
            unit_normal(d, i, n, &mag);
            rsolve(nd, ul, ur, n, fi, d);
            for (int k = 0; k < nd; k++)
                for (int v = 0; v < nv; v++) {
                    gl[k][v] = gf[(d->le[i] * nd * nfpts + (int64_t)k * nfpts + d->lpt[i]) * nv + v];
                    gr[k][v] = gf[(d->re[i] * nd * nfpts + (int64_t)k * nfpts + d->rpt[i]) * nv + v];
                }
            if (d->beta != -0.5) viscous_flux_add(nd, ul, gl, fvl, d);
            if (d->beta != 0.5) viscous_flux_add(nd, ur, gr, fvr, d);
            for (int v = 0; v < nv; v++) {
                double nfl = 0, nfr = 0, fvc;
                for (int k = 0; k < nd; k++) {
                    nfl += n[k] * fvl[k][v];
                    nfr += n[k] * fvr[k][v];
                }
                if (d->beta == -0.5) fvc = nfr;
                else if (d->beta == 0.5) fvc = nfl;
                else fvc = (0.5 + d->beta) * nfl + (0.5 - d->beta) * nfr;
                fvc += d->tau * (ul[v] - ur[v]);
                const double c = fi[v] + fvc;
                ul[v] = mag * c;
                ur[v] = -mag * c;
            }
        }
    } else {
        /* Euler: common flux, then flux and divergence */
        #pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < d->npairs; i++) {
            double *ul = uf + (d->le[i] * nfpts + d->lpt[i]) * nv;
            double *ur = uf + (d->re[i] * nfpts + d->rpt[i]) * nv;
            double n[MAXD], mag, fn[MAXV];
            unit_normal(d, i, n, &mag);
            rsolve(nd, ul, ur, n, fn, d);
            for (int v = 0; v < nv; v++) {
                ul[v] = mag * fn[v];
                ur[v] = -mag * fn[v];
            }
        }

        #pragma omp parallel
        {
            double *F = malloc(sizeof(double) * nd * nupts * nv);
            #pragma omp for schedule(static)
            for (int64_t e = 0; e < ne; e++) {
                const double *ue = u + e * nupts * nv;
                for (int p = 0; p < nupts; p++) {
                    double f[MAXD][MAXV], pp, vel[MAXD];
                    inviscid_flux(nd, ue + p * nv, f, &pp, vel, d->gamma);
                    transform_store(d, d->smats + (e * nupts + p) * nd * nd, f, F, p);
                }
                csr_apply(&d->M132, F, r + e * nupts * nv, nv, 0);
            }
            free(F);
        }
    }

    /* Correction and physical divergence */
    #pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < ne; e++) {
        double *re_ = r + e * nupts * nv;
        csr_apply(&d->M3, uf + e * nfpts * nv, re_, nv, 1);
        for (int p = 0; p < nupts; p++) {
            const double rj = d->rcpdjac[e * nupts + p];
            for (int v = 0; v < nv; v++) re_[p * nv + v] = -rj * re_[p * nv + v];
        }
    }
    return 0;
}
