"""CPU oracle for the flux-reconstruction right-hand side and RK45 stages.

TEST INFRASTRUCTURE ONLY: this module is the checker that the CUDA path
is compared against.  It is imported by ``tests/``, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU baseline leg, never by
the product package.

It restates, in plain numpy on a simple (npts, nvars, neles) layout, the
arithmetic of the reference's OpenMP/CUDA kernels on this path:

  operator applies (mul)     pyfr/solvers/baseadvec/elements.py:73-100,
                             pyfr/solvers/baseadvecdiff/elements.py:48-101
  Euler flux / tflux         pyfr/solvers/euler/kernels/flux.mako:3-26,
                             pyfr/solvers/euler/kernels/tflux.mako:8-30
  Rusanov / HLLC             pyfr/solvers/euler/kernels/rsolvers/rusanov.mako:4-26,
                             pyfr/solvers/euler/kernels/rsolvers/hllc.mako:4-77
  intcflux (Euler, NS)       pyfr/solvers/euler/kernels/intcflux.mako:6-22,
                             pyfr/solvers/navstokes/kernels/intcflux.mako:10-54
  intconu                    pyfr/solvers/navstokes/kernels/intconu.mako:4-19
  viscous flux               pyfr/solvers/navstokes/kernels/flux.mako:48-105
  gradient transform         pyfr/solvers/baseadvecdiff/kernels/transform_grad.mako:3-10
  negdivconf                 pyfr/solvers/baseadvec/kernels/negdivconf.mako:7-22
  source terms               pyfr/plugins/kernels/source.mako:3-7,
                             pyfr/plugins/source.py:15-31
  flux anti-aliasing         pyfr/solvers/baseadvec/elements.py:79-90
  rkvdh2 / RK45              pyfr/integrators/explicit/kernels/rkvdh2.mako:4-31,
                             pyfr/integrators/explicit/steppers.py:165-243
  graph order (Euler, NS)    pyfr/solvers/baseadvec/system.py:58-136,
                             pyfr/solvers/baseadvecdiff/system.py:54-231
  linear element geometry    pyfr/shapes.py:306-566 (interp_expr, jac_exprs)
  wave speed (CFL)           pyfr/solvers/euler/kernels/wavespeed.mako:9-44,
                             pyfr/integrators/controllers.py:22-26

Everything the oracle needs about the discretisation is passed in: the
operator matrices (tests feed the ones generated by the reference's own
``pyfr/shapes.py``, see tests/golden/make_golden.py), the element
vertices, the interface connectivity and the reference element's points.
Flux points of the two sides of an interface are paired here by matching
physical coordinates (modulo the mesh periods), an algorithm independent
of the sort-based pairing the product uses.

Pinning: the operator matrices are checked against the reference's
golden file ``pyfr/tests/hex-gleg-ord3.npz`` and against matrices generated
by the reference itself; the pointwise kernel arithmetic has no golden
vectors in the reference (parity of that part rests on this restatement
plus invariants: free-stream preservation, conservation, Riemann
consistency and the exact advected vortex).
"""

import numpy as np


# ---------------------------------------------------------------------------
# Physics
# ---------------------------------------------------------------------------

def inviscid_flux(u, gamma):
    """u: (nvars, ...) -> F: (ndims, nvars, ...), p, v (ndims, ...)."""
    nv = u.shape[0]
    nd = nv - 2
    rho, E = u[0], u[-1]
    invrho = 1.0/rho
    rhov = u[1:nd + 1]
    v = invrho*rhov
    p = (gamma - 1)*(E - 0.5*invrho*np.sum(rhov*rhov, axis=0))
    f = np.empty((nd,) + u.shape)
    for i in range(nd):
        f[i, 0] = rhov[i]
        f[i, -1] = (E + p)*v[i]
        for j in range(nd):
            f[i, j + 1] = rhov[i]*v[j] + (p if i == j else 0)
    return f, p, v


def viscous_flux(u, grad, c):
    """Negated-stress viscous flux; grad: (ndims, nvars, ...)."""
    nv = u.shape[0]
    nd = nv - 2
    rho, E = u[0], u[-1]
    rcprho = 1.0/rho
    vel = rcprho*u[1:nd + 1]
    dv = np.array([[grad[d, i + 1] - vel[i]*grad[d, 0] for d in range(nd)]
                   for i in range(nd)])

    if c.get('sutherland', False):
        cpT = c['gamma']*(rcprho*E - 0.5*np.sum(vel*vel, axis=0))
        Trat = cpT/c['cpTref']
        mu = c['mu']*(c['cpTref'] + c['cpTs'])*Trat*np.sqrt(Trat)/(cpT + c['cpTs'])
    else:
        mu = c['mu']

    dT = np.array([rcprho*(grad[d, -1] - (rcprho*grad[d, 0]*E +
                                          sum(vel[i]*dv[i, d] for i in range(nd))))
                   for d in range(nd)])
    div = sum(dv[i, i] for i in range(nd))
    tau = np.empty((nd, nd) + rho.shape)
    for i in range(nd):
        tau[i, i] = -2*mu*rcprho*(dv[i, i] - div/3.0)
        for j in range(i + 1, nd):
            tau[i, j] = tau[j, i] = -mu*rcprho*(dv[j, i] + dv[i, j])

    f = np.zeros((nd, nv) + rho.shape)
    for d in range(nd):
        for i in range(nd):
            f[d, i + 1] = tau[i, d]
        f[d, -1] = sum(vel[i]*tau[i, d] for i in range(nd)) \
            - mu*c['gamma']/c['Pr']*dT[d]
    return f


def rusanov(ul, ur, n, gamma):
    fl, pl, vl = inviscid_flux(ul, gamma)
    fr, pr, vr = inviscid_flux(ur, gamma)
    nv = np.sum(n*(vl + vr), axis=0)
    a = np.sqrt(0.25*gamma*(pl + pr)/(ul[0] + ur[0])) + 0.25*np.abs(nv)
    return 0.5*np.einsum('d...,dv...->v...', n, fl + fr) + a*(ul - ur)


def hllc(ul, ur, n, gamma):
    nvars = ul.shape[0]
    fl, pl, vl = inviscid_flux(ul, gamma)
    fr, pr, vr = inviscid_flux(ur, gamma)
    nvl, nvr = np.sum(n*vl, axis=0), np.sum(n*vr, axis=0)
    al, ar = np.sqrt(gamma*pl/ul[0]), np.sqrt(gamma*pr/ur[0])
    sql, sqr = np.sqrt(ul[0]), np.sqrt(ur[0])
    nvroe = (sql*nvl + sqr*nvr)/(sql + sqr)
    H = (sql*(pr + ur[-1]) + sqr*(pl + ul[-1]))/(sql*ur[0] + sqr*ul[0])
    va = (vl*sql + vr*sqr)/(sql + sqr)
    a = np.sqrt((gamma - 1)*(H - 0.5*np.sum(va*va, axis=0)))
    sl = np.minimum(nvroe - a, nvl - al)
    sr = np.maximum(nvroe + a, nvr + ar)
    ss = (pr - pl + ul[0]*nvl*(sl - nvl) - ur[0]*nvr*(sr - nvr)) / \
         (ul[0]*(sl - nvl) - ur[0]*(sr - nvr))
    lc, rc = (sl - nvl)/(sl - ss), (sr - nvr)/(sr - ss)

    usl, usr = np.empty_like(ul), np.empty_like(ur)
    usl[0], usr[0] = lc*ul[0], rc*ur[0]
    for i in range(nvars - 2):
        usl[i + 1] = usl[0]*(vl[i] + (ss - nvl)*n[i])
        usr[i + 1] = usr[0]*(vr[i] + (ss - nvr)*n[i])
    usl[-1] = lc*(ul[-1] + (ss - nvl)*(ul[0]*ss + pl/(sl - nvl)))
    usr[-1] = rc*(ur[-1] + (ss - nvr)*(ur[0]*ss + pr/(sr - nvr)))

    nfl = np.einsum('d...,dv...->v...', n, fl)
    nfr = np.einsum('d...,dv...->v...', n, fr)
    nfsl = nfl + sl*(usl - ul)
    nfsr = nfr + sr*(usr - ur)
    return np.where(0 <= sl, nfl,
                    np.where((sl <= 0) & (0 <= ss), nfsl,
                             np.where((ss <= 0) & (0 <= sr), nfsr, nfr)))


def _nflux(n, f):
    return np.einsum('d...,dv...->v...', n, f)


def _roe_avg(ul, ur, vl, vr, pl, pr):
    """Roe averages shared by HLL and HLLC: normal speed, enthalpy and
    velocity (pyfr/solvers/euler/kernels/rsolvers/hll.mako:21-36)."""
    sql, sqr = np.sqrt(ul[0]), np.sqrt(ur[0])
    H = (sql*(pr + ur[-1]) + sqr*(pl + ul[-1]))/(sql*ur[0] + sqr*ul[0])
    va = (vl*sql + vr*sqr)*(1/(sql + sqr))
    return sql, sqr, H, va


def hll(ul, ur, n, gamma):
    """HLL flux (pyfr/solvers/euler/kernels/rsolvers/hll.mako:4-53)."""
    fl, pl, vl = inviscid_flux(ul, gamma)
    fr, pr, vr = inviscid_flux(ur, gamma)
    nvl, nvr = np.sum(n*vl, axis=0), np.sum(n*vr, axis=0)
    ar = np.sqrt(gamma*pr/ur[0])
    sql, sqr, H, va = _roe_avg(ul, ur, vl, vr, pl, pr)
    nv = (sql*nvl + sqr*nvr)/(sql + sqr)
    a = np.sqrt((gamma - 1)*(H - 0.5*np.sum(va*va, axis=0)))
    # The reference takes the right state's sound speed on both sides
    sl = np.minimum(nv - a, nvl - ar)
    sr = np.maximum(nv + a, nvr + ar)
    nfl, nfr = _nflux(n, fl), _nflux(n, fr)
    sub = (sr*nfl - sl*nfr + sl*sr*(ur - ul))*(1/(sr - sl))
    return np.where(0 <= sl, nfl, np.where(0 >= sr, nfr, sub))


def _rot_to(n, u):
    """Momentum in the frame whose first axis is n (Moler and Hughes 1999;
    pyfr/solvers/baseadvec/kernels/transform.mako:5-38)."""
    t = u.copy()
    m = u[1:-1]
    if len(n) == 2:
        t[1] = n[0]*m[0] + n[1]*m[1]
        t[2] = n[0]*m[1] - n[1]*m[0]
        return t
    with np.errstate(all='ignore'):
        h1, h2, h3 = 1/(1 + n[0]), 1/(1 - n[1]), 1/(1 - n[2])
        a = (n[0]*m[0] + n[1]*m[1] + n[2]*m[2],
             (n[0] + h1*n[2]*n[2])*m[1] - n[1]*m[0] - h1*n[1]*n[2]*m[2],
             (n[0] + h1*n[1]*n[1])*m[2] - n[2]*m[0] - h1*n[1]*n[2]*m[1])
        b = (a[0],
             (1 - h2*n[0]*n[0])*m[0] + n[0]*m[1] - h2*n[0]*n[2]*m[2],
             n[2]*m[1] - h2*n[0]*n[2]*m[0] + (1 - h2*n[2]*n[2])*m[2])
        c = (a[0],
             (1 - h3*n[1]*n[1])*m[1] - h3*n[0]*n[1]*m[0] + n[1]*m[2],
             (1 - h3*n[0]*n[0])*m[0] - h3*n[0]*n[1]*m[1] + n[0]*m[2])
    ca, cb = np.abs(n[0]) < 0.99, np.abs(n[1]) < np.abs(n[2])
    for k in range(3):
        t[1 + k] = np.where(ca, a[k], np.where(cb, b[k], c[k]))
    return t


def _rot_from(n, t):
    """Inverse of _rot_to (transform.mako:41-75)."""
    u = t.copy()
    m = t[1:-1]
    if len(n) == 2:
        u[1] = n[0]*m[0] - n[1]*m[1]
        u[2] = n[1]*m[0] + n[0]*m[1]
        return u
    with np.errstate(all='ignore'):
        h1, h2, h3 = 1/(1 + n[0]), 1/(1 - n[1]), 1/(1 - n[2])
        a = (n[0]*m[0] - n[1]*m[1] - n[2]*m[2],
             n[1]*m[0] + (n[0] + h1*n[2]*n[2])*m[1] - h1*n[1]*n[2]*m[2],
             n[2]*m[0] - h1*n[1]*n[2]*m[1] + (n[0] + h1*n[1]*n[1])*m[2])
        b = (n[0]*m[0] + (1 - h2*n[0]*n[0])*m[1] - h2*n[0]*n[2]*m[2],
             n[1]*m[0] + n[0]*m[1] + n[2]*m[2],
             n[2]*m[0] - h2*n[0]*n[2]*m[1] + (1 - h2*n[2]*n[2])*m[2])
        c = (n[0]*m[0] - h3*n[0]*n[1]*m[1] + (1 - h3*n[0]*n[0])*m[2],
             n[1]*m[0] + (1 - h3*n[1]*n[1])*m[1] - h3*n[0]*n[1]*m[2],
             n[2]*m[0] + n[1]*m[1] + n[0]*m[2])
    ca, cb = np.abs(n[0]) < 0.99, np.abs(n[1]) < np.abs(n[2])
    for k in range(3):
        u[1 + k] = np.where(ca, a[k], np.where(cb, b[k], c[k]))
    return u


def _rsolve_rotated(solve1d, ul, ur, n, gamma):
    """A one-dimensional solver applied in the normal frame
    (pyfr/solvers/euler/kernels/rsolvers/rsolve1d.mako:5-22)."""
    return _rot_from(n, solve1d(_rot_to(n, ul), _rot_to(n, ur), gamma))


def _flux_1d(s, gamma):
    """x-direction flux of a rotated state (flux.mako:28-48)."""
    nd = s.shape[0] - 2
    invrho, E = 1/s[0], s[-1]
    v = invrho*s[1:nd + 1]
    p = (gamma - 1)*(E - 0.5*invrho*np.sum(s[1:nd + 1]**2, axis=0))
    f = np.empty_like(s)
    f[0] = s[1]
    f[-1] = (E + p)*v[0]
    f[1] = s[1]*v[0] + p
    for j in range(1, nd):
        f[j + 1] = s[1]*v[j]
    return f, p, v


def roe_1d(ul, ur, gamma, eps=0.001):
    """Roe flux with the entropy fix of
    pyfr/solvers/euler/kernels/rsolvers/roe.mako:6-84."""
    nd = ul.shape[0] - 2
    fl, pl, vl = _flux_1d(ul, gamma)
    fr, pr, vr = _flux_1d(ur, gamma)
    sql, sqr = np.sqrt(ul[0]), np.sqrt(ur[0])
    roa = sql*sqr
    ha = (sql*(pr + ur[-1]) + sqr*(pl + ul[-1]))/(sql*ur[0] + sqr*ul[0])
    va = (vl*sql + vr*sqr)*(1/(sql + sqr))
    qq = np.sum(va*va, axis=0)
    a = np.sqrt((gamma - 1)*(ha - 0.5*qq))
    l1, l2, l3 = np.abs(va[0] - a), np.abs(va[0]), np.abs(va[0] + a)
    l1 = np.where(l1 < eps, (0.5/eps)*(l1*l1 + eps**2), l1)
    l3 = np.where(l3 < eps, (0.5/eps)*(l3*l3 + eps**2), l3)
    dv = vr - vl
    dro, dp = ur[0] - ul[0], pr - pl
    ia2 = 1/(2*a*a)
    w1 = (dp - roa*a*dv[0])*ia2
    w2 = dro - dp*2*ia2
    w3 = (dp + roa*a*dv[0])*ia2
    nf = np.empty_like(ul)
    nf[0] = 0.5*(fl[0] + fr[0]) - (l1*w1 + l2*w2 + l3*w3)
    for i in range(nd):
        if i == 0:
            v1, v2, v3 = w1*(va[0] - a), w2*va[0], w3*(va[0] + a)
        else:
            v1, v2, v3 = w1*va[i], w2*va[i] + roa*dv[i], w3*va[i]
        nf[i + 1] = 0.5*(fl[i + 1] + fr[i + 1]) - (l1*v1 + l2*v2 + l3*v3)
    v1 = w1*(ha - a*va[0])
    v2 = roa*(np.sum(va*dv, axis=0) - va[0]*dv[0]) + w2*qq*0.5
    v3 = w3*(ha + a*va[0])
    nf[-1] = 0.5*(fl[-1] + fr[-1]) - (l1*v1 + l2*v2 + l3*v3)
    return nf


def roe(ul, ur, n, gamma):
    return _rsolve_rotated(roe_1d, ul, ur, n, gamma)


def roem(ul, ur, n, gamma):
    """RoeM flux (Kim, Kim and Rho, JCP 185(2), 2003;
    pyfr/solvers/euler/kernels/rsolvers/roem.mako:5-96)."""
    fl, pl, vl = inviscid_flux(ul, gamma)
    fr, pr, vr = inviscid_flux(ur, gamma)
    hl, hr = (ul[-1] + pl)/ul[0], (ur[-1] + pr)/ur[0]
    cl, cr = np.sum(n*vl, axis=0), np.sum(n*vr, axis=0)
    drho, dp, dh, dc = ur[0] - ul[0], pr - pl, hr - hl, cr - cl
    dv = vr - vl
    rrr = np.sqrt(ur[0]/ul[0])
    ratl = 1.0/(1.0 + rrr)
    ratr = rrr*ratl
    ra = rrr*ul[0]
    ha = hl*ratl + hr*ratr
    va = vl*ratl + vr*ratr
    qq = np.sum(va*va, axis=0)
    ca = np.sum(n*va, axis=0)
    aa = np.sqrt((gamma - 1)*(ha - 0.5*qq))
    rcp_aa = 1.0/aa
    abs_ma = np.abs(ca*rcp_aa) + 1e-15
    b1 = np.maximum(0.0, np.maximum(ca + aa, cr + aa))
    b2 = np.minimum(0.0, np.minimum(ca - aa, cl - aa))
    b1b2 = b1*b2
    rb = 1.0/(b1 - b2)
    b1, b2, b1b2 = b1*rb, b2*rb, b1b2*rb
    sdst = np.where(pl < pr, pl/pr, pr/pl)
    f = abs_ma**(1.0 - sdst)
    g = f/(1.0 + abs_ma)
    du = ur - ul
    du[-1] = ur[0]*hr - ul[0]*hl
    bdq = np.empty_like(ul)
    bdq[0] = drho - f*dp*rcp_aa*rcp_aa
    bdq[-1] = bdq[0]*ha + ra*dh
    for i in range(len(n)):
        bdq[i + 1] = bdq[0]*va[i] + ra*(dv[i] - n[i]*dc)
    return _nflux(n, b1*fl - b2*fr) + b1b2*(du - g*bdq)


def exact_1d(ul, ur, gamma, p_min):
    """Exact Riemann solution sampled at x/t = 0, three Newton iterations
    from the adaptive initial guess (Toro 2009, ch. 4 and 9;
    pyfr/solvers/euler/kernels/rsolvers/exact.mako:14-185)."""
    nd = ul.shape[0] - 2
    g = gamma
    hgm, grgm, trgm, trgp = 0.5*(g - 1), g/(g - 1), 2/(g - 1), 2/(g + 1)
    gmrtg, gprtg = (g - 1)/(2*g), (g + 1)/(2*g)
    tgrgm, gmrgp = 2*g/(g - 1), (g - 1)/(g + 1)

    def prim(s):
        inv = 1/s[0]
        v = inv*s[1:nd + 1]
        p = (g - 1)*(s[-1] - 0.5*inv*np.sum(s[1:nd + 1]**2, axis=0))
        return p, v, np.sqrt(g*p*inv)

    def star(p, ps, rs, cs):
        with np.errstate(all='ignore'):
            pr = p/ps
            prg = pr**(-gprtg)
            fd1, f1 = prg/(rs*cs), trgm*cs*(prg*pr - 1)
            pbs = 1/(p + gmrgp*ps)
            sapb = np.sqrt(trgp*pbs/rs)
            f2 = (p - ps)*sapb
            fd2 = sapb - 0.5*f2*pbs
        return np.where(p <= ps, f1, f2), np.where(p <= ps, fd1, fd2)

    pl, vl, cl = prim(ul)
    pr, vr, cr = prim(ur)
    rl, rr = ul[0], ur[0]
    with np.errstate(all='ignore'):
        bpv = np.maximum(0, 0.125*(vl[0] - vr[0])*(rl + rr)*(cl + cr) +
                         0.5*(pl + pr))
        pmin, pmax = np.minimum(pl, pr), np.maximum(pl, pr)
        pre = (pl/pr)**gmrtg
        um = (pre*vl[0]*cr + vr[0]*cl + trgm*(pre - 1)*cl*cr)/(pre*cr + cl)
        ptl = 1 - hgm*(um - vl[0])/cl
        ptr = 1 + hgm*(um - vr[0])/cr
        p_rr = 0.5*(pl*ptl**tgrgm + pr*ptr**tgrgm)
        gl = np.sqrt(trgp/(rl*(gmrgp*pl + bpv)))
        gr = np.sqrt(trgp/(rr*(gmrgp*pr + bpv)))
        p_ss = (gl*pl + gr*pr - vr[0] + vl[0])/(gl + gr)
    p0 = np.where((pmax <= 2*pmin) & (pmin <= bpv) & (bpv <= pmax), bpv,
                  np.where(bpv < pmin, p_rr, p_ss))

    for _ in range(3):
        fsl, fdl = star(p0, pl, rl, cl)
        fsr, fdr = star(p0, pr, rr, cr)
        p1 = p0 - (fsl + fsr + vr[0] - vl[0])/(fdl + fdr)
        p0 = np.where(p1 < 0, p_min, p1)
    us = 0.5*(vl[0] + vr[0] + fsr - fsl)

    with np.errstate(all='ignore'):
        # Left of the contact
        c_l = trgp + gmrgp*vl[0]/cl
        lfan = (rl*c_l**trgm, trgp*cl + gmrgp*vl[0], pl*c_l**tgrgm)
        lstar_r = (rl*(p0/pl)**(1/g), us, p0)
        lraref = np.where(vl[0] >= cl, 0,
                          np.where(us < cl*(p0/pl)**gmrtg, 1, 2))
        p0pl = p0/pl
        sl = vl[0] - cl*np.sqrt(gprtg*p0pl + gmrtg)
        lstar_s = (rl*(p0pl + gmrgp)/(p0pl*gmrgp + 1), us, p0)
        # Right of the contact
        c_r = trgp - gmrgp*vr[0]/cr
        rfan = (rr*c_r**trgm, gmrgp*vr[0] - trgp*cr, pr*c_r**tgrgm)
        p0pr = p0/pr
        sr = vr[0] + cr*np.sqrt(gprtg*p0pr + gmrtg)
        rstar_s = (rr*(p0pr + gmrgp)/(p0pr*gmrgp + 1), us, p0)
        rstar_r = (rr*p0pr**(1/g), us, p0)
        rraref = np.where(vr[0] + cr <= 0, 0,
                          np.where(us + cr*p0pr**gmrtg >= 0, 1, 2))

    lw = (rl, vl[0], pl)
    rw = (rr, vr[0], pr)
    w = []
    for k in range(3):
        left = np.where(p0 <= pl,
                        np.choose(lraref, [lw[k], lstar_r[k], lfan[k]]),
                        np.where(0 <= sl, lw[k], lstar_s[k]))
        right = np.where(p0 > pr,
                         np.where(sr <= 0, rw[k], rstar_s[k]),
                         np.choose(rraref, [rw[k], rstar_r[k], rfan[k]]))
        w.append(np.where(0 <= us, left, right))
    wt = [np.where(0 <= us, vl[i], vr[i]) for i in range(1, nd)]

    nf = np.empty_like(ul)
    nf[0] = w[0]*w[1]
    nf[1] = nf[0]*w[1] + w[2]
    for i, t in enumerate(wt):
        nf[i + 2] = nf[0]*t
    ke = w[1]**2 + sum(t**2 for t in wt)
    nf[-1] = (grgm*w[2] + 0.5*w[0]*ke)*w[1]
    return nf


def exact(ul, ur, n, gamma, p_min=5*np.finfo(float).eps):
    return _rsolve_rotated(lambda a, b, g: exact_1d(a, b, g, p_min), ul, ur,
                           n, gamma)


RSOLVERS = {'rusanov': rusanov, 'hllc': hllc, 'hll': hll, 'roe': roe,
            'roem': roem, 'exact': exact}


# ---------------------------------------------------------------------------
# Boundary conditions
# ---------------------------------------------------------------------------

def _uvw(bc, nd, npts):
    """The boundary velocity (ndims, npts): constants or per-point
    values."""
    u = bc.get('u', [0.0]*3)[:nd]
    return np.stack([np.broadcast_to(np.asarray(v, dtype=float), (npts,))
                     for v in u])


def bc_rsolve_state(bc, ul, n, gamma):
    """Ghost state of the boundary Riemann solve; ul (nvars, npts), n unit
    normals (ndims, npts).  pyfr/solvers/euler/kernels/bcs/*.mako and
    pyfr/solvers/navstokes/kernels/bcs/no-slp-*.mako (bc_rsolve_state)."""
    nd = ul.shape[0] - 2
    t = bc['type']
    ur = np.empty_like(ul)
    gm1 = gamma - 1
    uvw = _uvw(bc, nd, ul.shape[1])
    if t == 'sup-in-fa':
        ur[0] = bc['rho']
        ur[1:nd + 1] = bc['rho']*uvw
        ur[-1] = bc['p']/gm1 + 0.5*np.sum(ur[1:nd + 1]**2, axis=0)/ur[0]
    elif t == 'sup-out-fn':
        ur[:] = ul
    elif t == 'slp-adia-wall':
        nor = np.sum(ul[1:nd + 1]*n, axis=0)
        ur[0], ur[-1] = ul[0], ul[-1]
        ur[1:nd + 1] = ul[1:nd + 1] - 2*nor*n
    elif t == 'char-riem-inv':
        rho_e, p_e = bc['rho'], bc['p']
        cs = np.sqrt(gamma*p_e/rho_e)
        se = p_e*rho_e**-gamma
        ratio = 2*cs/gm1
        inv = 1/ul[0]
        ve = np.sum(uvw*n, axis=0)
        vi = inv*np.sum(ul[1:nd + 1]*n, axis=0)
        pi = gm1*ul[-1] - 0.5*gm1*inv*np.sum(ul[1:nd + 1]**2, axis=0)
        ci = np.sqrt(gamma*pi*inv)
        sup = np.abs(ve) >= cs
        re = np.where(sup & (vi >= 0), vi - 2*ci/gm1, ve - ratio)
        ri = np.where(sup & (vi < 0), ve + ratio, vi + 2*ci/gm1)
        vb, cb = 0.5*(re + ri), 0.25*gm1*(ri - re)
        rhob = np.where(vi < 0, (cb*cb/(gamma*se))**(1/gm1),
                        ul[0]*(ul[0]*cb*cb/(gamma*pi))**(1/gm1))
        pb = rhob*cb*cb/gamma
        ur[0] = rhob
        ur[1:nd + 1] = np.where(vi >= 0,
                                rhob*(ul[1:nd + 1]*inv + (vb - vi)*n),
                                rhob*(uvw + (vb - ve)*n))
        ur[-1] = pb/gm1 + 0.5*np.sum(ur[1:nd + 1]**2, axis=0)/ur[0]
    elif t == 'no-slp-adia-wall':
        ur[0], ur[-1] = ul[0], ul[-1]
        ur[1:nd + 1] = -ul[1:nd + 1]
    elif t == 'no-slp-isot-wall':
        ur[0] = ul[0]
        ur[1:nd + 1] = -ul[1:nd + 1] + 2*uvw*ul[0]
        ur[-1] = bc['cpTw']/gamma*ur[0] + \
            0.5*np.sum(ur[1:nd + 1]**2, axis=0)/ur[0]
    elif t == 'sub-in-frv':
        ur[0] = bc['rho']
        ur[1:nd + 1] = bc['rho']*uvw
        ur[-1] = ul[-1] - 0.5*np.sum(ul[1:nd + 1]**2, axis=0)/ul[0] + \
            0.5*np.sum(ur[1:nd + 1]**2, axis=0)/ur[0]
    elif t == 'sub-in-ftpttang':
        rdcp = gm1/gamma
        vc = np.array(bc['vc'][:nd])[:, None]
        pl = gm1*(ul[-1] - 0.5/ul[0]*np.sum(ul[1:nd + 1]**2, axis=0))
        udotu = np.maximum(0, 2*bc['cpTt']*(1 - bc['pt']**-rdcp*pl**rdcp))
        ur[0] = pl/(rdcp*(bc['cpTt'] - 0.5*udotu))
        ur[1:nd + 1] = vc*ur[0]*np.sqrt(udotu)
        ur[-1] = pl/gm1 + 0.5*ur[0]*udotu
    elif t == 'sub-out-fp':
        ur[:-1] = ul[:-1]
        ur[-1] = bc['p']/gm1 + 0.5*np.sum(ul[1:nd + 1]**2, axis=0)/ul[0]
    else:
        raise ValueError(t)
    return ur


def bc_ldg_state(bc, ul, n, gamma):
    """Boundary state of the LDG common solution (bc_ldg_state of
    pyfr/solvers/navstokes/kernels/bcs/*.mako)."""
    nd = ul.shape[0] - 2
    t = bc['type']
    if t == 'no-slp-adia-wall':
        ur = np.empty_like(ul)
        ur[0] = ul[0]
        ur[1:nd + 1] = 0
        ur[-1] = ul[-1] - 0.5/ul[0]*np.sum(ul[1:nd + 1]**2, axis=0)
        return ur
    if t == 'no-slp-isot-wall':
        uvw = _uvw(bc, nd, ul.shape[1])
        ur = np.empty_like(ul)
        ur[0] = ul[0]
        ur[1:nd + 1] = uvw*ul[0]
        ur[-1] = bc['cpTw']/gamma*ur[0] + \
            0.5*np.sum(ur[1:nd + 1]**2, axis=0)/ur[0]
        return ur
    return bc_rsolve_state(bc, ul, n, gamma)


def bc_ldg_grad_state(bc, us, n, gl):
    """Boundary gradient (bc_ldg_grad_state); gl (ndims, nvars, npts)."""
    t = bc['type']
    if t in ('sup-in-fa', 'char-riem-inv', 'sub-in-frv', 'sub-out-fp'):
        return np.zeros_like(gl)
    gr = gl.copy()
    if t == 'no-slp-adia-wall':
        nd = gl.shape[0]
        rcprho = 1/us[0]
        vel = rcprho*us[1:nd + 1]
        tl = np.empty((nd,) + us.shape[1:])
        for d in range(nd):
            kd = sum(vel[i]*(gl[d, i + 1] - vel[i]*gl[d, 0])
                     for i in range(nd))
            tl[d] = gl[d, -1] - (rcprho*gl[d, 0]*us[-1] + kd)
        for d in range(nd):
            gr[d, -1] -= sum(n[d]*n[e]*tl[e] for e in range(nd))
    return gr


def bc_flux_ns(bc, ul, gl, n, c, rsolver, av=None):
    """Common normal flux at a boundary (per unit normal): ghost,
    ghost-imperm or slip-wall flux state of
    pyfr/solvers/navstokes/kernels/bcs/{ghost,ghost-imperm,slp-adia-wall}
    .mako; av: the artificial viscosity at the points (or None)."""
    gamma, tau = c['gamma'], c['ldg-tau']
    t = bc['type']
    ur = bc_rsolve_state(bc, ul, n, gamma)
    fi = RSOLVERS[rsolver](ul, ur, n, gamma)
    if t == 'slp-adia-wall':
        return fi
    imperm = t in ('no-slp-adia-wall', 'no-slp-isot-wall')
    ul_dg = bc_ldg_state(bc, ul, n, gamma)
    gr = bc_ldg_grad_state(bc, ul_dg if imperm else ul, n, gl)
    fvs = viscous_flux(ul_dg, gr, c)
    if av is not None:
        fvs = fvs - av*gr
    fv = np.einsum('dn,dvn->vn', n, fvs)
    if not imperm:
        fv = fv + tau*(ul - ur)
    return fi + fv


# ---------------------------------------------------------------------------
# Geometry of linear elements
# ---------------------------------------------------------------------------

def vertex_signs(ndims):
    return np.array([[1.0 if (v >> d) & 1 else -1.0 for d in range(ndims)]
                     for v in range(2**ndims)])


def shape_values(pts, ndims):
    s = vertex_signs(ndims)
    return np.prod(1 + pts[:, None, :]*s[None], axis=2)/2**ndims


def jacobian(verts, pts):
    """J[p, i, j, e] = dX_j/dxi_i for linear elements; verts (nv, ne, nd)."""
    nd = verts.shape[2]
    s = vertex_signs(nd)
    dN = np.empty((len(pts), nd, len(s)))
    for i in range(nd):
        t = np.ones((len(pts), len(s)))
        for d in range(nd):
            t = t*(s[None, :, d] if d == i else 1 + pts[:, None, d]*s[None, :, d])
        dN[:, i] = t/2**nd
    return np.einsum('piv,vej->pije', dN, verts)


def smats_djac(verts, pts):
    J = jacobian(verts, pts)
    nd = J.shape[1]
    s = np.empty_like(J)
    if nd == 2:
        s[:, 0, 0], s[:, 0, 1] = J[:, 1, 1], -J[:, 1, 0]
        s[:, 1, 0], s[:, 1, 1] = -J[:, 0, 1], J[:, 0, 0]
        d = s[:, 0, 0]*s[:, 1, 1] - s[:, 0, 1]*s[:, 1, 0]
    else:
        for i in range(3):
            a, b = (i + 1) % 3, (i + 2) % 3
            s[:, i] = np.cross(J[:, a], J[:, b], axisa=1, axisb=1, axisc=1)
        d = np.einsum('pje,pje->pe', J[:, 0], s[:, 0])
    return s, d


# ---------------------------------------------------------------------------
# Source terms
# ---------------------------------------------------------------------------

_SRC_FUNCS = {'sin': np.sin, 'cos': np.cos, 'tan': np.tan, 'exp': np.exp,
              'log': np.log, 'sqrt': np.sqrt, 'tanh': np.tanh,
              'sinh': np.sinh, 'cosh': np.cosh, 'asin': np.arcsin,
              'acos': np.arccos, 'atan': np.arctan, 'atan2': np.arctan2,
              'pow': np.power, 'fabs': np.abs, 'floor': np.floor,
              'ceil': np.ceil, 'min': np.minimum, 'max': np.maximum,
              'fmin': np.fmin, 'fmax': np.fmax}


def source_terms(exprs, t, u, ploc):
    """The source plugin's terms: src[i] = exprs[i] at every point
    (pyfr/plugins/kernels/source.mako:3-7 expanded in
    pyfr/solvers/baseadvec/kernels/negdivconf.mako:13-19).  ``exprs`` are
    the kernel's C expressions of ploc[j], u[j] and t (as the source plugin
    writes them, pyfr/plugins/source.py:15-24); u is (nvars, ...) and ploc
    (ndims, ...).  Variables past len(exprs) get no source."""
    env = dict(_SRC_FUNCS, ploc=ploc, u=u, t=t)
    out = np.zeros_like(np.asarray(u, dtype=float))
    for i, e in enumerate(exprs):
        out[i] = eval(compile(e, '<source>', 'eval'),
                      {'__builtins__': {}}, env)
    return out


# ---------------------------------------------------------------------------
# The discretisation
# ---------------------------------------------------------------------------

class Discretisation:
    """Everything the oracle RHS needs for one element type.

    ops: dict with 'M0', 'M132' (= M1 - M3*M2), 'M3', and for NS 'M460'
    (= M4 - M6*M0), 'M6'; basis: dict with 'upts', 'fpts', 'norm_fpts',
    'facefpts' (list of index lists); verts: (nverts, neles, ndims);
    lhs/rhs: arrays (ninters, 2) of (element, face); periods: per-dim
    period of the mesh (or None).
    """

    def __init__(self, ops, basis, verts, lhs, rhs, periods=None, aa=None,
                 bcs=()):
        self.ops = {k: np.asarray(v, dtype=float) for k, v in ops.items()}
        # Flux anti-aliasing (pyfr/solvers/baseadvec/elements.py:79-90):
        # aa = dict(M7=..., M1329=(M1 - M3 M2) M9, qpts=...)
        self.aa = None if aa is None else \
            {k: np.asarray(v, dtype=float) for k, v in aa.items()}
        self.upts = np.asarray(basis['upts'], dtype=float)
        self.fpts = np.asarray(basis['fpts'], dtype=float)
        self.norm_fpts = np.asarray(basis['norm_fpts'], dtype=float)
        self.facefpts = [np.asarray(f) for f in basis['facefpts']]
        self.verts = np.asarray(verts, dtype=float)
        self.nverts, self.neles, self.ndims = self.verts.shape
        self.nupts, self.nfpts = len(self.upts), len(self.fpts)

        # Metric terms at the solution and flux points
        self.smats_u, self.djac_u = smats_djac(self.verts, self.upts)
        if self.aa is not None:
            self.smats_q, _ = smats_djac(self.verts, self.aa['qpts'])
        s_f, _ = smats_djac(self.verts, self.fpts)
        # Scaled normals S^T n at the flux points: (nfpts, ndims, neles)
        self.pnorm = np.einsum('plke,pl->pke', s_f, self.norm_fpts)
        self.ploc_f = np.einsum('pv,ved->pde',
                                shape_values(self.fpts, self.ndims), self.verts)

        self.faces_l, self.faces_r = np.asarray(lhs), np.asarray(rhs)
        self._pair(np.asarray(lhs), np.asarray(rhs), periods)

        # Boundaries: bcs is a sequence of (faces (n, 2) of (element, face),
        # boundary spec dict)
        self.bcs = []
        for faces, spec in bcs:
            faces = np.asarray(faces)
            fp = np.concatenate([self.facefpts[f] for _, f in faces])
            ee = np.concatenate([np.full(len(self.facefpts[f]), e)
                                 for e, f in faces])
            nl = self.pnorm[fp, :, ee].T                       # (nd, n)
            mag = np.sqrt(np.sum(nl**2, axis=0))
            self.bcs.append((fp, ee, nl/mag, mag, spec))

    def _bcs_at(self, t):
        """The boundaries with any value that is a function of (x, t)
        (x: (ndims, npts) coordinates of the boundary's points) evaluated
        at time t (expressions of pyfr/solvers/baseadvec/inters.py:95-116)."""
        out = []
        for fp, ee, n, mag, spec in self.bcs:
            if any(callable(v) for v in spec.values()) or \
                    any(callable(v) for v in spec.get('u', [])):
                x = self.ploc_f[fp, :, ee].T
                ev = dict(spec)
                for k, v in spec.items():
                    if callable(v):
                        ev[k] = v(x, t)
                if 'u' in spec:
                    ev['u'] = [v(x, t) if callable(v) else v
                               for v in spec['u']]
                spec = ev
            out.append((fp, ee, n, mag, spec))
        return out

    def _pair(self, lhs, rhs, periods):
        """Pair the flux points of the two sides of every interface by
        matching physical coordinates (modulo periods)."""
        # Interfaces are processed in batches sharing (left face, right face)
        nint = len(lhs)
        nfp = len(self.facefpts[0])
        li = np.empty((nint, nfp, 2), dtype=np.int64)
        ri = np.empty((nint, nfp, 2), dtype=np.int64)
        keys = lhs[:, 1]*64 + rhs[:, 1]
        for key in np.unique(keys):
            idx = np.flatnonzero(keys == key)
            fl, fr = lhs[idx[0], 1], rhs[idx[0], 1]
            el, er = lhs[idx, 0], rhs[idx, 0]
            pl = np.asarray(self.facefpts[fl])
            pr = np.asarray(self.facefpts[fr])
            xl = self.ploc_f[pl][:, :, el]                    # (nfp, nd, n)
            xr = self.ploc_f[pr][:, :, er]
            d = xl[:, None] - xr[None, :]                     # (nfp, nfp, nd, n)
            if periods is not None:
                for k, P in enumerate(periods):
                    if P is not None:
                        d[:, :, k] -= P*np.rint(d[:, :, k]/P)
            match = np.argmin(np.sum(d*d, axis=2), axis=1)    # (nfp, n)
            if np.any(np.sort(match, axis=0) != np.arange(nfp)[:, None]):
                raise RuntimeError('Flux points of an interface do not pair')
            li[idx, :, 0] = pl[None, :]
            li[idx, :, 1] = el[:, None]
            ri[idx, :, 0] = pr[match.T]
            ri[idx, :, 1] = er[:, None]

        self.pl = li.reshape(-1, 2)
        self.pr = ri.reshape(-1, 2)
        self.nl = self.pnorm[self.pl[:, 0], :, self.pl[:, 1]].T   # (nd, n)

    # ---- operator applies ---------------------------------------------------

    @staticmethod
    def apply(op, x):
        """op (m, k) @ x (k, nvars, neles) -> (m, nvars, neles)."""
        return np.einsum('mk,kve->mve', op, x)

    def _gather(self, fld, side):
        p = self.pl if side == 'l' else self.pr
        return fld[p[:, 0], :, p[:, 1]].T                        # (nvars, n)

    def _scatter(self, fld, side, vals):
        p = self.pl if side == 'l' else self.pr
        fld[p[:, 0], :, p[:, 1]] = vals.T

    # ---- right-hand sides ----------------------------------------------------

    def _transform_flux(self, f):
        # f: (ndims, nupts, nvars, neles) physical -> reference (smats)
        return np.einsum('pike,kpve->ipve', self.smats_u, f)

    @property
    def ploc_upts(self):
        """Physical coordinates of the solution points (nupts, ndims,
        neles)."""
        return np.einsum('pv,ved->pde',
                         shape_values(self.upts, self.ndims), self.verts)

    def _add_src(self, r, u, src, t):
        """r + the source terms ``src`` (expressions) at time t."""
        if not src:
            return r
        s = source_terms(src, t, u.transpose(1, 0, 2),
                         self.ploc_upts.transpose(1, 0, 2))
        return r + s.transpose(1, 0, 2)

    def rhs_euler(self, u, c, rsolver='rusanov', t=0.0, src=None):
        gamma = c['gamma']
        nd = self.ndims
        bcs = self._bcs_at(t)
        uf = self.apply(self.ops['M0'], u)

        # Common interface flux (intcflux)
        ul, ur = self._gather(uf, 'l'), self._gather(uf, 'r')
        mag = np.sqrt(np.sum(self.nl**2, axis=0))
        fn = RSOLVERS[rsolver](ul, ur, self.nl/mag, gamma)
        self._scatter(uf, 'l', mag*fn)
        self._scatter(uf, 'r', -mag*fn)

        # Boundary common fluxes (bccflux)
        for fp, ee, n, bmag, spec in bcs:
            ub = uf[fp, :, ee].T
            ug = bc_rsolve_state(spec, ub, n, gamma)
            uf[fp, :, ee] = (bmag*RSOLVERS[rsolver](ub, ug, n, gamma)).T

        # Transformed flux at the solution points (tflux), or at the
        # quadrature points and projected back
        if self.aa is not None:
            uq = self.apply(self.aa['M7'], u)
            fq, _, _ = inviscid_flux(uq.transpose(1, 0, 2), gamma)
            ft = np.einsum('pike,kpve->ipve', self.smats_q,
                           fq.transpose(0, 2, 1, 3))
            r = self.apply(self.aa['M1329'],
                           ft.reshape(nd*len(self.aa['qpts']), -1, self.neles))
            r += self.apply(self.ops['M3'], uf)
            return self._add_src(-r/self.djac_u[:, None, :], u, src, t)

        fp, _, _ = inviscid_flux(u.transpose(1, 0, 2), gamma)   # (nd, nv, p, e)
        ft = self._transform_flux(fp.transpose(0, 2, 1, 3))

        r = self.apply(self.ops['M132'], ft.reshape(nd*self.nupts, -1, self.neles))
        r += self.apply(self.ops['M3'], uf)
        return self._add_src(-r/self.djac_u[:, None, :], u, src, t)

    def rhs_ns(self, u, c, rsolver='rusanov', grads_out=None, av=None,
               t=0.0, src=None):
        """av: the artificial-viscosity parameters of shock_sensor and
        artvisc_points (pyfr/solvers/baseadvecdiff/artvisc.py), or None."""
        gamma, beta, tau = c['gamma'], c['ldg-beta'], c['ldg-tau']
        bcs = self._bcs_at(t)
        nd, nupts, nfpts, ne = self.ndims, self.nupts, self.nfpts, self.neles
        uf = self.apply(self.ops['M0'], u)
        if av is not None:
            avf, avu = artvisc_points(shock_sensor(u, av), av)

        # Common solution (intconu) on the flux points
        ul, ur = self._gather(uf, 'l'), self._gather(uf, 'r')
        if beta == -0.5:
            cl, cr = ul, ul
        elif beta == 0.5:
            cl, cr = ur, ur
        else:
            cl = cr = ur*(0.5 + beta) + ul*(0.5 - beta)
        comm = uf.copy()
        self._scatter(comm, 'l', cl)
        self._scatter(comm, 'r', cr)
        for fp, ee, n, bmag, spec in bcs:
            comm[fp, :, ee] = bc_ldg_state(spec, uf[fp, :, ee].T, n, gamma).T

        # Corrected reference gradient, transformed to physical space
        g = self.apply(self.ops['M460'], u) + self.apply(self.ops['M6'], comm)
        g = g.reshape(nd, nupts, -1, ne)
        g = np.einsum('pkie,kpve->ipve', self.smats_u, g)/self.djac_u[None, :, None, :]
        if grads_out is not None:
            grads_out.append(g)

        # Flux at the solution points or, with flux anti-aliasing, at the
        # quadrature points from the interpolated solution and physical
        # gradient (pyfr/solvers/baseadvecdiff/elements.py:103-116); the
        # artificial viscosity av['opu'] is then taken at those points
        if self.aa is not None:
            m7 = self.aa['M7']
            uq = self.apply(m7, u)
            gq = np.stack([self.apply(m7, g[d]) for d in range(nd)])
            ut, gt, sm = uq.transpose(1, 0, 2), gq.transpose(0, 2, 1, 3), \
                self.smats_q
        else:
            ut, gt, sm = u.transpose(1, 0, 2), g.transpose(0, 2, 1, 3), \
                self.smats_u
        fi, _, _ = inviscid_flux(ut, gamma)
        fv = viscous_flux(ut, gt, c)
        if av is not None:
            fv = fv - avu[None, None]*gt
        ft = np.einsum('pike,kpve->ipve', sm, (fi + fv).transpose(0, 2, 1, 3))

        # Physical gradient at the flux points and the common flux
        gf = np.stack([self.apply(self.ops['M0'], g[d]) for d in range(nd)])
        # Advanced indices split by a slice put the point axis first
        gl = gf[:, self.pl[:, 0], :, self.pl[:, 1]].transpose(1, 2, 0)
        gr = gf[:, self.pr[:, 0], :, self.pr[:, 1]].transpose(1, 2, 0)
        mag = np.sqrt(np.sum(self.nl**2, axis=0))
        n = self.nl/mag
        fic = RSOLVERS[rsolver](ul, ur, n, gamma)
        fvl_, fvr_ = viscous_flux(ul, gl, c), viscous_flux(ur, gr, c)
        if av is not None:
            # (the left side's viscosity for both sides)
            a = avf[self.pl[:, 0], self.pl[:, 1]]
            fvl_, fvr_ = fvl_ - a*gl, fvr_ - a*gr
        fvl = np.einsum('dn,dvn->vn', n, fvl_)
        fvr = np.einsum('dn,dvn->vn', n, fvr_)
        if beta == -0.5:
            fvc = fvr
        elif beta == 0.5:
            fvc = fvl
        else:
            fvc = (0.5 + beta)*fvl + (0.5 - beta)*fvr
        fvc = fvc + tau*(ul - ur)
        # (boundary states first: the interior scatter overwrites uf)
        bflux = []
        for fp, ee, n, bmag, spec in bcs:
            ub = uf[fp, :, ee].T
            gb = gf[:, fp, :, ee].transpose(1, 2, 0)
            ab = avf[fp, ee] if av is not None else None
            bflux.append(bmag*bc_flux_ns(spec, ub, gb, n, c, rsolver, ab))
        self._scatter(uf, 'l', mag*(fic + fvc))
        self._scatter(uf, 'r', -mag*(fic + fvc))
        for (fp, ee, *_), f in zip(bcs, bflux):
            uf[fp, :, ee] = f.T

        if self.aa is not None:
            r = self.apply(self.aa['M1329'],
                           ft.reshape(nd*len(self.aa['qpts']), -1, ne))
        else:
            r = self.apply(self.ops['M132'], ft.reshape(nd*nupts, -1, ne))
        r += self.apply(self.ops['M3'], uf)
        return self._add_src(-r/self.djac_u[:, None, :], u, src, t)


def shock_sensor(u, av):
    """Artificial viscosity of every element from the modal content of
    its density (pyfr/solvers/baseadvecdiff/kernels/shocksensor.mako, with
    the parameters of pyfr/solvers/baseadvecdiff/artvisc.py:160-196).

    av: invvdm (nmodes, nupts) nodal->modal, degs (largest degree of each
    mode), order, and c = {'max-artvisc', 'kappa', 's0'}; u (nupts, nvars,
    neles).  Orders from 2 up take the Klockner-Warburton-Hesthaven decay
    fit, order 1 the Persson-Peraire modal ratio."""
    c, order = av['c'], av['order']
    kappa, amax = c['kappa'], c['max-artvisc']
    degs = list(av['degs'])
    modes = av['invvdm'] @ u[:, 0, :]                        # (nmodes, ne)
    ne = u.shape[2]
    fit = list(range(1, order + 1))
    if len(fit) >= 2:
        x = np.log(np.array(fit, dtype=float) + 1)
        w = np.linalg.pinv(np.column_stack([np.ones(len(x)), x]))[1]
        bd = np.array([1.0/(d + 1)**(2*order) for d in fit])
        bd /= bd.sum()
        en = np.zeros((order + 1, ne))
        for k, d in enumerate(degs):
            en[d] += modes[k]**2
        tot = en.sum(axis=0)
        for i, d in enumerate(fit):
            en[d] += tot*bd[i]
        for d in range(order - 1, -1, -1):
            en[d] = np.maximum(en[d], en[d + 1])
        s = -0.5*sum(w[i]*np.log(en[d]) for i, d in enumerate(fit))
        mu = np.where(s > 2 + kappa, 0.0,
                      0.5*amax*(1 - np.sin(0.5*np.pi/kappa*(s - 2))))
        return np.where(s < 2 - kappa, amax, mu)

    tot = np.sum(modes**2, axis=0)
    top = np.array([d == order for d in degs])
    pn = 1e-15 + np.sum(modes[top]**2, axis=0)
    se = np.log10(pn/tot)
    se0 = np.log10(c['s0']/order**4)
    mu = np.where(se < se0 - kappa, 0.0,
                  0.5*amax*(1 + np.sin(0.5*np.pi/kappa*(se - se0))))
    return np.where(se < se0 + kappa, mu, amax)


def artvisc_points(mu, av):
    """Vertex maxima of the element viscosities, interpolated linearly to
    the flux and solution points: (nfpts, neles), (nupts, neles); av adds
    vnodes (nverts, neles) node numbers, nnodes, and the linear shape
    functions opf (nfpts, nverts), opu (nupts, nverts)."""
    vn = av['vnodes']
    vtx = np.zeros(av['nnodes'])
    np.maximum.at(vtx, vn.ravel(), np.broadcast_to(mu, vn.shape).ravel())
    ve = vtx[vn]                                             # (nverts, ne)
    return av['opf'] @ ve, av['opu'] @ ve


def wavespeed(u, smats, djac, gamma):
    """Largest reference-space wave speed of each element
    (pyfr/solvers/euler/kernels/wavespeed.mako:9-44): max over the points
    of sum_i |sum_j (S_ij/|J|) v_j| + c sqrt(sum_j (S_ij/|J|)^2);
    u (npts, nvars, neles), smats S[p, i, j, e], djac (npts, neles)."""
    nd = u.shape[1] - 2
    rho, E = u[:, 0], u[:, -1]
    v = u[:, 1:nd + 1]/rho[:, None]
    p = (gamma - 1)*(E - 0.5*rho*np.sum(v*v, axis=1))
    c = np.sqrt(gamma*p/rho)
    sij = smats/djac[:, None, None, :]
    vn = np.einsum('pije,pje->pie', sij, v)
    lam = np.sum(np.abs(vn), axis=1) + c*np.sum(np.sqrt(np.sum(sij*sij,
                                                                axis=2)),
                                                 axis=1)
    return lam.max(axis=0)


# ---------------------------------------------------------------------------
# Meshes of several element types
# ---------------------------------------------------------------------------

def linear_shape(etype, pts):
    """Values (npts, nverts) and reference gradients (npts, ndims, nverts)
    of the linear shape functions of ``etype`` (the interpolation and
    Jacobian expressions of pyfr/shapes.py:306-566), vertices in the
    reference's order."""
    pts = np.asarray(pts, dtype=float)
    n = len(pts)
    if etype in ('quad', 'hex'):
        nd = pts.shape[1]
        s = vertex_signs(nd)
        N = shape_values(pts, nd)
        dN = np.empty((n, nd, len(s)))
        for i in range(nd):
            t = np.ones((n, len(s)))
            for d in range(nd):
                t = t*(s[None, :, d] if d == i
                       else 1 + pts[:, None, d]*s[None, :, d])
            dN[:, i] = t/2**nd
        return N, dN
    if etype == 'tri':
        r, q = pts.T
        N = np.stack([-(r + q)/2, (1 + r)/2, (1 + q)/2], axis=1)
        g = np.array([[-0.5, 0.5, 0.0], [-0.5, 0.0, 0.5]])
        return N, np.broadcast_to(g, (n, 2, 3)).copy()
    if etype == 'tet':
        r, q, t = pts.T
        N = np.stack([-(1 + r + q + t)/2, (1 + r)/2, (1 + q)/2, (1 + t)/2],
                     axis=1)
        g = np.array([[-0.5, 0.5, 0.0, 0.0], [-0.5, 0.0, 0.5, 0.0],
                      [-0.5, 0.0, 0.0, 0.5]])
        return N, np.broadcast_to(g, (n, 3, 4)).copy()
    if etype == 'pri':
        r, q, t = pts.T
        tri = np.stack([-(r + q)/2, (1 + r)/2, (1 + q)/2], axis=1)
        lo, hi = (1 - t)/2, (1 + t)/2
        N = np.hstack([tri*lo[:, None], tri*hi[:, None]])
        dN = np.empty((n, 3, 6))
        gt = np.array([[-0.5, 0.5, 0.0], [-0.5, 0.0, 0.5]])
        for i in range(2):
            dN[:, i, :3] = gt[i][None, :]*lo[:, None]
            dN[:, i, 3:] = gt[i][None, :]*hi[:, None]
        dN[:, 2, :3] = -tri/2
        dN[:, 2, 3:] = tri/2
        return N, dN
    if etype == 'pyr':
        # The pyramid's interpolation and Jacobian expressions term by term
        # (pyfr/shapes.py:590-616)
        x, y, z = pts.T
        N = np.stack([2*x*y - 2*x - 2*y - z + 1, -2*x*y + 2*x - 2*y - z + 1,
                      -2*x*y - 2*x + 2*y - z + 1, 2*x*y + 2*x + 2*y - z + 1,
                      4*(1 + z)], axis=1)/8
        zero, eighth = np.zeros(n), np.full(n, 1/8)
        dN = np.stack([
            np.stack([y - 1, 1 - y, -y - 1, y + 1, zero], axis=1)/4,
            np.stack([x - 1, -x - 1, 1 - x, x + 1, zero], axis=1)/4,
            np.stack([-eighth, -eighth, -eighth, -eighth, 4*eighth], axis=1)
        ], axis=1)
        return N, dN
    raise ValueError(etype)


def linear_smats_djac(etype, verts, pts):
    """Adjugate metric S[p, i, :, e] and |J| of linear elements."""
    _, dN = linear_shape(etype, pts)
    J = np.einsum('piv,vej->pije', dN, verts)
    nd = J.shape[1]
    s = np.empty_like(J)
    if nd == 2:
        s[:, 0, 0], s[:, 0, 1] = J[:, 1, 1], -J[:, 1, 0]
        s[:, 1, 0], s[:, 1, 1] = -J[:, 0, 1], J[:, 0, 0]
        d = s[:, 0, 0]*s[:, 1, 1] - s[:, 0, 1]*s[:, 1, 0]
    else:
        for i in range(3):
            a, b = (i + 1) % 3, (i + 2) % 3
            s[:, i] = np.cross(J[:, a], J[:, b], axisa=1, axisb=1, axisc=1)
        d = np.einsum('pje,pje->pe', J[:, 0], s[:, 0])
    return s, d


class MixedDiscretisation:
    """The Euler right-hand side on a mesh of several element types
    (pyfr/solvers/baseadvec/system.py:58-136 over every element type).

    parts: {etype: dict(ops=..., basis=..., verts=...)} as for
    ``Discretisation``; lhs/rhs: sequences of (etype, element, face) of
    the interfaces; periods as for ``Discretisation``.  Fields are dicts
    {etype: (npts, nvars, neles)}; ``pack``/``unpack`` flatten them for
    ``rk45_step``.
    """

    def __init__(self, parts, lhs, rhs, periods=None):
        self.etypes = list(parts)
        self.p = {}
        for et, d in parts.items():
            e = dict(ops={k: np.asarray(v, dtype=float)
                          for k, v in d['ops'].items()},
                     upts=np.asarray(d['basis']['upts'], dtype=float),
                     fpts=np.asarray(d['basis']['fpts'], dtype=float),
                     norm=np.asarray(d['basis']['norm_fpts'], dtype=float),
                     facefpts=[np.asarray(f) for f in d['basis']['facefpts']],
                     verts=np.asarray(d['verts'], dtype=float))
            e['neles'] = e['verts'].shape[1]
            e['smats_u'], e['djac_u'] = linear_smats_djac(et, e['verts'],
                                                          e['upts'])
            s_f, _ = linear_smats_djac(et, e['verts'], e['fpts'])
            e['pnorm'] = np.einsum('plke,pl->pke', s_f, e['norm'])
            N, _ = linear_shape(et, e['fpts'])
            e['ploc_f'] = np.einsum('pv,ved->pde', N, e['verts'])
            self.p[et] = e
        self.ndims = next(iter(self.p.values()))['verts'].shape[2]
        self._pair(lhs, rhs, periods)

    def _pair(self, lhs, rhs, periods):
        """Pair the flux points of every interface by coordinates."""
        lhs = [(str(a), int(b), int(c)) for a, b, c in lhs]
        rhs = [(str(a), int(b), int(c)) for a, b, c in rhs]
        groups = {}
        for (tl, el, fl), (tr, er, fr) in zip(lhs, rhs):
            groups.setdefault((tl, fl, tr, fr), []).append((el, er))

        sides = {'l': [], 'r': []}
        for (tl, fl, tr, fr), ee in groups.items():
            ee = np.array(ee)
            el, er = ee[:, 0], ee[:, 1]
            pl = self.p[tl]['facefpts'][fl]
            pr = self.p[tr]['facefpts'][fr]
            xl = self.p[tl]['ploc_f'][pl][:, :, el]
            xr = self.p[tr]['ploc_f'][pr][:, :, er]
            d = xl[:, None] - xr[None, :]
            if periods is not None:
                P = np.asarray(periods)[:, None]
                d = d - P*np.rint(d/P)
            match = np.argmin(np.sum(d*d, axis=2), axis=1)      # (nfp, n)
            nfp = len(pl)
            if np.any(np.sort(match, axis=0) != np.arange(nfp)[:, None]):
                raise RuntimeError('Flux points of an interface do not pair')
            n = len(el)
            sides['l'].append((np.full(n*nfp, self.etypes.index(tl)),
                               np.tile(pl, n), np.repeat(el, nfp)))
            sides['r'].append((np.full(n*nfp, self.etypes.index(tr)),
                               pr[match.T].ravel(), np.repeat(er, nfp)))
        self.side = {k: tuple(np.concatenate(a) for a in zip(*v))
                     for k, v in sides.items()}
        t, f, e = self.side['l']
        nl = np.empty((self.ndims, len(t)))
        for i, et in enumerate(self.etypes):
            m = t == i
            nl[:, m] = self.p[et]['pnorm'][f[m], :, e[m]].T
        self.nl = nl

    def _gather(self, fld, side):
        t, f, e = self.side[side]
        nv = next(iter(fld.values())).shape[1]
        out = np.empty((nv, len(t)))
        for i, et in enumerate(self.etypes):
            m = t == i
            out[:, m] = fld[et][f[m], :, e[m]].T
        return out

    def _scatter(self, fld, side, vals):
        t, f, e = self.side[side]
        for i, et in enumerate(self.etypes):
            m = t == i
            fld[et][f[m], :, e[m]] = vals[:, m].T

    def rhs_euler(self, u, c, rsolver='rusanov'):
        gamma, nd = c['gamma'], self.ndims
        uf = {et: Discretisation.apply(self.p[et]['ops']['M0'], u[et])
              for et in self.etypes}
        ul, ur = self._gather(uf, 'l'), self._gather(uf, 'r')
        mag = np.sqrt(np.sum(self.nl**2, axis=0))
        fn = RSOLVERS[rsolver](ul, ur, self.nl/mag, gamma)
        self._scatter(uf, 'l', mag*fn)
        self._scatter(uf, 'r', -mag*fn)

        out = {}
        for et in self.etypes:
            e = self.p[et]
            nupts, ne = len(e['upts']), e['neles']
            fp, _, _ = inviscid_flux(u[et].transpose(1, 0, 2), gamma)
            ft = np.einsum('pike,kpve->ipve', e['smats_u'],
                           fp.transpose(0, 2, 1, 3))
            r = Discretisation.apply(e['ops']['M132'],
                                     ft.reshape(nd*nupts, -1, ne))
            r += Discretisation.apply(e['ops']['M3'], uf[et])
            out[et] = -r/e['djac_u'][:, None, :]
        return out

    def rhs_ns(self, u, c, rsolver='rusanov'):
        """Navier-Stokes right-hand side over every element type (the
        graphs of pyfr/solvers/baseadvecdiff/system.py:54-231)."""
        gamma, beta, tau = c['gamma'], c['ldg-beta'], c['ldg-tau']
        nd = self.ndims
        ap = Discretisation.apply
        uf = {et: ap(self.p[et]['ops']['M0'], u[et]) for et in self.etypes}

        # Common solution at the interface points (intconu)
        ul, ur = self._gather(uf, 'l'), self._gather(uf, 'r')
        if beta == -0.5:
            cl = cr = ul
        elif beta == 0.5:
            cl = cr = ur
        else:
            cl = cr = ur*(0.5 + beta) + ul*(0.5 - beta)
        comm = {et: v.copy() for et, v in uf.items()}
        self._scatter(comm, 'l', cl)
        self._scatter(comm, 'r', cr)

        # Corrected physical gradient at the solution points, interpolated
        # to the flux points
        grad, gfp, ft = {}, {}, {}
        for et in self.etypes:
            e = self.p[et]
            nup, ne = len(e['upts']), e['neles']
            g = ap(e['ops']['M460'], u[et]) + ap(e['ops']['M6'], comm[et])
            g = g.reshape(nd, nup, -1, ne)
            g = np.einsum('pkie,kpve->ipve', e['smats_u'], g) / \
                e['djac_u'][None, :, None, :]
            grad[et] = g
            gfp[et] = np.stack([ap(e['ops']['M0'], g[d]) for d in range(nd)])
            ut = u[et].transpose(1, 0, 2)
            fi, _, _ = inviscid_flux(ut, gamma)
            fv = viscous_flux(ut, g.transpose(0, 2, 1, 3), c)
            ft[et] = np.einsum('pike,kpve->ipve', e['smats_u'],
                               (fi + fv).transpose(0, 2, 1, 3))

        # Common flux at the interface points
        def gather_grad(side):
            t, f, ee = self.side[side]
            out = np.empty((nd, nd + 2, len(t)))
            for i, et in enumerate(self.etypes):
                m = t == i
                out[:, :, m] = gfp[et][:, f[m], :, ee[m]].transpose(1, 2, 0)
            return out

        gl, gr = gather_grad('l'), gather_grad('r')
        mag = np.sqrt(np.sum(self.nl**2, axis=0))
        n = self.nl/mag
        fic = RSOLVERS[rsolver](ul, ur, n, gamma)
        fvl = np.einsum('dn,dvn->vn', n, viscous_flux(ul, gl, c))
        fvr = np.einsum('dn,dvn->vn', n, viscous_flux(ur, gr, c))
        if beta == -0.5:
            fvc = fvr
        elif beta == 0.5:
            fvc = fvl
        else:
            fvc = (0.5 + beta)*fvl + (0.5 - beta)*fvr
        fvc = fvc + tau*(ul - ur)
        self._scatter(uf, 'l', mag*(fic + fvc))
        self._scatter(uf, 'r', -mag*(fic + fvc))

        out = {}
        for et in self.etypes:
            e = self.p[et]
            nup, ne = len(e['upts']), e['neles']
            r = ap(e['ops']['M132'], ft[et].reshape(nd*nup, -1, ne))
            r += ap(e['ops']['M3'], uf[et])
            out[et] = -r/e['djac_u'][:, None, :]
        return out

    def pack(self, fld):
        return np.concatenate([fld[et].ravel() for et in self.etypes])

    def unpack(self, flat, nvars):
        out, off = {}, 0
        for et in self.etypes:
            e = self.p[et]
            shp = (len(e['upts']), nvars, e['neles'])
            n = int(np.prod(shp))
            out[et] = flat[off:off + n].reshape(shp)
            off += n
        return out


# ---------------------------------------------------------------------------
# Entropy filter (pyfr/solvers/baseadvec/entfilter.py,
# pyfr/solvers/euler/kernels/{entropy,entropylocal,entropyfilter}.mako)
# ---------------------------------------------------------------------------

def entropy_state(u, gamma, big):
    """Density, pressure and entropy function of states u (nvars, ...)."""
    nd = u.shape[0] - 2
    d = u[0]
    with np.errstate(divide='ignore', invalid='ignore'):
        rcpd = 1/d
        p = (gamma - 1)*(u[-1] - 0.5*rcpd*np.sum(u[1:nd + 1]**2, axis=0))
        e = np.where((d > 0) & (p > 0), p*np.abs(rcpd)**gamma, big)
    return d, p, e


class EntropyFilterOracle:
    """The entropy filter over one element type of a Discretisation:
    ops = dict(vdm (nefpts, nupts), invvdm (nupts, nupts: nodal -> modal),
    m0 or None, degs, mean_wts (nupts, neles)); opts = d_min, p_min, e_tol,
    f_tol, niters, order, linearise; bcs as the Discretisation's, with
    their ghost states."""

    def __init__(self, disc, ops, opts, gamma, big=np.finfo(float).max):
        self.d, self.ops, self.o, self.gamma, self.big = disc, ops, opts, \
            gamma, big
        self.nfaces = len(disc.facefpts)
        self.entmin = np.full((self.nfaces, disc.neles), -big)

    def _minima(self, ue):
        """ue (nupts, nvars) -> (dmin, pmin, emin) over the points (and the
        flux points when they are not solution points)."""
        pts = ue
        if self.ops['m0'] is not None:
            pts = np.vstack([ue, self.ops['m0'] @ ue])
        d, p, e = entropy_state(pts.T, self.gamma, self.big)
        return d.min(), p.min(), e.min()

    def _bad(self, d, p, e, entmin):
        o = self.o
        return d < o['d_min'] or p < o['p_min'] or e < entmin - o['e_tol']

    def _filter_point(self, up, f):
        ui = up[0].copy()
        v = v2 = 1.0
        for k in range(1, self.o['order'] + 1):
            v2 *= v*v*f
            v *= f
            ui += v2*up[k]
        return entropy_state(ui[:, None], self.gamma, self.big)

    def filter_element(self, ue, e):
        """Filter one element's solution (nupts, nvars) in place; returns
        (filter strength, new minimum entropy)."""
        o, ops = self.o, self.ops
        entmin = self.entmin[:, e].min()
        dmin, pmin, emin = self._minima(ue)
        uavg = ops['mean_wts'][:, e] @ ue
        f = 1.0
        if not o['linearise'] and self._bad(dmin, pmin, emin, entmin):
            um = ops['invvdm'] @ ue
            degs = ops['degs']
            for i in range(ops['vdm'].shape[0]):
                up = np.zeros((o['order'] + 1, ue.shape[1]))
                for m in range(len(degs)):
                    up[degs[m]] += ops['vdm'][i, m]*um[m]
                d, p, s = (x[0] for x in self._filter_point(up, f))
                if self._bad(d, p, s, entmin):
                    fhi, flo = f, 0.0
                    it = 0
                    while it < o['niters'] and fhi - flo > o['f_tol']:
                        fnew = 0.5*(flo + fhi)
                        d, p, s = (x[0] for x in self._filter_point(up, fnew))
                        if self._bad(d, p, s, entmin):
                            fhi = fnew
                        else:
                            flo = fnew
                        it += 1
                    f = flo
            ffac = np.empty(o['order'] + 1)
            v = ffac[0] = 1.0
            for k in range(1, o['order'] + 1):
                ffac[k] = ffac[k - 1]*v*v*f
                v *= f
            nup = ue.shape[0]
            ue[:] = (ops['vdm'][:nup]*ffac[degs][None, :]) @ um
            ue += uavg - ops['mean_wts'][:, e] @ ue
            dmin, pmin, emin = self._minima(ue)

        if self._bad(dmin, pmin, emin, entmin):
            davg, pavg, eavg = (x[0] for x in entropy_state(uavg[:, None],
                                                            self.gamma,
                                                            self.big))
            for vmin, vavg, bound, nv in (
                    ('d', davg, o['d_min'], 1), ('p', pavg, o['p_min'], None),
                    ('e', eavg, entmin - o['e_tol'], None)):
                cur = dict(d=dmin, p=pmin, e=emin)[vmin]
                if cur < bound:
                    # (fmax/fmin semantics: a 0/0 ratio gives 0, an
                    # infinite one the clamp, as in the kernel)
                    with np.errstate(divide='ignore', invalid='ignore'):
                        ratio = np.float64(cur - bound)/np.float64(cur - vavg)
                    alpha = float(np.fmin(np.fmax(ratio, 0.0), 1.0))
                    f = min(f, 1.0 - alpha)
                    sl = slice(0, nv)
                    ue[:, sl] += alpha*(uavg[sl] - ue[:, sl])
                    dmin, pmin, emin = self._minima(ue)
        self.entmin[:, e] = emin
        return f, emin

    def filter(self, u):
        """Filter every element of u (nupts, nvars, neles) in place."""
        fs = np.empty(u.shape[2])
        for e in range(u.shape[2]):
            ue = u[:, :, e].copy()
            fs[e], _ = self.filter_element(ue, e)
            u[:, :, e] = ue
        return fs

    def local(self, u):
        for e in range(u.shape[2]):
            self.entmin[:, e] = self._minima(u[:, :, e])[2]

    def exchange(self):
        """Interfaces take the smaller of their two faces' minima."""
        fl, fr = self.d.faces_l, self.d.faces_r
        m = np.minimum(self.entmin[fl[:, 1], fl[:, 0]],
                       self.entmin[fr[:, 1], fr[:, 0]])
        self.entmin[fl[:, 1], fl[:, 0]] = m
        self.entmin[fr[:, 1], fr[:, 0]] = m

    def exchange_bcs(self, u):
        """Boundary faces take the smaller of their minimum and the entropy
        of the ghost state at their flux points."""
        uf = Discretisation.apply(self.d.ops['M0'], u)
        for fp, ee, n, bmag, spec in self.d.bcs:
            ub = uf[fp, :, ee].T
            ug = bc_rsolve_state(spec, ub, n, self.gamma)
            _, _, s = entropy_state(ug, self.gamma, self.big)
            # faces of the points: the face whose point list holds fp
            face = np.array([next(f for f, pts in enumerate(self.d.facefpts)
                                  if q in pts) for q in fp])
            np.minimum.at(self.entmin, (face, ee), s)


def rk45_step_ef(rhs, u, dt, ef):
    """rk45_step with the entropy filter: every right-hand side filters its
    input register in place first and exchanges the new minima, and the
    step ends with a filter of the result."""
    def frhs(x):
        ef.filter(x)
        ef.exchange()
        ef.exchange_bcs(x)
        return rhs(x)

    r1, r2 = u.copy(), u
    ns = len(RK45_B)
    for i in range(ns):
        if i == 0:
            r2 = frhs(r1)
        else:
            r2 = frhs(r2)
        if i < ns - 1:
            r1, r2 = r1 + dt*RK45_B[i]*r2, r1 + dt*RK45_A[i]*r2
        else:
            r1 = r1 + dt*RK45_B[i]*r2
    ef.filter(r1)
    return r1


# ---------------------------------------------------------------------------
# Time integration
# ---------------------------------------------------------------------------

RK45_A = [970286171893 / 4311952581923, 6584761158862 / 12103376702013,
          2251764453980 / 15575788980749, 26877169314380 / 34165994151039]
RK45_B = [1153189308089 / 22510343858157, 1772645290293 / 4653164025191,
          -1672844663538 / 4480602732383, 2114624349019 / 3568978502595,
          5198255086312 / 14908931495163]


def rk45_step_t(rhs, u, t, dt):
    """rk45_step with the stage times passed to rhs(u, t): stage i at
    t + c_i dt, c_0 = 0 and c_i = sum(b[:i-1]) + a[i-1] (the low-storage
    scheme's abscissae)."""
    cs = [0.0] + [sum(RK45_B[:i]) + a for i, a in enumerate(RK45_A)]
    r1, r2 = u.copy(), u
    ns = len(RK45_B)
    for i in range(ns):
        r2 = rhs(r2 if i else r1, t + cs[i]*dt)
        if i < ns - 1:
            r1, r2 = r1 + dt*RK45_B[i]*r2, r1 + dt*RK45_A[i]*r2
        else:
            r1 = r1 + dt*RK45_B[i]*r2
    return r1


def rkvdh2_stage(stage, nstages, a, b, e, dt, r1, r2, rold=None, rerr=None,
                 errest=False):
    """One stage of the two-register scheme with the optional embedded
    error register (pyfr/integrators/explicit/kernels/rkvdh2.mako:4-31);
    returns the new (r1, r2, rold, rerr)."""
    t1, t2 = r1.copy(), r2.copy()
    if errest and stage == 0:
        rerr = dt*e[stage]*t2
        rold = t1.copy()
    elif errest:
        rerr = rerr + dt*e[stage]*t2
    if stage < nstages - 1:
        return t1 + dt*a[stage]*t2, t1 + dt*b[stage]*t2, rold, rerr
    return t1 + dt*b[stage]*t2, r2, rold, rerr


def rk45_step(rhs, u, dt):
    """One step of the two-register RK45 scheme (rkvdh2 semantics)."""
    r1, r2 = u.copy(), u
    ns = len(RK45_B)
    for i in range(ns):
        r2 = rhs(r2 if i else r1)
        if i < ns - 1:
            r1, r2 = r1 + dt*RK45_B[i]*r2, r1 + dt*RK45_A[i]*r2
        else:
            r1 = r1 + dt*RK45_B[i]*r2
    return r1
