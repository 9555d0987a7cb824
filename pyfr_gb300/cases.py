"""Synthetic test cases: configurations and meshes.

* ``euler_vortex``: 2-D isentropic vortex advected by a uniform free stream
  (rho=1, u=v=1, p=1/gamma) on a periodic square, Rusanov fluxes, RK45.
  With T = p/rho and the isentropic relation p = rho^gamma/gamma, radial
  equilibrium of a vortex with swirl speed (beta/2 pi)(r/R) exp((1-r^2/R^2)/2)
  gives rho = (1 - (gamma-1) beta^2/(8 pi^2) exp(1 - r^2/R^2))^(1/(gamma-1)).
  The exact solution is the initial field translated by (t, t).
* ``ns_tgv``: 3-D compressible Taylor-Green vortex on [-pi, pi]^3,
  Re=1600, Ma=0.1, Pr=0.71, rho0=1, isothermal initial density
  rho = rho0 p/p0, Rusanov + LDG (beta=1/2, tau=0.1), RK45.
* ``euler_mixed``: 3-D Euler on a conforming periodic box of n^3 cells on
  [-pi, pi]^3 made of hexahedra and prisms, or of prisms and tetrahedra:
  a density wave rho = 1 + A sin(x + y + z) carried by the uniform
  velocity (u, v, w) at uniform pressure, whose exact solution is the
  initial field translated by (u, v, w) t.
"""

import math

from pyfr_gb300.inifile import Inifile
from pyfr_gb300.mesh import mixed_box, periodic_box


def euler_vortex(n=40, order=3, dt=1e-3, beta=5.0, radius=1.0,
                 rsolver='rusanov', precision='double', half=10.0,
                 upts='gauss-legendre'):
    cfg = Inifile()
    cfg.set('backend', 'precision', precision)
    for k, v in dict(gamma=1.4, beta=beta, R=radius, uinf=1.0, vinf=1.0,
                     rhoinf=1.0).items():
        cfg.set('constants', k, repr(v))
    cfg.set('solver', 'system', 'euler')
    cfg.set('solver', 'order', order)
    cfg.set('solver-interfaces', 'riemann-solver', rsolver)
    cfg.set('solver-interfaces-line', 'flux-pts', upts)
    cfg.set('solver-elements-quad', 'soln-pts', upts)
    cfg.set('solver-time-integrator', 'scheme', 'rk45')
    cfg.set('solver-time-integrator', 'controller', 'none')
    cfg.set('solver-time-integrator', 'dt', repr(dt))

    f = '(1 - (x*x + y*y)/(R*R))'
    cfg.set('soln-ics', 'rho',
            f'pow(1 - (gamma - 1)*beta*beta/(8*pi*pi)*exp({f}), 1/(gamma - 1))')
    cfg.set('soln-ics', 'u', f'uinf - beta/(2*pi)*(y/R)*exp(0.5*{f})')
    cfg.set('soln-ics', 'v', f'vinf + beta/(2*pi)*(x/R)*exp(0.5*{f})')
    cfg.set('soln-ics', 'p',
            f'pow(1 - (gamma - 1)*beta*beta/(8*pi*pi)*exp({f}), '
            'gamma/(gamma - 1))/gamma')

    mesh = periodic_box('quad', n, -half, half)
    return cfg, mesh


def vortex_exact(x, y, t, cfg, half=10.0):
    """Exact primitive solution (rho, u, v, p) of the advected vortex at
    physical points (x, y), with periodic images."""
    import numpy as np

    c = cfg.items_as('constants', float)
    g, b, R = c['gamma'], c['beta'], c['R']
    L = 2*half
    xc, yc = c['uinf']*t, c['vinf']*t
    dx = (x - xc + half) % L - half
    dy = (y - yc + half) % L - half
    f = 1 - (dx*dx + dy*dy)/(R*R)
    rho = (1 - (g - 1)*b*b/(8*math.pi**2)*np.exp(f))**(1/(g - 1))
    u = c['uinf'] - b/(2*math.pi)*(dy/R)*np.exp(0.5*f)
    v = c['vinf'] + b/(2*math.pi)*(dx/R)*np.exp(0.5*f)
    p = rho**g/g
    return rho, u, v, p


def ns_tgv(n=48, order=3, dt=5e-4, rsolver='rusanov', precision='double',
           beta=0.5, tau=0.1, memory_model='normal', upts='gauss-legendre'):
    gamma, Ma, Re, Pr, rho0, U0 = 1.4, 0.1, 1600.0, 0.71, 1.0, 1.0
    p0 = rho0*U0*U0/(gamma*Ma*Ma)

    cfg = Inifile()
    cfg.set('backend', 'precision', precision)
    cfg.set('backend', 'memory-model', memory_model)
    for k, v in dict(gamma=gamma, mu=rho0*U0/Re, Pr=Pr, rho0=rho0,
                     p0=p0).items():
        cfg.set('constants', k, repr(v))
    cfg.set('solver', 'system', 'navier-stokes')
    cfg.set('solver', 'order', order)
    cfg.set('solver-interfaces', 'riemann-solver', rsolver)
    cfg.set('solver-interfaces', 'ldg-beta', repr(beta))
    cfg.set('solver-interfaces', 'ldg-tau', repr(tau))
    cfg.set('solver-interfaces-quad', 'flux-pts', upts)
    cfg.set('solver-elements-hex', 'soln-pts', upts)
    cfg.set('solver-time-integrator', 'scheme', 'rk45')
    cfg.set('solver-time-integrator', 'controller', 'none')
    cfg.set('solver-time-integrator', 'dt', repr(dt))

    pexpr = 'p0 + (rho0/16)*(cos(2*x) + cos(2*y))*(cos(2*z) + 2)'
    cfg.set('soln-ics', 'rho', f'rho0*({pexpr})/p0')
    cfg.set('soln-ics', 'u', 'sin(x)*cos(y)*cos(z)')
    cfg.set('soln-ics', 'v', '-cos(x)*sin(y)*cos(z)')
    cfg.set('soln-ics', 'w', '0*x')
    cfg.set('soln-ics', 'p', pexpr)

    mesh = periodic_box('hex', n, -math.pi, math.pi)
    return cfg, mesh


def euler_mixed(n=32, order=3, kinds='hex-pri', dt=1e-3, amp=0.2,
                vel=(1.0, 0.5, 0.25), rsolver='rusanov', precision='double'):
    cfg = Inifile()
    cfg.set('backend', 'precision', precision)
    for k, v in dict(gamma=1.4, amp=amp, uc=vel[0], vc=vel[1],
                     wc=vel[2]).items():
        cfg.set('constants', k, repr(v))
    cfg.set('solver', 'system', 'euler')
    cfg.set('solver', 'order', order)
    cfg.set('solver-interfaces', 'riemann-solver', rsolver)
    cfg.set('solver-interfaces-quad', 'flux-pts', 'gauss-legendre')
    cfg.set('solver-interfaces-tri', 'flux-pts', 'alpha-opt')
    cfg.set('solver-elements-hex', 'soln-pts', 'gauss-legendre')
    cfg.set('solver-elements-pri', 'soln-pts',
            'alpha-opt~gauss-legendre-lobatto')
    cfg.set('solver-elements-tet', 'soln-pts', 'alpha-opt')
    cfg.set('solver-elements-pyr', 'soln-pts', 'gauss-legendre')
    cfg.set('solver-time-integrator', 'scheme', 'rk45')
    cfg.set('solver-time-integrator', 'controller', 'none')
    cfg.set('solver-time-integrator', 'dt', repr(dt))

    cfg.set('soln-ics', 'rho', '1 + amp*sin(x + y + z)')
    cfg.set('soln-ics', 'u', 'uc + 0*x')
    cfg.set('soln-ics', 'v', 'vc + 0*x')
    cfg.set('soln-ics', 'w', 'wc + 0*x')
    cfg.set('soln-ics', 'p', '1 + 0*x')

    mesh = mixed_box(n, -math.pi, math.pi, kinds)
    return cfg, mesh


def density_wave_exact(x, y, z, t, cfg):
    """Exact density of the advected wave of ``euler_mixed``."""
    import numpy as np

    c = cfg.items_as('constants', float)
    return 1 + c['amp']*np.sin(x + y + z - (c['uc'] + c['vc'] + c['wc'])*t)
