"""Boundary-condition test cases (test infrastructure): the configuration
of a box bounded in one direction, shared by the boundary tests and the
reference-stack driver (``tests/refstack.py``)."""

import numpy as np

GAS = dict(gamma=1.4, mu=0.02, Pr=0.72, **{'ldg-beta': 0.5, 'ldg-tau': 0.1})
FREE = dict(rho=1.1, p=0.95, u=[0.35, -0.15, 0.2])

# Total state of the sub-in-ftpttang inflow: cp*T_t, p_t and the direction
# (theta, phi) in degrees
TOTAL = dict(cpTt=3.9, pt=1.08, theta=20.0, phi=80.0)

# The controllers of the characteristic boundaries (mass-flow target or
# target mean pressure, relaxation alpha, gain eta, update every nsteps
# right-hand sides, surface quadrature degree)
CONTROL = {'char-riem-inv-mass-flow': {'mass-flow-rate': 0.14,
                                       'alpha': 0.5, 'eta': 2.0,
                                       'nsteps': 3, 'quad-deg': 5},
           'char-riem-inv-pressure': {'pressure': 0.97, 'alpha': 0.5,
                                      'eta': 3.0, 'nsteps': 3,
                                      'quad-deg': 5}}


def vc(theta, phi):
    t, f = np.radians(theta), np.radians(phi)
    return [np.cos(t)*np.sin(f), np.sin(t)*np.sin(f), np.cos(f)]


def bc_cfg(ndims, specs, rsolver='rusanov', precision='double', ns=False):
    """The configuration of a box with the boundaries of ``specs``
    ({name: dict(type=..., values...)}) and a smooth non-uniform initial
    state."""
    from pyfr_gb300.inifile import Inifile
    cfg = Inifile()
    cfg.set('backend', 'precision', precision)
    for k in ('gamma', 'mu', 'Pr'):
        cfg.set('constants', k, GAS[k])
    cfg.set('solver', 'system', 'navier-stokes' if ns else 'euler')
    cfg.set('solver', 'order', 3)
    cfg.set('solver-interfaces', 'riemann-solver', rsolver)
    cfg.set('solver-interfaces', 'ldg-beta', GAS['ldg-beta'])
    cfg.set('solver-interfaces', 'ldg-tau', GAS['ldg-tau'])
    cfg.set('solver-time-integrator', 'scheme', 'rk45')
    cfg.set('solver-time-integrator', 'controller', 'none')
    cfg.set('solver-time-integrator', 'dt', 1e-3)
    et, ft = ('quad', 'line') if ndims == 2 else ('hex', 'quad')
    cfg.set(f'solver-elements-{et}', 'soln-pts', 'gauss-legendre')
    cfg.set(f'solver-interfaces-{ft}', 'flux-pts', 'gauss-legendre')
    for name, spec in specs.items():
        sect = f'soln-bcs-{name}'
        cfg.set(sect, 'type', spec['type'])
        for k in ('rho', 'p', 'cpTw', 'cpTt', 'pt', 'theta', 'phi'):
            if k in spec:
                cfg.set(sect, k, spec[k])
        for k, v in zip('uvw', spec.get('u', [])[:ndims]):
            cfg.set(sect, k, v)
        for k, v in CONTROL.get(spec['type'], {}).items():
            cfg.set(sect, k, v)
    x = '2*pi*x'
    cfg.set('soln-ics', 'rho', f'1 + 0.1*sin({x})*cos(2*pi*y)')
    cfg.set('soln-ics', 'u', '0.3 + 0.1*y')
    cfg.set('soln-ics', 'v', f'0.1*sin({x})')
    if ndims == 3:
        cfg.set('soln-ics', 'w', '0.05*cos(2*pi*z)')
    cfg.set('soln-ics', 'p', '1 + 0.05*cos(2*pi*y)')
    return cfg


def bc_case(kind, types):
    """(cfg, mesh, specs) of the boundary case ``kind`` ('euler': a quad
    box bounded in y, boundaries ylo and yhi; 'ns': a hex box bounded in z,
    boundaries zlo and zhi) with the boundary types ``types``."""
    from pyfr_gb300.mesh import box
    if kind == 'euler':
        names, nd = ('ylo', 'yhi'), 2
        mesh = box('quad', (4, 3), 0.0, 1.0, (True, False))
    else:
        names, nd = ('zlo', 'zhi'), 3
        mesh = box('hex', (2, 2, 3), 0.0, 1.0, (True, True, False))
    extra = dict(TOTAL, vc=vc(TOTAL['theta'], TOTAL['phi']))
    specs = {n: dict(type=t, cpTw=3.2 + 0.4*i, **FREE, **extra)
             for i, (n, t) in enumerate(zip(names, types))}
    cfg = bc_cfg(nd, specs, ns=kind == 'ns')
    if any(t in CONTROL for t in types):
        # A mean flow through the boundaries, which the controllers measure
        if kind == 'euler':
            cfg.set('soln-ics', 'v', '-0.15 + 0.05*sin(2*pi*x)')
        else:
            cfg.set('soln-ics', 'w', '0.2 + 0.05*cos(2*pi*y)')
    return cfg, mesh, specs
