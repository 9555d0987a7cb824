"""Helpers that build oracle discretisations (test infrastructure)."""
import numpy as np

from oracle.fr_oracle import Discretisation
from pyfr_gb300.shapes import get_shape


def ops_from_shape(s, ns=False):
    ops = dict(M0=s.m0, M132=s.opmat('M1 - M3*M2'), M3=s.m3)
    if ns:
        ops |= dict(M460=s.opmat('M4 - M6*M0'), M6=s.m6)
    return ops


def ops_from_golden(g, key, ns=False):
    ops = dict(M0=g[f'{key}/m0'], M132=g[f'{key}/M132'], M3=g[f'{key}/m3'])
    if ns:
        ops |= dict(M460=g[f'{key}/M460'], M6=g[f'{key}/m6'])
    return ops


def basis_of(s):
    return dict(upts=s.upts, fpts=s.fpts, norm_fpts=s.norm_fpts,
                facefpts=s.facefpts)


def disc_for_mesh(mesh, order, ns=False, ops=None, upts='gauss-legendre'):
    etype = mesh.etypes[0]
    s = get_shape(etype, order, upts, upts)
    lhs, rhs = mesh.con
    return Discretisation(ops or ops_from_shape(s, ns), basis_of(s),
                          mesh.spts[etype],
                          np.stack([lhs.eidxs, lhs.fidxs], 1),
                          np.stack([rhs.eidxs, rhs.fidxs], 1),
                          periods=mesh.periods)


# [solver-plugin-source] options of the source-term tests: the 2-D vortex
# (Euler) and the Taylor-Green vortex (Navier-Stokes), with terms of the
# coordinates, the conserved variables, the time and abs/pow/exp
SOURCES = {
    'vortex': {'rho': '0.01*sin(x)*cos(y) + 0.001*t',
               'rhou': '-0.05*rhou + 0.01*exp(-0.1*(x*x + y*y))',
               'rhov': '-0.05*rhov + 0.002*t*t',
               'E': '0.002*pow(abs(rho), 1.5)*cos(t) + 0.001*y'},
    'tgv': {'rho': '0',
            'rhou': '0.1*rho*sin(x)*cos(y)*cos(z)',
            'rhov': '-0.1*rho*cos(x)*sin(y)*cos(z)',
            'rhow': '0.01*t',
            'E': '0.1*(rhou*sin(x)*cos(y) - rhov*cos(x)*sin(y))*cos(z)'},
}


def add_source(cfg, case):
    """Add the case's [solver-plugin-source] section to cfg."""
    for k, v in SOURCES[case].items():
        cfg.set('solver-plugin-source', k, v)


def source_c_exprs(opts, convars, consts):
    """The source plugin's kernel expressions for ``opts``: x, y, z ->
    ploc[i], the conserved variables -> u[i], abs -> fabs, pi and the
    [constants] substituted as whole words (the substitution of
    pyfr/plugins/source.py:15-24, written out here independently of the
    product's configuration code)."""
    import math
    import re
    subs = {k: repr(float(v)) for k, v in consts.items()}
    subs |= dict(x='ploc[0]', y='ploc[1]', z='ploc[2]', abs='fabs',
                 pi=repr(math.pi))
    subs |= {v: f'u[{i}]' for i, v in enumerate(convars)}
    pat = re.compile(r'\b(' + '|'.join(sorted(subs, key=len, reverse=True)) +
                     r')\b')
    return [pat.sub(lambda m: f'({subs[m[1]]})', opts[v]) for v in convars]
