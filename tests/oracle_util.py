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
