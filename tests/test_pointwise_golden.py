"""The oracle's pointwise arithmetic against the reference's own kernels.

``tests/golden/pointwise.npz`` holds inputs and outputs of the reference's
``.mako`` kernels, rendered and compiled by ``oracle/refkernels.py``
(``tests/golden/make_pointwise.py``).  Here the numpy oracle
(``oracle/fr_oracle.py``) is evaluated on the same inputs and must agree to
1e-14 relative (per output variable, against its largest magnitude): the
two differ only in the order of floating-point operations.  Where the
reference checkout is present the compiled reference kernels are rebuilt
and must reproduce the fixtures bit for bit.
"""
import json

import numpy as np
import pytest

from oracle import fr_oracle as fo

TOL = 1e-14


@pytest.fixture(scope='module')
def pw(golden):
    g = golden['pointwise']
    return g, json.loads(str(g['meta']))


def _inputs(g, fam):
    pre = f'in:{fam}:'
    return {k[len(pre):]: v for k, v in g.items() if k.startswith(pre)}


def _relerr(a, b):
    """Largest error per trailing variable, relative to that variable's
    largest magnitude."""
    a, b = np.asarray(a), np.asarray(b)
    ax = tuple(range(a.ndim - 1)) if a.ndim > 1 else None
    scale = np.maximum(np.abs(b).max(axis=ax), 1e-300)
    return (np.abs(a - b).max(axis=ax)/scale).max()


def _ns_consts(c):
    return dict(c, sutherland='cpTref' in c)


def oracle_eval(m, x):
    """The oracle's value of fixture variant ``m`` on inputs ``x``; the
    dict of its outputs in the fixture's (npoints, ...) layout."""
    mod, tp, c = m['module'], m['tplargs'], m['tplargs'].get('c', {})
    gamma = c.get('gamma')
    if mod.endswith('euler.kernels.tflux'):
        f, _, _ = fo.inviscid_flux(x['u'].T, gamma)
        return {'f': np.einsum('nik,kvn->niv', x['smats'], f)}
    if mod.endswith('euler.kernels.wavespeed'):
        u = x['u'].T[None]
        sm = x['smats'].transpose(1, 2, 0)[None]
        return {'wspd': fo.wavespeed(u, sm, 1/x['rcpdjac'][None], gamma)}
    if mod.endswith('euler.kernels.intcflux'):
        nl = x['nl'].T
        mag = np.sqrt(np.sum(nl**2, axis=0))
        rs = fo.RSOLVERS[tp['rsolver']]
        fn = rs(x['ul'].T, x['ur'].T, (1/mag)*nl, gamma)
        return {'ul': (mag*fn).T, 'ur': (-mag*fn).T}
    if mod.endswith('navstokes.kernels.tflux'):
        g = np.einsum('n,nki,nkv->niv', x['rcpdjac'], x['smats'],
                      x['gradu'])
        u = x['u'].T
        f, _, _ = fo.inviscid_flux(u, gamma)
        f = f + fo.viscous_flux(u, g.transpose(1, 2, 0), _ns_consts(c))
        return {'f': np.einsum('nik,kvn->niv', x['smats'], f), 'gradu': g}
    if mod.endswith('navstokes.kernels.intcflux'):
        nl = x['nl'].T
        mag = np.sqrt(np.sum(nl**2, axis=0))
        n = (1/mag)*nl
        ul, ur = x['ul'].T, x['ur'].T
        beta, tau = c['ldg-beta'], c['ldg-tau']
        fic = fo.RSOLVERS[tp['rsolver']](ul, ur, n, gamma)
        cc = _ns_consts(c)
        fvl = np.einsum('dn,dvn->vn', n,
                        fo.viscous_flux(ul, x['gradul'].transpose(1, 2, 0),
                                        cc))
        fvr = np.einsum('dn,dvn->vn', n,
                        fo.viscous_flux(ur, x['gradur'].transpose(1, 2, 0),
                                        cc))
        if beta == -0.5:
            fvc = fvr
        elif beta == 0.5:
            fvc = fvl
        else:
            fvc = (0.5 + beta)*fvl + (0.5 - beta)*fvr
        fvc = fvc + tau*(ul - ur)
        return {'ul': (mag*(fic + fvc)).T, 'ur': (-mag*(fic + fvc)).T}
    if mod.endswith('intconu'):
        beta = c['ldg-beta']
        lo, ro = x['ulout'].copy(), x['urout'].copy()
        if beta == -0.5:
            ro = x['ulin'].copy()
        elif beta == 0.5:
            lo = x['urin'].copy()
        else:
            lo = ro = x['urin']*(0.5 + beta) + x['ulin']*(0.5 - beta)
        return {'ulout': lo, 'urout': ro}
    if mod.endswith('gradcoru'):
        return {'gradu': np.einsum('n,nki,nkv->niv', x['rcpdjac'],
                                   x['smats'], x['gradu'])}
    if mod.endswith('negdivconf') or mod.endswith('evalsrcmacros'):
        src = 0.0
        if tp.get('src_macros'):
            src = fo.source_terms(tp['src_exprs'], float(x['t']), x['u'].T,
                                  x['ploc'].T).T
        if mod.endswith('evalsrcmacros'):
            return {'u': src}
        return {'tdivtconf': -x['rcpdjac'][:, None]*x['tdivtconf'] + src}
    if mod.endswith('rkvdh2'):
        r1, r2, rold, rerr = fo.rkvdh2_stage(
            tp['stage'], tp['nstages'], tp['a'], tp['b'], tp['e'],
            float(x['dt']), x['r1'], x['r2'], x['rold'], x['rerr'],
            tp['errest'])
        return {'r1': r1, 'r2': r2, 'rold': rold, 'rerr': rerr}
    raise KeyError(mod)


def test_fixtures_cover_the_path(pw):
    g, meta = pw
    mods = {m['module'].rsplit('.', 1)[-1] for m in meta.values()}
    assert {'tflux', 'intcflux', 'intconu', 'gradcoru', 'negdivconf',
            'rkvdh2', 'wavespeed', 'evalsrcmacros'} <= mods
    assert any(m['tplargs'].get('src_macros') for m in meta.values())
    rs = {m['tplargs']['rsolver'] for m in meta.values()
          if 'rsolver' in m['tplargs']}
    assert rs == set(fo.RSOLVERS)
    for name, m in meta.items():
        for o in m['outputs']:
            assert np.all(np.isfinite(g[f'out:{name}:{o}'])), (name, o)


def test_oracle_matches_reference_kernels(pw):
    g, meta = pw
    worst = {}
    for name, m in meta.items():
        x = _inputs(g, m['family'])
        got = oracle_eval(m, x)
        for o in m['outputs']:
            ref = g[f'out:{name}:{o}']
            e = _relerr(np.reshape(got[o], ref.shape), ref)
            worst[f'{name}:{o}'] = e
    bad = {k: v for k, v in worst.items() if not v <= TOL}
    assert not bad, bad


def test_riemann_solvers_consistent(pw):
    """F(u, u, n) equals the physical normal flux for every solver (the
    last eight pairs of each interface family are equal states)."""
    g, meta = pw
    for nd in (2, 3):
        x = _inputs(g, f'euler{nd}_iface')
        ul, n = x['ul'][-8:].T, x['nl'][-8:].T
        n = n/np.sqrt(np.sum(n**2, axis=0))
        f, _, _ = fo.inviscid_flux(ul, 1.4)
        want = np.einsum('dn,dvn->vn', n, f)
        for rs, fn in fo.RSOLVERS.items():
            got = fn(ul, ul, n, 1.4)
            assert _relerr(got.T, want.T) < 1e-12, (nd, rs)


def test_reference_library_reproduces_fixtures(pw):
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip('reference checkout not present')
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).parent / 'golden'))
    import make_pointwise as mp
    g, meta = pw
    var = mp.variants()
    assert set(var) == set(meta)
    lib = refkernels.RefLibrary({k: (m, kn, tp, None)
                                 for k, (m, kn, tp, _) in var.items()})
    for name, (_, _, _, fam) in var.items():
        x = _inputs(g, fam)
        k = lib.kernels[name]
        args = {a.name: x[a.name] for a in k.vectargs if a.name in x}
        args |= {a.name: x[a.name] for a in k.scalargs}
        res = lib(name, len(next(iter(x.values()))), **args)
        for o in meta[name]['outputs']:
            np.testing.assert_array_equal(res[o], g[f'out:{name}:{o}'])
