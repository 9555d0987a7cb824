"""Each FP64 CUDA pointwise kernel against the reference's own kernels.

The inputs and outputs in ``tests/golden/pointwise.npz`` come from the
reference's ``.mako`` kernel sources, rendered to C and compiled on the
host (``tests/golden/make_pointwise.py``).  Here the b200 backend runs the
same kernels through the C ABI on the same inputs: element kernels over
one solution point of N elements, interface kernels over N point pairs
reached through gather views.  Tolerance 1e-13 relative per output
variable (against its largest magnitude): the CUDA kernels contract
multiply-adds and use the GPU's own sqrt, pow and division, so results
may differ in the last bits, never more.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


@pytest.fixture(scope='module')
def pw(golden):
    g = golden['pointwise']
    return g, json.loads(str(g['meta']))


def _inputs(g, fam):
    pre = f'in:{fam}:'
    return {k[len(pre):]: v for k, v in g.items() if k.startswith(pre)}


def _relerr(a, b):
    ax = tuple(range(a.ndim - 1)) if a.ndim > 1 else None
    scale = np.maximum(np.abs(b).max(axis=ax), 1e-300)
    return (np.abs(a - b).max(axis=ax)/scale).max()


def _backend():
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    cfg = Inifile()
    cfg.set('backend-b200', 'cuda-graphs', 'false')
    return B200Backend(cfg)


class _Points:
    """Fixture arrays as backend matrices and views over N points."""

    def __init__(self, be, n):
        self.be, self.n = be, n

    def scal(self, x):
        """(n, nvars) -> matrix of io-shape (1, nvars, n) and its view."""
        m = self.be.matrix((1, x.shape[1], self.n), x.T[None].copy(),
                           tags={'align'})
        return m

    def scal_view(self, m, nvars):
        n = self.n
        return self.be.view([m.mid]*n, [0]*n, list(range(n)),
                            vshape=(nvars,))

    def vect(self, x):
        """(n, ndims, nvars) -> matrix (ndims, nvars, n)."""
        return self.be.matrix((x.shape[1], x.shape[2], self.n),
                              x.transpose(1, 2, 0).copy(), tags={'align'})

    def vect_view(self, m, nd, nvars):
        n = self.n
        return self.be.view([m.mid]*n, [0]*n, list(range(n)), [1]*n,
                            vshape=(nd, nvars))

    def elem_geom(self, x):
        """smats (n, nd, nd) -> (nd, 1, nd, n); rcpdjac (n,) -> (1, n)."""
        nd = x['smats'].shape[1]
        s = self.be.const_matrix(x['smats'].transpose(1, 2, 0)[:, None],
                                 tags={'align'})
        r = self.be.const_matrix(x['rcpdjac'][None], tags={'align'})
        return s, r


def run_variant(be, m, x):
    """Run fixture variant m on inputs x through the b200 backend; returns
    the outputs in the fixture layout."""
    mod, tp = m['module'], dict(m['tplargs'])
    n = len(next(iter(x.values())))
    P = _Points(be, n)
    kname = mod.rsplit('.', 1)[-1]
    be.pointwise.register(mod)
    get_scal = lambda M: M.get()[0].T                       # noqa: E731
    get_vect = lambda M: M.get().transpose(2, 0, 1)          # noqa: E731

    if mod.endswith('euler.kernels.tflux') or \
            mod.endswith('euler.kernels.wavespeed'):
        nd, nv = tp['ndims'], tp['nvars']
        u = P.scal(x['u'])
        s, r = P.elem_geom(x)
        if kname == 'tflux':
            f = be.matrix((nd, 1, nv, n), tags={'align'})
            be.commit()
            k = be.kernel('tflux', tplargs=tp, dims=[1, n], u=u, f=f,
                          smats=s)
            be.run_kernels([k], wait=True)
            return {'f': f.get()[:, 0].transpose(2, 0, 1)}
        w = be.matrix((1, n), tags={'align'})
        be.commit()
        k = be.kernel('wavespeed', tplargs=tp, dims=[1, n], u=u, wspd=w,
                      smats=s, rcpdjac=r)
        be.run_kernels([k], wait=True)
        return {'wspd': w.get()[0]}

    if mod.endswith('euler.kernels.intcflux') or \
            mod.endswith('navstokes.kernels.intcflux'):
        nd, nv = tp['ndims'], tp['nvars']
        ul, ur = P.scal(x['ul']), P.scal(x['ur'])
        nl = be.const_matrix(x['nl'].T.copy(), tags={'align'})
        args = {}
        if 'gradul' in x:
            gl, gr = P.vect(x['gradul']), P.vect(x['gradur'])
        be.commit()
        if 'gradul' in x:
            args = dict(gradul=P.vect_view(gl, nd, nv),
                        gradur=P.vect_view(gr, nd, nv))
        k = be.kernel('intcflux', tplargs=tp, dims=[n],
                      ul=P.scal_view(ul, nv), ur=P.scal_view(ur, nv),
                      nl=nl, **args)
        be.run_kernels([k], wait=True)
        return {'ul': get_scal(ul), 'ur': get_scal(ur)}

    if mod.endswith('navstokes.kernels.tflux'):
        nd, nv = tp['ndims'], tp['nvars']
        u = P.scal(x['u'])
        gu = be.matrix((nd, 1, nv, n), x['gradu'].transpose(1, 2, 0)[:, None]
                       .copy(), tags={'align'})
        f = be.matrix((nd, 1, nv, n), tags={'align'})
        s, r = P.elem_geom(x)
        be.commit()
        k = be.kernel('tflux', tplargs=tp, dims=[1, n], u=u, f=f, gradu=gu,
                      smats=s, rcpdjac=r)
        be.run_kernels([k], wait=True)
        return {'f': f.get()[:, 0].transpose(2, 0, 1),
                'gradu': gu.get()[:, 0].transpose(2, 0, 1)}

    if mod.endswith('gradcoru'):
        nd, nv = tp['ndims'], tp['nvars']
        gu = be.matrix((nd, 1, nv, n), x['gradu'].transpose(1, 2, 0)[:, None]
                       .copy(), tags={'align'})
        s, r = P.elem_geom(x)
        be.commit()
        k = be.kernel('gradcoru', tplargs=tp, dims=[1, n], gradu=gu,
                      smats=s, rcpdjac=r)
        be.run_kernels([k], wait=True)
        return {'gradu': gu.get()[:, 0].transpose(2, 0, 1)}

    if mod.endswith('intconu'):
        nv = tp['nvars']
        mats = {a: P.scal(x[a]) for a in ('ulin', 'urin', 'ulout', 'urout')}
        be.commit()
        views = {a: P.scal_view(M, nv) for a, M in mats.items()}
        k = be.kernel('intconu', tplargs=tp, dims=[n], **views)
        be.run_kernels([k], wait=True)
        return {'ulout': get_scal(mats['ulout']),
                'urout': get_scal(mats['urout'])}

    if tp.get('src_macros'):
        # negdivconf and evalsrcmacros with the source plugin's macro
        ploc, u = P.scal(x['ploc']), P.scal(x['u'])
        if kname == 'negdivconf':
            t = P.scal(x['tdivtconf'])
            r = be.const_matrix(x['rcpdjac'][None], tags={'align'})
            be.commit()
            k = be.kernel('negdivconf', tplargs=tp, dims=[1, n], tdivtconf=t,
                          rcpdjac=r, ploc=ploc, u=u)
            out = {'tdivtconf': t}
        else:
            be.commit()
            k = be.kernel('evalsrcmacros', tplargs=tp, dims=[1, n], u=u,
                          ploc=ploc)
            out = {'u': u}
        k.bind(t=float(x['t']))
        be.run_kernels([k], wait=True)
        return {a: get_scal(M) for a, M in out.items()}

    if mod.endswith('negdivconf'):
        t = P.scal(x['tdivtconf'])
        r = be.const_matrix(x['rcpdjac'][None], tags={'align'})
        be.commit()
        k = be.kernel('negdivconf', tplargs=tp, dims=[1, n], tdivtconf=t,
                      rcpdjac=r)
        be.run_kernels([k], wait=True)
        return {'tdivtconf': get_scal(t)}

    if mod.endswith('rkvdh2'):
        regs = {a: P.scal(x[a]) for a in ('r1', 'r2', 'rold', 'rerr')}
        be.commit()
        k = be.kernel('rkvdh2', tplargs=tp, dims=[1, n], dt=float(x['dt']),
                      **regs)
        be.run_kernels([k], wait=True)
        return {a: get_scal(M) for a, M in regs.items()}

    raise KeyError(mod)


def test_cuda_kernels_match_reference_kernels(built, pw):
    g, meta = pw
    worst, missing = {}, []
    for name, m in meta.items():
        be = _backend()
        x = _inputs(g, m['family'])
        got = run_variant(be, m, x)
        for o in m['outputs']:
            ref = g[f'out:{name}:{o}']
            worst[f'{name}:{o}'] = _relerr(np.reshape(got[o], ref.shape), ref)
    bad = {k: v for k, v in worst.items() if not v <= TOL}
    assert not bad, bad
    assert not missing


@pytest.mark.parametrize('rsolver', ['hll', 'roe', 'roem', 'exact'])
def test_euler_rhs_other_riemann_solvers(built, rsolver):
    """The right-hand side with each further Riemann solver against the
    oracle (distorted quad mesh of the 2-D vortex) at 1e-10."""
    from oracle.fr_oracle import RSOLVERS  # noqa: F401
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.solvers.system import EulerSystem
    from tests.oracle_util import disc_for_mesh
    cfg, mesh = euler_vortex(n=8, order=3, rsolver=rsolver)
    from pyfr_gb300.backend import B200Backend
    be = B200Backend(cfg)
    s = EulerSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    d = disc_for_mesh(mesh, 3)
    ref = d.rhs_euler(u, cfg.items_as('constants', float), rsolver=rsolver)
    err = np.abs(r - ref).max()/np.abs(ref).max()
    assert err < 1e-10, err
