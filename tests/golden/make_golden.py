"""Generate golden fixtures from the reference implementation itself.

Run where the PyFR source tree is present (read-only), named by the
``PYFR_REFERENCE`` environment variable (default ``/root/reference``); the
GPU hosts do not need it, they use the committed ``.npz`` files this script
writes next to itself:

  PYFR_REFERENCE=/path/to/PyFR python tests/golden/make_golden.py [step...]

What is generated (all with the reference's own code):

* ``operators.npz``: for each (shape, order, point set) the operator
  matrices m0, m1, m2, m3, m4, m6 and the combined expressions
  'M1 - M3*M2', 'M4 - M6*M0' from ``pyfr.shapes`` (``opmat``), plus the
  solution/flux points, face normals and face point lists.  Before writing,
  the hex p=3 Gauss-Legendre matrices are checked against the reference's
  own golden file ``pyfr/tests/hex-gleg-ord3.npz`` (its unit test
  ``pyfr/tests/test_ele_mats.py``).
* ``bases.npz``: the orthonormal simplex bases at the solution points.
* ``surf_flux.npz``: operators with surface-flux anti-aliasing.
* pyramids (``make_pyr``): the pyramid's operators at orders 1-4, the
  geometry of pyramids whose maps are not affine, and a periodic box where
  hexahedra meet tetrahedra through pyramids.
* ``geometry_<case>.npz``: element geometry computed by the reference's
  ``EulerElements``/``NavierStokesElements`` (``pyfr/solvers/base/elements.py``)
  on small periodic meshes whose interior vertices are randomly perturbed
  (valid multilinear elements): sorted face flux points, scaled normals,
  1/|J| at the solution points, metric terms and physical point locations,
  and the initial conditions evaluated by ``set_ics_from_cfg``.

The reference needs third-party packages that are not installed here
(platformdirs, mako, h5py, mpi4py, gimmik, pytools, rtree); none of them is
used by the code paths above, so empty stand-in modules are registered
before importing it.
"""

from io import BytesIO
import os
from pathlib import Path
import sys
import types

import numpy as np

REF = Path(os.environ.get('PYFR_REFERENCE', '/root/reference'))
HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _install_standins():
    class _Any:
        def __init__(self, *a, **k):
            pass

        def __call__(self, *a, **k):
            return _Any()

        def __getattr__(self, n):
            return _Any()

        def __mro_entries__(self, bases):
            return (object,)

    for name in ['platformdirs', 'mako', 'mako.lookup', 'mako.template',
                 'mako.runtime', 'mako.exceptions', 'h5py', 'mpi4py',
                 'mpi4py.MPI', 'gimmik', 'pytools', 'pytools.prefork',
                 'rtree', 'rtree.index']:
        m = types.ModuleType(name)
        m.__getattr__ = lambda n: _Any()
        m.__path__ = []
        sys.modules[name] = m

    sys.modules['platformdirs'].user_cache_dir = lambda *a, **k: '/tmp/pyfrc'
    sys.modules['mpi4py.MPI'].__file__ = 'libc.so.6'
    sys.modules['mpi4py'].MPI = sys.modules['mpi4py.MPI']


def _cfg(etype, order, upts, fpts, consts=None, ics=None, extra=()):
    from pyfr.inifile import Inifile

    cfg = Inifile()
    cfg.set('solver', 'order', str(order))
    if isinstance(fpts, str):
        fkind = {'quad': 'line', 'hex': 'quad', 'tri': 'line',
                 'tet': 'tri'}[etype]
        fpts = {fkind: fpts}
    for fkind, rule in fpts.items():
        cfg.set(f'solver-interfaces-{fkind}', 'flux-pts', rule)
    cfg.set(f'solver-elements-{etype}', 'soln-pts', upts)
    for k, v in (consts or {}).items():
        cfg.set('constants', k, repr(v))
    for k, v in (ics or {}).items():
        cfg.set('soln-ics', k, v)
    for s, k, v in extra:
        cfg.set(s, k, v)
    return cfg


OPERATOR_CASES = [
    ('quad', 2, 'gauss-legendre'), ('quad', 3, 'gauss-legendre'),
    ('quad', 4, 'gauss-legendre'), ('quad', 3, 'gauss-legendre-lobatto'),
    ('hex', 2, 'gauss-legendre'), ('hex', 3, 'gauss-legendre'),
    ('hex', 4, 'gauss-legendre'),
]


# Simplex and prism shapes with the reference's named 'alpha-opt' point
# sets: (etype, order, solution points, flux points per face kind)
SIMPLEX_CASES = [
    ('tri', p, 'alpha-opt', {'line': 'gauss-legendre'}) for p in (2, 3, 4)
] + [
    ('tet', p, 'alpha-opt', {'tri': 'alpha-opt'}) for p in (2, 3, 4)
] + [
    ('pri', p, 'alpha-opt~gauss-legendre-lobatto',
     {'tri': 'alpha-opt', 'quad': 'gauss-legendre'}) for p in (2, 3, 4)
]


def _store_shape(out, key, s):
    for m in ('m0', 'm1', 'm2', 'm3', 'm4', 'm6'):
        out[f'{key}/{m}'] = getattr(s, m)
    out[f'{key}/M132'] = s.opmat('M1 - M3*M2')
    out[f'{key}/M460'] = s.opmat('M4 - M6*M0')
    out[f'{key}/upts'] = s.upts
    out[f'{key}/fpts'] = s.fpts
    out[f'{key}/norm_fpts'] = s.norm_fpts
    out[f'{key}/nfacefpts'] = np.array(s.nfacefpts)


def make_operators():
    from pyfr.shapes import HexShape, PriShape, QuadShape, TetShape, TriShape

    shapes = {'quad': QuadShape, 'hex': HexShape, 'tri': TriShape,
              'tet': TetShape, 'pri': PriShape}
    out = {}
    for etype, order, upts, fpts in SIMPLEX_CASES:
        cfg = _cfg(etype, order, upts, fpts)
        _store_shape(out, f'{etype}_p{order}_{upts}', shapes[etype](None, cfg))

    for etype, order, pts in OPERATOR_CASES:
        cfg = _cfg(etype, order, pts, pts)
        s = shapes[etype](None, cfg)
        key = f'{etype}_p{order}_{pts}'
        for m in ('m0', 'm1', 'm2', 'm3', 'm4', 'm6'):
            out[f'{key}/{m}'] = getattr(s, m)
        out[f'{key}/M132'] = s.opmat('M1 - M3*M2')
        out[f'{key}/M460'] = s.opmat('M4 - M6*M0')
        out[f'{key}/upts'] = s.upts
        out[f'{key}/fpts'] = s.fpts
        out[f'{key}/norm_fpts'] = s.norm_fpts
        out[f'{key}/nfacefpts'] = np.array(s.nfacefpts)

    # Flux anti-aliasing operators (default quadrature: Gauss-Legendre,
    # (p + 2)^ndims points)
    for etype in ('quad', 'hex'):
        cfg = _cfg(etype, 3, 'gauss-legendre', 'gauss-legendre',
                   extra=[('solver', 'anti-alias', 'flux')])
        s = shapes[etype](None, cfg)
        key = f'{etype}_p3_aa'
        out[f'{key}/m7'] = s.m7
        out[f'{key}/m9'] = s.m9
        out[f'{key}/M1329'] = s.opmat('(M1 - M3*M2)*M9')
        out[f'{key}/qpts'] = s.qpts

    # The reference's own golden values for hex p=3 (test_ele_mats.py)
    ref = np.load(BytesIO((REF / 'pyfr/tests/hex-gleg-ord3.npz').read_bytes()))
    for m in ('m0', 'm1', 'm2', 'm3'):
        if not np.allclose(ref[m], out[f'hex_p3_gauss-legendre/{m}']):
            raise RuntimeError(f'reference {m} does not match its golden file')
        out[f'refgolden/hex_p3/{m}'] = ref[m]

    np.savez_compressed(HERE / 'operators.npz', **out)
    print('operators.npz:', len(out), 'arrays')


def perturbed_box(etype, n, lo, hi, amp, seed):
    """Periodic box with interior vertices jittered (same jitter on
    periodic images so the mesh stays periodic)."""
    sys.path.insert(0, str(REPO))
    from pyfr_gb300.mesh import periodic_box

    mesh = periodic_box(etype, n, lo, hi)
    ndims = mesh.ndims
    h = (hi - lo)/n
    rng = np.random.default_rng(seed)
    jit = rng.uniform(-amp*h, amp*h, size=(n,)*ndims + (ndims,))

    spts = mesh.spts[etype]
    for v in range(spts.shape[0]):
        idx = np.rint((spts[v] - lo)/h).astype(int) % n      # (neles, ndims)
        spts[v] += jit[tuple(idx[:, d] for d in range(ndims))]
    return mesh


GEOM_CASES = {
    'quad_p3': dict(etype='quad', order=3, n=4, system='euler'),
    'hex_p3': dict(etype='hex', order=3, n=3, system='navier-stokes'),
}


def make_geometry():
    from pyfr.shapes import HexShape, QuadShape
    from pyfr.solvers.euler.elements import EulerElements
    from pyfr.solvers.navstokes.elements import NavierStokesElements

    shapes = {'quad': QuadShape, 'hex': HexShape}
    for name, c in GEOM_CASES.items():
        etype, order, n = c['etype'], c['order'], c['n']
        mesh = perturbed_box(etype, n, -1.0, 1.0, 0.12, seed=7)
        spts = mesh.spts[etype]

        if etype == 'quad':
            ics = dict(rho='1 + 0.2*sin(pi*x)*cos(pi*y)', u='0.5 + 0.1*y',
                       v='-0.3 + 0.1*x', p='1 + 0.1*cos(pi*x)')
            elescls = EulerElements
        else:
            ics = dict(rho='1 + 0.2*sin(pi*x)*cos(pi*y)*cos(pi*z)',
                       u='0.5 + 0.1*y', v='-0.3 + 0.1*z', w='0.2*x',
                       p='1 + 0.1*cos(pi*x)')
            elescls = NavierStokesElements

        cfg = _cfg(etype, order, 'gauss-legendre', 'gauss-legendre',
                   consts=dict(gamma=1.4), ics=ics)
        e = elescls(shapes[etype], spts, cfg)

        out = dict(spts=spts, upts=e.basis.upts, fpts=e.basis.fpts)
        for fi, sf in enumerate(e.srtd_face_fpts):
            out[f'srtd_face_fpts/{fi}'] = sf
        out['pnorm_fpts'] = e._pnorm_fpts
        out['rcpdjac_upts'] = e.rcpdjac_at_np('upts')
        out['smat_upts'] = e.smat_at_np('upts')
        out['ploc_upts'] = e.ploc_at_np('upts')
        out['ics'] = e.set_ics_from_cfg()
        lhs, rhs = mesh.con
        out['lhs'] = np.stack([lhs.eidxs, lhs.fidxs], axis=1)
        out['rhs'] = np.stack([rhs.eidxs, rhs.fidxs], axis=1)
        for k, v in ics.items():
            out[f'icexpr/{k}'] = np.array(v)

        np.savez_compressed(HERE / f'geometry_{name}.npz', **out)
        print(f'geometry_{name}.npz')


def _literal(pts):
    """A point set in the reference's literal rule syntax."""
    return ', '.join('(' + ', '.join(repr(float(x)) for x in p) + ')'
                     for p in pts)


def perturbed_mixed_box(kinds, n, lo, hi, amp, seed):
    """Mixed periodic box with every grid vertex jittered (periodic images
    and all elements sharing a vertex move together)."""
    sys.path.insert(0, str(REPO))
    from pyfr_gb300.mesh import mixed_box

    mesh = mixed_box(n, lo, hi, kinds)
    h = (hi - lo)/n
    rng = np.random.default_rng(seed)
    jit = rng.uniform(-amp*h, amp*h, size=(n, n, n, 3))
    for sp in mesh.spts.values():
        for v in range(sp.shape[0]):
            idx = np.rint((sp[v] - lo)/h).astype(int) % n
            sp[v] += jit[idx[:, 0], idx[:, 1], idx[:, 2]]
    return mesh


MIXED_CASES = {'hexpri_p3': ('hex-pri', 3), 'pritet_p3': ('pri-tet', 3)}


def make_mixed():
    """Operators (in this package's point order, handed to the reference
    as literal point sets) and element geometry of the mixed meshes."""
    from pyfr.shapes import HexShape, PriShape, TetShape
    from pyfr.solvers.euler.elements import EulerElements
    from pyfr_gb300.quadrules import point_set

    shapes = {'hex': HexShape, 'pri': PriShape, 'tet': TetShape}
    ops = dict(np.load(HERE / 'operators.npz'))
    for name, (kinds, order) in MIXED_CASES.items():
        mesh = perturbed_mixed_box(kinds, 2, -1.0, 1.0, 0.1, seed=11)
        upts = {'hex': 'gauss-legendre',
                'pri': _literal(point_set(
                    'pri', 'alpha-opt~gauss-legendre-lobatto', order)),
                'tet': _literal(point_set('tet', 'alpha-opt', order))}
        fpts = {'quad': 'gauss-legendre',
                'tri': _literal(point_set('tri', 'alpha-opt', order))}
        ics = dict(rho='1 + 0.2*sin(pi*x)*cos(pi*y)*cos(pi*z)',
                   u='0.5 + 0.1*y', v='-0.3 + 0.1*z', w='0.2*x',
                   p='1 + 0.1*cos(pi*x)')
        out = {}
        for et, spts in mesh.spts.items():
            cfg = _cfg(et, order, upts[et], fpts, consts=dict(gamma=1.4),
                       ics=ics)
            e = EulerElements(shapes[et], spts, cfg)
            b = e.basis
            key = f'{et}_p{order}_mixed'
            _store_shape(ops, key, b)
            out[f'{et}/spts'] = spts
            for fi, sf in enumerate(e.srtd_face_fpts):
                out[f'{et}/srtd_face_fpts/{fi}'] = sf
            out[f'{et}/pnorm_fpts'] = e._pnorm_fpts
            out[f'{et}/rcpdjac_upts'] = e.rcpdjac_at_np('upts')
            out[f'{et}/smat_upts'] = e.smat_at_np('upts')
            out[f'{et}/ploc_upts'] = e.ploc_at_np('upts')
            out[f'{et}/ics'] = e.set_ics_from_cfg()
        lhs, rhs = mesh.con
        out['lhs'] = np.stack([lhs.etypes, lhs.eidxs.astype(str),
                               lhs.fidxs.astype(str)], axis=1)
        out['rhs'] = np.stack([rhs.etypes, rhs.eidxs.astype(str),
                               rhs.fidxs.astype(str)], axis=1)
        for k, v in ics.items():
            out[f'icexpr/{k}'] = np.array(v)
        np.savez_compressed(HERE / f'geometry_{name}.npz', **out)
        print(f'geometry_{name}.npz')
    np.savez_compressed(HERE / 'operators.npz', **ops)


PYR_CASES = [(p, r) for p in (1, 2, 3, 4)
             for r in ('gauss-legendre', 'gauss-legendre-lobatto')]


def hexpyrtet_box(n, lo, hi, amp, seed):
    """The hexahedron-pyramid-tetrahedron box with the centre vertex of
    every cut cell (the apex of its pyramids, a vertex of its tetrahedra)
    moved by a random offset: watertight, every element affine, the
    pyramids oblique."""
    sys.path.insert(0, str(REPO))
    from pyfr_gb300.mesh import mixed_box

    mesh = mixed_box(n, lo, hi, 'hex-pyr-tet')
    h = (hi - lo)/n
    rng = np.random.default_rng(seed)
    jit = rng.uniform(-amp*h, amp*h, size=(n, n, n, 3))
    for et, v in (('pyr', 4), ('tet', 3)):
        c = mesh.spts[et][v]
        cell = np.floor((c - lo)/h).astype(int)
        c += jit[cell[:, 0], cell[:, 1], cell[:, 2]]
    return mesh


def make_pyr():
    """Pyramids (appended to ``operators.npz``; ``geometry_pyrskew_p3.npz``
    and ``geometry_hexpyrtet_p3.npz``): the reference's pyramid operators
    at orders 1-4 with its tabulated 'gauss-legendre' and
    'gauss-legendre-lobatto' solution points (Gauss-Legendre flux points on
    the square face, this package's 'alpha-opt' points given literally on
    the triangular faces); the geometry of pyramids with random vertices
    (bases that are not parallelograms: maps that are not affine); and the
    geometry and initial conditions of a periodic box where hexahedra meet
    tetrahedra through pyramids."""
    sys.path.insert(0, str(REPO))
    from pyfr.shapes import HexShape, PyrShape, TetShape
    from pyfr.solvers.euler.elements import EulerElements
    from pyfr_gb300.quadrules import point_set

    ops = dict(np.load(HERE / 'operators.npz'))
    for p, r in PYR_CASES:
        fpts = {'quad': 'gauss-legendre',
                'tri': _literal(point_set('tri', 'alpha-opt', p))}
        _store_shape(ops, f'pyr_p{p}_{r}', PyrShape(None, _cfg('pyr', p, r,
                                                             fpts)))
    np.savez_compressed(HERE / 'operators.npz', **ops)
    print('operators.npz:', len(ops), 'arrays')

    fpts = {'quad': 'gauss-legendre',
            'tri': _literal(point_set('tri', 'alpha-opt', 3))}
    upts = {'hex': 'gauss-legendre', 'pyr': 'gauss-legendre',
            'tet': _literal(point_set('tet', 'alpha-opt', 3))}
    shapes = {'hex': HexShape, 'pyr': PyrShape, 'tet': TetShape}
    ics = dict(rho='1 + 0.2*sin(pi*x)*cos(pi*y)*cos(pi*z)',
               u='0.5 + 0.1*y', v='-0.3 + 0.1*z', w='0.2*x',
               p='1 + 0.1*cos(pi*x)')

    def elements(et, spts):
        cfg = _cfg(et, 3, upts[et], fpts, consts=dict(gamma=1.4), ics=ics)
        return EulerElements(shapes[et], spts, cfg)

    # Pyramids with random vertices about the reference pyramid
    rng = np.random.default_rng(5)
    base = np.array([(-1, -1, -1), (1, -1, -1), (-1, 1, -1), (1, 1, -1),
                     (0, 0, 1)], dtype=float)
    spts = base[:, None, :]*0.5 + rng.uniform(-0.12, 0.12, size=(5, 6, 3))
    e = elements('pyr', spts)
    out = dict(spts=spts, pnorm_fpts=e._pnorm_fpts,
               rcpdjac_upts=e.rcpdjac_at_np('upts'),
               smat_upts=e.smat_at_np('upts'), ploc_upts=e.ploc_at_np('upts'),
               ics=e.set_ics_from_cfg())
    np.savez_compressed(HERE / 'geometry_pyrskew_p3.npz', **out)
    print('geometry_pyrskew_p3.npz')

    mesh = hexpyrtet_box(2, -1.0, 1.0, 0.15, seed=13)
    out = {}
    for et, spts in mesh.spts.items():
        e = elements(et, spts)
        out[f'{et}/spts'] = spts
        for fi, sf in enumerate(e.srtd_face_fpts):
            out[f'{et}/srtd_face_fpts/{fi}'] = sf
        out[f'{et}/pnorm_fpts'] = e._pnorm_fpts
        out[f'{et}/rcpdjac_upts'] = e.rcpdjac_at_np('upts')
        out[f'{et}/smat_upts'] = e.smat_at_np('upts')
        out[f'{et}/ploc_upts'] = e.ploc_at_np('upts')
        out[f'{et}/ics'] = e.set_ics_from_cfg()
    lhs, rhs = mesh.con
    out['lhs'] = np.stack([lhs.etypes, lhs.eidxs.astype(str),
                           lhs.fidxs.astype(str)], axis=1)
    out['rhs'] = np.stack([rhs.etypes, rhs.eidxs.astype(str),
                           rhs.fidxs.astype(str)], axis=1)
    for k, v in ics.items():
        out[f'icexpr/{k}'] = np.array(v)
    np.savez_compressed(HERE / 'geometry_hexpyrtet_p3.npz', **out)
    print('geometry_hexpyrtet_p3.npz')


def make_bases():
    """``bases.npz``: the reference's orthonormal simplex and pyramid bases
    (``pyfr.polys``) at the solution points of tri, tet, pri and pyr at
    orders 1-4 (their degree tuples too), which the entropy filter and the
    shock sensor group by degree."""
    from pyfr.polys import get_polybasis
    from pyfr.quadrules import get_quadrule

    rules = {'tri': 'alpha-opt', 'tet': 'alpha-opt',
             'pri': 'alpha-opt~gauss-legendre-lobatto',
             'pyr': 'gauss-legendre'}
    out = {}
    for kind, rule in rules.items():
        for p in range(1, 5):
            npts = len(get_polybasis(kind, p, None).degrees)
            pts = get_quadrule(kind, rule, npts).pts
            b = get_polybasis(kind, p, pts)
            out[f'{kind}_p{p}/pts'] = np.asarray(pts)
            out[f'{kind}_p{p}/vdm'] = np.asarray(b.vdm)
            out[f'{kind}_p{p}/degrees'] = np.asarray(b.degrees)
    np.savez_compressed(HERE / 'bases.npz', **out)
    print('bases.npz')


def make_surf():
    """``surf_flux.npz``: the reference's operators with surface-flux
    anti-aliasing (``anti-alias = surf-flux``, its default face rules) for
    quadrilaterals and hexahedra at orders 2 and 3: flux points, M0, M3."""
    from pyfr.inifile import Inifile
    from pyfr.shapes import HexShape, QuadShape

    out = {}
    for name, cls, fk in (('quad', QuadShape, 'line'),
                          ('hex', HexShape, 'quad')):
        for p in (2, 3):
            cfg = Inifile()
            cfg.set('solver', 'order', p)
            cfg.set('solver', 'anti-alias', 'surf-flux')
            cfg.set(f'solver-elements-{name}', 'soln-pts', 'gauss-legendre')
            cfg.set(f'solver-interfaces-{fk}', 'flux-pts', 'gauss-legendre')
            s = cls(None, cfg)
            key = f'{name}_p{p}'
            out[f'{key}/fpts'] = np.asarray(s.fpts)
            out[f'{key}/m0'] = np.asarray(s.m0)
            out[f'{key}/m3'] = np.asarray(s.m3)
    np.savez_compressed(HERE / 'surf_flux.npz', **out)
    print('surf_flux.npz')


if __name__ == '__main__':
    sys.path.insert(0, str(REF))
    _install_standins()
    steps = dict(operators=make_operators, geometry=make_geometry,
                 mixed=make_mixed, bases=make_bases, surf=make_surf,
                 pyr=make_pyr)
    for name in sys.argv[1:] or list(steps):
        steps[name]()
