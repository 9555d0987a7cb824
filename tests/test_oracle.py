"""The oracle against the reference's fixtures and physical invariants."""
import numpy as np
import pytest

from oracle.fr_oracle import Discretisation, hllc, inviscid_flux, rusanov
from tests.oracle_util import basis_of, ops_from_golden
from pyfr_gb300.shapes import get_shape

GAS = dict(gamma=1.4, mu=0.01, Pr=0.72, **{'ldg-beta': 0.5, 'ldg-tau': 0.1})


def _disc(golden, case, etype, ns):
    g = golden[f'geometry_{case}']
    ops = ops_from_golden(golden['operators'], f'{etype}_p3_gauss-legendre',
                          ns)
    s = get_shape(etype, 3)
    return Discretisation(ops, basis_of(s), g['spts'], g['lhs'], g['rhs'],
                          periods=(2.0,)*s.ndims), g


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_oracle_geometry_is_the_references(golden, case, etype):
    d, g = _disc(golden, case, etype, etype == 'hex')
    np.testing.assert_allclose(1/d.djac_u, g['rcpdjac_upts'], rtol=1e-11)
    np.testing.assert_allclose(d.pnorm.transpose(0, 2, 1), g['pnorm_fpts'],
                               rtol=1e-11, atol=1e-13)


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_oracle_pairing_is_the_references(golden, case, etype):
    # The reference pairs the k-th sorted flux point of each side
    d, g = _disc(golden, case, etype, False)
    srt = [g[f'srtd_face_fpts/{f}'] for f in range(len(d.facefpts))]
    ref = set()
    for (el, fl), (er, fr) in zip(g['lhs'], g['rhs']):
        for a, b in zip(srt[fl][el], srt[fr][er]):
            ref.add((a, el, b, er))
    mine = {(a, el, b, er) for (a, el), (b, er) in zip(d.pl, d.pr)}
    assert mine == ref


@pytest.mark.parametrize('rs', [rusanov, hllc])
def test_riemann_consistency_and_symmetry(rs):
    rng = np.random.default_rng(1)
    n = rng.normal(size=(3, 50))
    n /= np.linalg.norm(n, axis=0)
    u = np.stack([1 + 0.1*rng.random(50), *(0.3*rng.normal(size=(3, 50))),
                  2.5 + 0.1*rng.random(50)])
    u2 = u*(1 + 0.05*rng.normal(size=u.shape))
    f, _, _ = inviscid_flux(u, 1.4)
    np.testing.assert_allclose(rs(u, u, n, 1.4),
                               np.einsum('dn,dvn->vn', n, f), atol=1e-13)
    np.testing.assert_allclose(rs(u, u2, n, 1.4), -rs(u2, u, -n, 1.4),
                               atol=1e-12)


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_free_stream_preserved_on_distorted_mesh(golden, case, etype):
    d, g = _disc(golden, case, etype, etype == 'hex')
    nd = d.ndims
    cons = np.array([1.2, *[0.3*(i + 1) for i in range(nd)], 3.0])
    u = np.broadcast_to(cons[None, :, None], (d.nupts, nd + 2, d.neles)).copy()
    r = d.rhs_ns(u, GAS) if etype == 'hex' else d.rhs_euler(u, GAS)
    assert np.abs(r).max() < 1e-11


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_discrete_conservation(golden, case, etype):
    d, g = _disc(golden, case, etype, etype == 'hex')
    u = g['ics']
    r = d.rhs_ns(u, GAS) if etype == 'hex' else d.rhs_euler(u, GAS)
    s = get_shape(etype, 3)
    x, w = np.polynomial.legendre.leggauss(4)
    wts = np.prod(np.array(np.meshgrid(*[w]*s.ndims, indexing='ij')), axis=0)
    wts = wts.T.reshape(-1) if s.ndims == 2 else wts.transpose(2, 1, 0).reshape(-1)
    tot = np.einsum('p,pve,pe->v', wts, r, d.djac_u)
    scale = np.einsum('p,pve,pe->v', wts, np.abs(r), d.djac_u)
    assert np.all(np.abs(tot) <= 1e-12*scale)


# ---------------------------------------------------------------------------
# Meshes of several element types
# ---------------------------------------------------------------------------

MIXED_UPTS = {'hex': 'gauss-legendre', 'pri': 'alpha-opt~gauss-legendre-lobatto',
              'tet': 'alpha-opt', 'pyr': 'gauss-legendre'}
MIXED_FPTS = {'tri': 'alpha-opt', 'quad': 'gauss-legendre'}


def mixed_key(et):
    """Key of the reference's order-3 operators of ``et`` with the mixed
    meshes' point sets in the golden operators."""
    return {'hex': 'hex_p3_gauss-legendre',
            'pyr': 'pyr_p3_gauss-legendre'}.get(et, f'{et}_p3_mixed')


def mixed_disc(golden, case):
    """Oracle discretisation of a golden mixed mesh with the reference's
    operators (hexes: the reference's Gauss-Legendre hex operators)."""
    from oracle.fr_oracle import MixedDiscretisation
    g = golden[f'geometry_{case}']
    ops = golden['operators']
    parts = {}
    for et in ('hex', 'pri', 'tet', 'pyr'):
        if f'{et}/spts' not in g:
            continue
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_golden(ops, mixed_key(et)),
                         basis=basis_of(s), verts=g[f'{et}/spts'])
    return MixedDiscretisation(parts, g['lhs'], g['rhs'],
                               periods=(2.0,)*3), g


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3'])
def test_mixed_oracle_geometry_is_the_references(golden, case):
    d, g = mixed_disc(golden, case)
    for et, e in d.p.items():
        np.testing.assert_allclose(1/e['djac_u'], g[f'{et}/rcpdjac_upts'],
                                   rtol=1e-11)
        np.testing.assert_allclose(e['pnorm'].transpose(0, 2, 1),
                                   g[f'{et}/pnorm_fpts'], rtol=1e-11,
                                   atol=1e-13)


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3'])
def test_mixed_oracle_pairing_is_the_references(golden, case):
    # The reference pairs the k-th sorted flux point of each side
    d, g = mixed_disc(golden, case)
    srt = {et: [g[f'{et}/srtd_face_fpts/{f}'] for f in range(len(e['facefpts']))]
           for et, e in d.p.items()}
    ref = set()
    for (tl, el, fl), (tr, er, fr) in zip(g['lhs'], g['rhs']):
        el, fl, er, fr = int(el), int(fl), int(er), int(fr)
        for a, b in zip(srt[tl][fl][el], srt[tr][fr][er]):
            ref.add((tl, int(a), el, tr, int(b), er))
    tl, fl, el = d.side['l']
    tr, fr, er = d.side['r']
    mine = {(d.etypes[a], int(b), int(c), d.etypes[x], int(y), int(z))
            for a, b, c, x, y, z in zip(tl, fl, el, tr, fr, er)}
    assert mine == ref


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3'])
def test_mixed_free_stream_and_conservation(golden, case):
    from pyfr_gb300.quadrules import EXACT_RULES
    d, g = mixed_disc(golden, case)
    cons = np.array([1.2, 0.3, 0.6, 0.9, 3.0])
    u = {et: np.broadcast_to(cons[None, :, None],
                             (len(e['upts']), 5, e['neles'])).copy()
         for et, e in d.p.items()}
    r = d.rhs_euler(u, GAS)
    assert max(np.abs(v).max() for v in r.values()) < 1e-11

    # The integral of the right-hand side over the mesh vanishes: |J| R is
    # the polynomial -(M132 F + M3 Fc) of the solution space, integrated
    # exactly by interpolation to an exact rule
    r = d.rhs_euler({et: g[f'{et}/ics'] for et in d.p}, GAS)
    tot, scale = 0, 0
    for et, e in d.p.items():
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        qp, qw = EXACT_RULES[et](6)
        L = s.ubasis.nodal_basis_at(qp)
        rq = np.einsum('qp,pve->qve', L, r[et]*e['djac_u'][:, None, :])
        tot = tot + np.einsum('q,qve->v', qw, rq)
        scale = scale + np.einsum('q,qve->v', qw, np.abs(rq))
    assert np.all(np.abs(tot) <= 1e-12*scale)


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
def test_antialiased_free_stream_and_conservation(golden, case, etype):
    """Flux anti-aliasing keeps free-stream preservation and conservation
    (the projection M9 is exact on the polynomial space)."""
    g = golden[f'geometry_{case}']
    ops = ops_from_golden(golden['operators'], f'{etype}_p3_gauss-legendre')
    ref = golden['operators']
    aa = dict(M7=ref[f'{etype}_p3_aa/m7'], M1329=ref[f'{etype}_p3_aa/M1329'],
              qpts=ref[f'{etype}_p3_aa/qpts'])
    s = get_shape(etype, 3)
    d = Discretisation(ops, basis_of(s), g['spts'], g['lhs'], g['rhs'],
                       periods=(2.0,)*s.ndims, aa=aa)
    nd = d.ndims
    cons = np.array([1.2, *[0.3*(i + 1) for i in range(nd)], 3.0])
    u = np.broadcast_to(cons[None, :, None], (d.nupts, nd + 2, d.neles)).copy()
    assert np.abs(d.rhs_euler(u, GAS)).max() < 1e-11

    u = g['ics'][:, :nd + 2] if etype == 'quad' else g['ics']
    r = d.rhs_euler(u, GAS)
    x, w = np.polynomial.legendre.leggauss(4)
    wts = np.prod(np.array(np.meshgrid(*[w]*s.ndims, indexing='ij')), axis=0)
    wts = wts.T.reshape(-1) if s.ndims == 2 else wts.transpose(2, 1, 0).reshape(-1)
    tot = np.einsum('p,pve,pe->v', wts, r, d.djac_u)
    scale = np.einsum('p,pve,pe->v', wts, np.abs(r), d.djac_u)
    assert np.all(np.abs(tot) <= 1e-12*scale)
    # and differs from the collocated flux (aliasing is removed, not zero)
    d0 = Discretisation(ops, basis_of(s), g['spts'], g['lhs'], g['rhs'],
                        periods=(2.0,)*s.ndims)
    assert np.abs(r - d0.rhs_euler(u, GAS)).max() > 1e-8


# ---------------------------------------------------------------------------
# Boundary conditions
# ---------------------------------------------------------------------------

def bc_disc(etype, n, periodic, bcspecs, ns=False):
    """Oracle discretisation of a box with boundaries (product operators;
    the boundary arithmetic is what is under test here)."""
    from pyfr_gb300.mesh import box
    from tests.oracle_util import ops_from_shape
    mesh = box(etype, n, 0.0, 1.0, periodic)
    s = get_shape(etype, 3)
    lhs, rhs = mesh.con
    bcs = [(np.stack([side.eidxs, side.fidxs], 1), bcspecs[name])
           for name, side in sorted(mesh.bcon.items())]
    d = Discretisation(ops_from_shape(s, ns), basis_of(s),
                       mesh.spts[etype], np.stack([lhs.eidxs, lhs.fidxs], 1),
                       np.stack([rhs.eidxs, rhs.fidxs], 1),
                       periods=mesh.periods, bcs=bcs)
    return d, mesh


def _uniform(d, prim, gamma=1.4):
    nd = d.ndims
    rho, vel, p = prim[0], np.array(prim[1:nd + 1]), prim[-1]
    cons = np.array([rho, *(rho*vel), p/(gamma - 1) + 0.5*rho*vel @ vel])
    return np.broadcast_to(cons[None, :, None],
                           (d.nupts, nd + 2, d.neles)).copy()


FREE = dict(rho=1.2, p=0.9, u=[0.4, -0.2, 0.3])


@pytest.mark.parametrize('bctypes', [('sup-in-fa', 'sup-out-fn'),
                                     ('char-riem-inv', 'char-riem-inv'),
                                     ('sup-out-fn', 'char-riem-inv')])
def test_bc_free_stream_euler(bctypes):
    """A free stream at the boundary state is steady through inflow,
    outflow and characteristic boundaries."""
    specs = {'xlo': dict(type=bctypes[0], **FREE),
             'xhi': dict(type=bctypes[1], **FREE)}
    d, _ = bc_disc('quad', (3, 3), (False, True), specs)
    u = _uniform(d, [FREE['rho'], *FREE['u'][:2], FREE['p']])
    assert np.abs(d.rhs_euler(u, GAS)).max() < 1e-11


def test_bc_slip_wall_tangential_stream_and_mass():
    """A stream along slip walls is steady; with any state, no mass crosses
    a slip wall (the total mass is conserved)."""
    specs = {'ylo': dict(type='slp-adia-wall'), 'yhi': dict(type='slp-adia-wall')}
    d, mesh = bc_disc('quad', (3, 4), (True, False), specs)
    u = _uniform(d, [1.1, 0.6, 0.0, 1.3])
    assert np.abs(d.rhs_euler(u, GAS)).max() < 1e-11

    rng = np.random.default_rng(2)
    u = u*(1 + 0.05*rng.normal(size=u.shape))
    r = d.rhs_euler(u, GAS)
    x, w = np.polynomial.legendre.leggauss(4)
    wts = np.outer(w, w).reshape(-1)
    tot = np.einsum('p,pe,pe->', wts, r[:, 0], d.djac_u)
    scale = np.einsum('p,pe,pe->', wts, np.abs(r[:, 0]), d.djac_u)
    assert abs(tot) <= 1e-12*scale


@pytest.mark.parametrize('walls', [('no-slp-adia-wall', 'no-slp-adia-wall'),
                                   ('no-slp-isot-wall', 'slp-adia-wall')])
def test_bc_walls_navier_stokes_rest_state(walls):
    """A gas at rest at the wall temperature is steady between walls."""
    gamma, rho, p = 1.4, 1.0, 1.0/1.4
    cpTw = gamma/(gamma - 1)*p/rho
    specs = {'zlo': dict(type=walls[0], u=[0, 0, 0], cpTw=cpTw),
             'zhi': dict(type=walls[1], u=[0, 0, 0], cpTw=cpTw)}
    d, _ = bc_disc('hex', (2, 2, 3), (True, True, False), specs, ns=True)
    u = _uniform(d, [rho, 0, 0, 0, p])
    assert np.abs(d.rhs_ns(u, GAS)).max() < 1e-11


def test_mixed_ns_oracle_equals_single_type_oracle(golden):
    """The multi-type Navier-Stokes RHS on a one-type mesh is the
    single-type oracle's."""
    from oracle.fr_oracle import MixedDiscretisation
    d, g = _disc(golden, 'hex_p3', 'hex', True)
    ops = ops_from_golden(golden['operators'], 'hex_p3_gauss-legendre', True)
    n = len(g['lhs'])
    m = MixedDiscretisation(
        {'hex': dict(ops=ops, basis=basis_of(get_shape('hex', 3)),
                     verts=g['spts'])},
        [('hex', e, f) for e, f in g['lhs']],
        [('hex', e, f) for e, f in g['rhs']], periods=(2.0,)*3)
    a = m.rhs_ns({'hex': g['ics']}, GAS)['hex']
    b = d.rhs_ns(g['ics'], GAS)
    assert n > 0 and np.abs(a - b).max() <= 1e-13*np.abs(b).max()


@pytest.mark.parametrize('case', ['hexpri_p3', 'pritet_p3'])
def test_mixed_ns_free_stream_and_conservation(golden, case):
    from oracle.fr_oracle import MixedDiscretisation
    from pyfr_gb300.quadrules import EXACT_RULES
    g = golden[f'geometry_{case}']
    ops = golden['operators']
    parts = {}
    for et in ('hex', 'pri', 'tet'):
        if f'{et}/spts' not in g:
            continue
        key = 'hex_p3_gauss-legendre' if et == 'hex' else f'{et}_p3_mixed'
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        parts[et] = dict(ops=ops_from_golden(ops, key, True), basis=basis_of(s),
                         verts=g[f'{et}/spts'])
    d = MixedDiscretisation(parts, g['lhs'], g['rhs'], periods=(2.0,)*3)
    cons = np.array([1.2, 0.3, 0.6, 0.9, 3.0])
    u = {et: np.broadcast_to(cons[None, :, None],
                             (len(e['upts']), 5, e['neles'])).copy()
         for et, e in d.p.items()}
    assert max(np.abs(v).max() for v in d.rhs_ns(u, GAS).values()) < 1e-11

    r = d.rhs_ns({et: g[f'{et}/ics'] for et in d.p}, GAS)
    tot, scale = 0, 0
    for et, e in d.p.items():
        s = get_shape(et, 3, MIXED_UPTS[et], MIXED_FPTS)
        qp, qw = EXACT_RULES[et](6)
        L = s.ubasis.nodal_basis_at(qp)
        rq = np.einsum('qp,pve->qve', L, r[et]*e['djac_u'][:, None, :])
        tot = tot + np.einsum('q,qve->v', qw, rq)
        scale = scale + np.einsum('q,qve->v', qw, np.abs(rq))
    assert np.all(np.abs(tot) <= 1e-12*scale)
