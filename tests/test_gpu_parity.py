"""Parity of the CUDA path (through the b200 backend and the C ABI) with the
CPU oracle.  Plain FP64: relative max-norm tolerance 1e-10 on every
conserved variable, as required of the plain form."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step
from tests.oracle_util import basis_of, disc_for_mesh, ops_from_golden
from oracle.fr_oracle import Discretisation

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _backend(cfg, graphs=True):
    from pyfr_gb300.backend import B200Backend
    cfg.set('backend-b200', 'cuda-graphs', str(graphs).lower())
    return B200Backend(cfg)


def _golden_mesh(g, etype):
    from pyfr_gb300.mesh import Mesh, Side
    n = len(g['lhs'])
    lhs = Side([etype]*n, g['lhs'][:, 0], g['lhs'][:, 1])
    rhs = Side([etype]*n, g['rhs'][:, 0], g['rhs'][:, 1])
    nd = g['spts'].shape[2]
    return Mesh(ndims=nd, spts={etype: g['spts']}, con=(lhs, rhs),
                spts_curved={etype: np.zeros(g['spts'].shape[1], bool)},
                periods=(2.0,)*nd)


# ---------------------------------------------------------------------------

@pytest.mark.parametrize('key', ['quad_p3_gauss-legendre', 'hex_p3_gauss-legendre',
                                 'hex_p4_gauss-legendre', 'quad_p2_gauss-legendre'])
@pytest.mark.parametrize('opname', ['m0', 'M132', 'm3', 'M460', 'm6'])
def test_mul_matches_numpy(built, golden, key, opname):
    from pyfr_gb300.inifile import Inifile
    a = golden['operators'][f'{key}/{opname}']
    cfg = Inifile()
    be = _backend(cfg)
    rng = np.random.default_rng(3)
    nvars, neles = 5, 77
    b = rng.normal(size=(a.shape[1], nvars, neles))
    c0 = rng.normal(size=(a.shape[0], nvars, neles))

    A = be.const_matrix(a)
    B = be.matrix(b.shape, b, tags={'align'})
    C = be.matrix(c0.shape, c0, tags={'align'})
    be.commit()

    for alpha, beta in [(1.0, 0.0), (2.0, 1.0), (-0.5, 0.25)]:
        C.set(c0)
        be.run_kernels([be.kernel('mul', A, B, out=C, alpha=alpha, beta=beta)],
                       wait=True)
        ref = alpha*np.einsum('mk,kve->mve', a, b) + beta*c0
        np.testing.assert_allclose(C.get(), ref, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize('rsolver', ['rusanov', 'hllc'])
def test_euler_rhs_vortex(built, rsolver):
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.solvers.system import EulerSystem
    cfg, mesh = euler_vortex(n=12, order=3, rsolver=rsolver)
    be = _backend(cfg)
    s = EulerSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3)
    ref = d.rhs_euler(u, cfg.items_as('constants', float), rsolver)
    assert _relerr(r, ref) < TOL


def test_euler_rhs_distorted_mesh_reference_geometry(built, golden):
    """Distorted periodic quads; the oracle uses the reference's operator
    matrices and the reference's initial condition."""
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.solvers.system import EulerSystem
    from pyfr_gb300.shapes import get_shape
    g = golden['geometry_quad_p3']
    mesh = _golden_mesh(g, 'quad')
    cfg = Inifile()
    cfg.set('constants', 'gamma', 1.4)
    cfg.set('solver', 'order', 3)
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    be = _backend(cfg)
    s = EulerSystem(be, mesh, {'quad': g['ics']}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    ops = ops_from_golden(golden['operators'], 'quad_p3_gauss-legendre')
    d = Discretisation(ops, basis_of(get_shape('quad', 3)), g['spts'],
                       g['lhs'], g['rhs'], periods=(2.0, 2.0))
    ref = d.rhs_euler(g['ics'], dict(gamma=1.4))
    assert _relerr(r, ref) < TOL


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
@pytest.mark.parametrize('graphs', [True, False])
def test_euler_rhs_flux_antialiasing(built, golden, case, etype, graphs):
    """Flux anti-aliasing (solution interpolated to the (p+2)^d
    Gauss-Legendre points, flux there, projected back by M9) on distorted
    meshes against the oracle with the reference's operators."""
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.solvers.system import EulerSystem
    from pyfr_gb300.shapes import get_shape
    g = golden[f'geometry_{case}']
    mesh = _golden_mesh(g, etype)
    nd = mesh.ndims
    cfg = Inifile()
    cfg.set('constants', 'gamma', 1.4)
    cfg.set('solver', 'order', 3)
    cfg.set('solver', 'anti-alias', 'flux')
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    be = _backend(cfg, graphs)
    ics = g['ics'][:, :nd + 2]
    s = EulerSystem(be, mesh, {etype: ics}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    ops = ops_from_golden(golden['operators'], f'{etype}_p3_gauss-legendre')
    ref = golden['operators']
    aa = dict(M7=ref[f'{etype}_p3_aa/m7'], M1329=ref[f'{etype}_p3_aa/M1329'],
              qpts=ref[f'{etype}_p3_aa/qpts'])
    d = Discretisation(ops, basis_of(get_shape(etype, 3)), g['spts'],
                       g['lhs'], g['rhs'], periods=(2.0,)*nd, aa=aa)
    assert _relerr(r, d.rhs_euler(ics, dict(gamma=1.4))) < TOL


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
@pytest.mark.parametrize('artvisc', [False, True])
def test_ns_rhs_flux_antialiasing(built, golden, case, etype, artvisc):
    """Navier-Stokes flux anti-aliasing: the solution and the physical
    gradient interpolated to the quadrature points, the unfused flux there
    (with the artificial viscosity at those points), projected back by M9,
    on distorted meshes against the oracle with the reference's
    operators."""
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.mesh import vertex_nodes
    from pyfr_gb300.shapes import get_shape, linear_shape_fn
    from pyfr_gb300.polys import modal_basis
    from pyfr_gb300.solvers.artvisc import sensor_params
    from pyfr_gb300.solvers.system import NavierStokesSystem
    g = golden[f'geometry_{case}']
    mesh = _golden_mesh(g, etype)
    nd = mesh.ndims
    c = dict(gamma=1.4, mu=0.05, Pr=0.72, **{'ldg-beta': 0.5,
                                             'ldg-tau': 0.1})
    cfg = Inifile()
    for k in ('gamma', 'mu', 'Pr'):
        cfg.set('constants', k, c[k])
    cfg.set('solver', 'order', 3)
    cfg.set('solver', 'anti-alias', 'flux')
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    cfg.set('solver-interfaces', 'ldg-beta', 0.5)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    avc = {'max-artvisc': 0.02, 'kappa': 1.5, 's0': 0.01}
    if artvisc:
        cfg.set('solver', 'shock-capturing', 'artificial-viscosity')
        for k, v in avc.items():
            cfg.set('solver-artificial-viscosity', k, v)
    ics = g['ics'][:, :nd + 2]
    s = NavierStokesSystem(_backend(cfg, True), mesh, {etype: ics}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    ops = ops_from_golden(golden['operators'], f'{etype}_p3_gauss-legendre',
                          ns=True)
    ref = golden['operators']
    aa = dict(M7=ref[f'{etype}_p3_aa/m7'], M1329=ref[f'{etype}_p3_aa/M1329'],
              qpts=ref[f'{etype}_p3_aa/qpts'])
    shp = get_shape(etype, 3)
    av = None
    if artvisc:
        degs, *_ = sensor_params(*modal_basis(shp)[1:], 3)
        vn, nn = vertex_nodes(mesh)
        av = dict(invvdm=np.linalg.inv(shp.ubasis.vdm).T, degs=degs, order=3,
                  c=avc, vnodes=vn[etype], nnodes=nn,
                  opf=linear_shape_fn(etype, shp.fpts),
                  opu=linear_shape_fn(etype, aa['qpts']))
    d = Discretisation(ops, basis_of(shp), g['spts'], g['lhs'], g['rhs'],
                       periods=(2.0,)*nd, aa=aa)
    assert _relerr(r, d.rhs_ns(ics, c, av=av)) < TOL


def test_ns_rhs_distorted_hex_reference_geometry(built, golden):
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.solvers.system import NavierStokesSystem
    from pyfr_gb300.shapes import get_shape
    g = golden['geometry_hex_p3']
    mesh = _golden_mesh(g, 'hex')
    cfg = Inifile()
    for k, v in dict(gamma=1.4, mu=0.05, Pr=0.72).items():
        cfg.set('constants', k, v)
    cfg.set('solver', 'order', 3)
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    cfg.set('solver-interfaces', 'ldg-beta', 0.5)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    be = _backend(cfg)
    s = NavierStokesSystem(be, mesh, {'hex': g['ics']}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    ops = ops_from_golden(golden['operators'], 'hex_p3_gauss-legendre', True)
    d = Discretisation(ops, basis_of(get_shape('hex', 3)), g['spts'],
                       g['lhs'], g['rhs'], periods=(2.0,)*3)
    c = dict(gamma=1.4, mu=0.05, Pr=0.72, **{'ldg-beta': 0.5, 'ldg-tau': 0.1})
    ref = d.rhs_ns(g['ics'], c)
    assert _relerr(r, ref) < TOL


@pytest.mark.parametrize('beta,tau,rsolver', [(0.5, 0.1, 'rusanov'),
                                              (0.0, 0.2, 'hllc'),
                                              (-0.5, 0.0, 'rusanov')])
def test_ns_rhs_tgv(built, beta, tau, rsolver):
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=5, order=3, beta=beta, tau=tau, rsolver=rsolver)
    be = _backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u, c, rsolver)
    assert _relerr(r, ref) < TOL


@pytest.mark.parametrize('prec', ['double', 'single'])
def test_ns_rhs_large_memory_model(built, prec):
    """memory-model = large: 64-bit interface gather maps (the reference's
    ixdtype int64), as the 128^3 configuration needs; same RHS as the
    oracle (FP64: 1e-10; FP32: 1e-4 of p0/h)."""
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4, order=3, precision=prec)
    cfg.set('backend', 'memory-model', 'large')
    be = _backend(cfg)
    assert be.ixdtype == np.int64
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u.astype(np.float64), c)
    if prec == 'double':
        assert _relerr(r, ref) < TOL
    else:
        assert np.abs(r - ref).max() <= 1e-4*c['p0']/(2*np.pi/4)


@pytest.mark.parametrize('graphs', [True, False])
def test_pi_controller_steps(built, graphs):
    """Adaptive RK45 under the PI controller (the step size read from
    device memory inside the captured step graphs): the accepted steps,
    replayed with the same dt sequence on the oracle, agree to 1e-10."""
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4, order=3, dt=2e-3)
    sect = 'solver-time-integrator'
    cfg.set(sect, 'controller', 'pi')
    cfg.set(sect, 'rtol', '1e-7')
    cfg.set(sect, 'atol', '1e-7')
    be = _backend(cfg, graphs)
    intg = RKVdH2Integrator(be, NavierStokesSystem, mesh, cfg)
    (u,) = intg.soln
    intg.run_pi_steps(6)
    (ug,) = intg.soln
    dts = intg.dt_accepted
    assert len(dts) == 6 and len(set(dts)) > 1

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    for dt in dts:
        u = rk45_step(lambda x: d.rhs_ns(x, c), u, dt)
    assert _relerr(ug, u) < TOL


@pytest.mark.parametrize('graphs', [True, False])
def test_rk45_vortex_steps(built, graphs):
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem
    cfg, mesh = euler_vortex(n=10, order=3, dt=2e-3)
    be = _backend(cfg, graphs)
    intg = RKVdH2Integrator(be, EulerSystem, mesh, cfg)
    (u,) = intg.soln
    intg.run_steps(10)
    (ug,) = intg.soln

    d = disc_for_mesh(mesh, 3)
    c = cfg.items_as('constants', float)
    for _ in range(10):
        u = rk45_step(lambda x: d.rhs_euler(x, c), u, intg.dt)
    assert _relerr(ug, u) < TOL


def test_rk45_tgv_steps(built):
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4, order=3, dt=1e-3)
    be = _backend(cfg)
    intg = RKVdH2Integrator(be, NavierStokesSystem, mesh, cfg)
    (u,) = intg.soln
    intg.run_steps(3)
    (ug,) = intg.soln

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    for _ in range(3):
        u = rk45_step(lambda x: d.rhs_ns(x, c), u, intg.dt)
    assert _relerr(ug, u) < TOL


def test_gradients_for_diagnostics(built):
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4, order=3)
    be = _backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.compute_grads(0.0, 0)
    (g,) = s.grad_upts()
    (u,) = s.ele_scal_upts(0)

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    gl = []
    d.rhs_ns(u, c, grads_out=gl)
    assert _relerr(g, gl[0]) < TOL


def test_pi_controller_error_norm(built):
    from pyfr_gb300.inifile import Inifile
    cfg = Inifile()
    be = _backend(cfg)
    rng = np.random.default_rng(5)
    shape = (16, 4, 45)
    cur, err = rng.normal(size=shape), 1e-6*rng.normal(size=shape)
    C = be.matrix(shape, cur, tags={'align'})
    E = be.matrix(shape, err, tags={'align'})
    be.commit()
    atols = [1e-6, 2e-6, 3e-6, 4e-6]
    k = be.kernel('errest', C, E, atols)
    k.bind(rtol=1e-5)
    k.run(be.stream)
    be.wait()
    ref = np.sum((err/(np.array(atols)[None, :, None] + 1e-5*np.abs(cur)))**2)
    assert abs(k.retval[0] - ref) <= 1e-12*ref


def test_field_integrals_plain(built):
    """Kinetic energy and enstrophy integrals against the oracle's
    gradients and the solution-point quadrature."""
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.plugins import FieldIntegrals
    from pyfr_gb300.shapes import tensor_rule
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=4, order=3)
    be = _backend(cfg)
    intg = RKVdH2Integrator(be, NavierStokesSystem, mesh, cfg)
    intg.run_steps(2)
    got = FieldIntegrals(intg)()

    (u,) = intg.soln
    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    gl = []
    d.rhs_ns(u, c, grads_out=gl)
    g = gl[0]                                   # (nd, nupts, nvars, neles)
    _, qw = tensor_rule('gauss-legendre', 4, 3)
    w = qw[:, None]*d.djac_u
    rho = u[:, 0]
    vel = u[:, 1:4]/rho[:, None]
    du = (g[:, :, 1:4] - vel[None]*g[:, :, :1])/rho[None, :, None]  # (d,p,i,e)
    w1 = du[1, :, 2] - du[2, :, 1]
    w2 = du[2, :, 0] - du[0, :, 2]
    w3 = du[0, :, 1] - du[1, :, 0]
    E = np.sum(w*rho*np.sum(vel**2, axis=1))
    enst = np.sum(w*rho*(w1**2 + w2**2 + w3**2))
    assert abs(got['E'] - E) <= 1e-12*E
    assert abs(got['enst'] - enst) <= 1e-10*enst
    assert abs(got['vol'] - (2*np.pi)**3) <= 1e-12*(2*np.pi)**3


@pytest.mark.parametrize('case,etype', [('quad_p3', 'quad'), ('hex_p3', 'hex')])
@pytest.mark.parametrize('system', ['euler', 'navier-stokes'])
@pytest.mark.parametrize('aa', ['surf-flux', 'flux, surf-flux'])
def test_rhs_surface_antialiasing(built, golden, case, etype, system, aa):
    """Surface-flux anti-aliasing (flux points at the (p+2)^(d-1)
    Gauss-Legendre face points, the correction lift through the L2
    projection onto the face basis), alone and with flux anti-aliasing, on
    the reference's distorted meshes against the oracle with the shape's
    operators (pinned to the reference's in tests/test_operators.py)."""
    from pyfr_gb300.inifile import Inifile
    from pyfr_gb300.quadrules import tensor_rule
    from pyfr_gb300.shapes import get_shape
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    from tests.oracle_util import ops_from_shape
    g = golden[f'geometry_{case}']
    mesh = _golden_mesh(g, etype)
    nd = mesh.ndims
    ns = system == 'navier-stokes'
    c = dict(gamma=1.4, mu=0.05, Pr=0.72, **{'ldg-beta': 0.5,
                                             'ldg-tau': 0.1})
    cfg = Inifile()
    for k in ('gamma', 'mu', 'Pr'):
        cfg.set('constants', k, c[k])
    cfg.set('solver', 'order', 3)
    cfg.set('solver', 'anti-alias', aa)
    cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
    cfg.set('solver-interfaces', 'ldg-beta', 0.5)
    cfg.set('solver-interfaces', 'ldg-tau', 0.1)
    ics = g['ics'][:, :nd + 2]
    scls = NavierStokesSystem if ns else EulerSystem
    s = scls(_backend(cfg), mesh, {etype: ics}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    shp = get_shape(etype, 3)
    shp.set_surf_rules({('line' if nd == 2 else 'quad'):
                        tensor_rule('gauss-legendre', 5, nd - 1)})
    daa = None
    if 'flux,' in aa:
        daa = dict(M7=shp.m7, M1329=shp.opmat('(M1 - M3*M2)*M9'),
                   qpts=shp.qpts)
    d = Discretisation(ops_from_shape(shp, ns), basis_of(shp), g['spts'],
                       g['lhs'], g['rhs'], periods=(2.0,)*nd, aa=daa)
    ref = d.rhs_ns(ics, c) if ns else d.rhs_euler(ics, dict(gamma=1.4))
    assert _relerr(r, ref) < TOL
