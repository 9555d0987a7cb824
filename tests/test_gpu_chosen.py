"""The chosen precision form: FP32 right-hand side (operators and fluxes),
FP64 solution accumulation.  Its solution must stay within a relative L2
error of 1e-6 of the FP64 oracle; single RHS evaluations are checked at
FP32 accuracy (relative max-norm 1e-4 of the RHS scale)."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step
from tests.oracle_util import disc_for_mesh

pytestmark = pytest.mark.gpu

L2_TOL = 1e-6


def _l2rel(a, b):
    return np.linalg.norm((a - b).ravel())/np.linalg.norm(b.ravel())


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


@pytest.mark.parametrize('key', ['hex_p3_gauss-legendre', 'quad_p3_gauss-legendre',
                                 'hex_p2_gauss-legendre'])
@pytest.mark.parametrize('opname', ['m0', 'M132', 'm3', 'M460', 'm6'])
def test_mul_bf16x3_tensor_cores(built, golden, key, opname):
    """Split-BF16 tcgen05 operator apply against an FP64 product: the
    error of the three-product split is bounded by ~2^-16 |A||B|."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.inifile import Inifile
    a = golden['operators'][f'{key}/{opname}']
    cfg = Inifile()
    cfg.set('backend', 'precision', 'single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    be = B200Backend(cfg)
    rng = np.random.default_rng(7)
    for nvars, neles in [(5, 77), (4, 1000)]:
        b = rng.normal(size=(a.shape[1], nvars, neles))
        c0 = rng.normal(size=(a.shape[0], nvars, neles))
        A = be.const_matrix(a)
        B = be.matrix(b.shape, b, tags={'align'})
        C = be.matrix(c0.shape, c0, tags={'align'})
        be.commit()
        bound = 1e-4*np.einsum('mk,kve->mve', np.abs(a), np.abs(b)) + 1e-6
        for alpha, beta in [(1.0, 0.0), (1.0, 1.0), (-0.5, 1.0), (2.0, 0.25)]:
            C.set(c0)
            k = be.kernel('mul', A, B, out=C, alpha=alpha, beta=beta)
            # The tensor-core epilogue stores or adds; other beta fall back
            assert k.meta['impl'] == ('bf16x3' if beta in (0.0, 1.0) else 'csr')
            be.run_kernels([k], wait=True)
            ref = alpha*np.einsum('mk,kve->mve', a, b.astype(np.float32)) + \
                beta*c0.astype(np.float32)
            assert np.all(np.abs(C.get() - ref) <= abs(alpha)*bound +
                          1e-6*np.abs(ref))


def test_fp32_ns_rhs(built):
    """The TGV fluxes carry the mean pressure p0 = 1/(gamma Ma^2) ~ 71
    while the RHS is O(1): FP32 rounding of the fluxes (relative 6e-8 of
    p0) is amplified by the divergence and lift operators, so the RHS error
    is bounded relative to p0/h, not to the RHS itself.  A numpy emulation
    of the same arithmetic in float32 gives 6e-5 p0/h on this case; the
    bound is 1e-4 p0/h."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=5, order=3, precision='single')
    be = B200Backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    assert r.dtype == np.float32

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u.astype(np.float64), c)
    h = 2*np.pi/5
    assert np.abs(r - ref).max() <= 1e-4*c['p0']/h


def test_fp32_ns_rhs_reference_shift(built):
    """With the reference-state transform the FP32 input is
    q = T(u - u_ref) (energy replaced by dE - h_ref*drho) and the kernels
    return T times the right-hand side: no flux carries the mean pressure
    or enthalpy any more, so the error is bounded relative to the RHS
    itself (1e-4 on every variable)."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg, mesh = ns_tgv(n=5, order=3, precision='single')
    gamma = cfg.getfloat('constants', 'gamma')
    be = B200Backend(cfg)
    s = NavierStokesSystem(be, mesh, None, 2, cfg)
    (eles,) = s.ele_map.values()
    u = eles.set_ics_from_cfg()
    rho_ref, p_ref = 1.0, cfg.getfloat('constants', 'p0')
    hs = gamma/(gamma - 1)*p_ref/rho_ref
    be.ref_state = (rho_ref, p_ref)
    s.commit()
    uref = np.zeros(5)
    uref[0], uref[-1] = rho_ref, p_ref/(gamma - 1)
    q = u - uref[None, :, None]
    q[:, -1] -= hs*q[:, 0]
    s.ele_banks[0][0].set(q.astype(np.float32))
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3, ns=True)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    ref = d.rhs_ns(u, c)
    ref[:, -1] -= hs*ref[:, 0]
    assert np.abs(r - ref).max() <= 1e-4*np.abs(ref).max()


def test_fp32_euler_rhs(built):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.solvers.system import EulerSystem
    cfg, mesh = euler_vortex(n=12, order=3, precision='single')
    be = B200Backend(cfg)
    s = EulerSystem(be, mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)

    d = disc_for_mesh(mesh, 3)
    ref = d.rhs_euler(u.astype(np.float64), cfg.items_as('constants', float))
    assert np.abs(r - ref).max() <= 1e-4*np.abs(ref).max()


@pytest.mark.parametrize('mulprec', ['native', 'bf16x3'])
@pytest.mark.parametrize('case', ['vortex', 'tgv'])
def test_mixed_rk45_l2_error(built, case, mulprec):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex, ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem

    if case == 'vortex':
        cfg, mesh = euler_vortex(n=10, order=3, dt=2e-3, precision='single')
        scls, nsteps, ns = EulerSystem, 20, False
    else:
        cfg, mesh = ns_tgv(n=5, order=3, dt=5e-4, precision='single')
        scls, nsteps, ns = NavierStokesSystem, 10, True
    cfg.set('backend-b200', 'mul-precision', mulprec)

    be = B200Backend(cfg)
    intg = MixedRKIntegrator(be, scls, mesh, cfg)
    (u,) = intg.soln
    assert u.dtype == np.float64
    intg.run_steps(nsteps)
    (ug,) = intg.soln

    d = disc_for_mesh(mesh, 3, ns=ns)
    c = cfg.items_as('constants', float) | cfg.items_as('solver-interfaces',
                                                       float)
    rhs = (lambda x: d.rhs_ns(x, c)) if ns else (lambda x: d.rhs_euler(x, c))
    for _ in range(nsteps):
        u = rk45_step(rhs, u, intg.dt)

    assert _l2rel(ug, u) <= L2_TOL


def test_kinetic_energy_history(built):
    """Kinetic-energy history of the chosen form against the FP64 plain
    form.  The history is the normalised Taylor-Green kinetic energy
    E_k = int rho |u|^2 / (2 rho0 V) (about 0.125 here); the chosen form
    must stay within 1e-8 of the FP64 value at every logged step."""
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.plugins import FieldIntegrals
    from pyfr_gb300.solvers.system import NavierStokesSystem

    hist = {}
    for form, prec, icls in [('plain', 'double', RKVdH2Integrator),
                             ('chosen', 'single', MixedRKIntegrator)]:
        cfg, mesh = ns_tgv(n=6, order=3, dt=5e-4, precision=prec)
        intg = icls(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
        fi = FieldIntegrals(intg)
        h = []
        for _ in range(10):
            intg.run_steps(2)
            r = fi()
            h.append(0.5*r['E']/r['vol'])
        hist[form] = np.array(h)

    assert np.abs(hist['chosen'] - hist['plain']).max() <= 1e-8
