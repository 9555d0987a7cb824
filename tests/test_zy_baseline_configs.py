"""Parity on the benchmark configurations themselves, at their full sizes,
against the C oracle built with IEEE arithmetic (``oracle/fr_oracle.c``,
whose arithmetic equals the numpy oracle's, itself pinned to the
reference's kernels by ``tests/test_pointwise_golden.py``).

* 2-D isentropic vortex: periodic [-10, 10]^2 of 40 x 40 quadrilaterals,
  p = 3, beta = 5, Rusanov, RK45 with dt = 1e-3 for 1000 steps: the plain
  FP64 form within 1e-10 (relative max-norm per conserved variable:
  density, momentum, energy).
* 3-D Taylor-Green vortex: 48^3 hexahedra, p = 3, Re = 1600, Ma = 0.1,
  Rusanov + LDG, RK45 with dt = 5e-4: the plain FP64 form within 1e-10
  after 20 steps, with the kinetic energy and enstrophy integrals compared
  at every one of those steps (1e-10 relative); the chosen precision form
  (split-BF16 operators with the three-term operator, FP32 fluxes, FP64
  accumulation) after 200 steps within relative L2 1e-6 of the oracle's
  FP64 state, its kinetic-energy history within 1e-8 (absolute, on
  E_k = int rho|u|^2 / 2V).

These are the slowest GPU tests (the oracle advances the 48^3 case by
1000 right-hand sides on the host cores), so they are collected last but
one.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ge.build_oracle()


def _relerr_per_var(a, b):
    """Largest over the conserved variables (density, momentum, energy) of
    max|a - b| / max|b|; a and b are (nupts, nvars, neles).  Momentum is
    one (vector) variable: its components' errors are measured against
    the momentum's largest magnitude.  A component on its own is no scale:
    the TGV's z-momentum starts at exactly zero and is 2.5e-3 after 20
    steps, so rounding differences of 1e-13 in it -- the size they have in
    the other components, against which the IEEE oracle and the GPU's
    contracted FP64 differ -- would read as 1.5e-10."""
    nv = b.shape[1]
    groups = [[0], list(range(1, nv - 1)), [nv - 1]]
    return max(np.abs(a[:, g] - b[:, g]).max()/np.abs(b[:, g]).max()
               for g in groups)


def _c_oracle(mesh, cfg, ns):
    from oracle.c_oracle import COracle
    from tests.oracle_util import disc_for_mesh
    d = disc_for_mesh(mesh, 3, ns=ns)
    c = cfg.items_as('constants', float)
    if ns:
        c |= cfg.items_as('solver-interfaces', float)
    return COracle(d, c)


def _rk45(rhs, u, dt):
    from oracle.fr_oracle import rk45_step
    return rk45_step(rhs, u, dt)


def test_vortex_40x40_p3_1000_steps(built):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import euler_vortex
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem

    cfg, mesh = euler_vortex(n=40, order=3, dt=1e-3, beta=5.0)
    intg = RKVdH2Integrator(B200Backend(cfg), EulerSystem, mesh, cfg)
    (u0,) = intg.soln
    intg.run_steps(1000)
    (ug,) = intg.soln
    assert intg.nsteps == 1000

    co = _c_oracle(mesh, cfg, ns=False)
    ue = np.ascontiguousarray(u0.transpose(2, 0, 1))
    for _ in range(1000):
        ue = _rk45(co.rhs_native, ue, 1e-3)
    ref = ue.transpose(1, 2, 0)
    assert _relerr_per_var(ug, ref) < TOL


@pytest.fixture(scope='module')
def tgv48_oracle(built):
    """The oracle's FP64 trajectory of the 48^3 Taylor-Green case: the
    state after 20 and 200 steps, and (E, enstrophy, volume) after every
    step."""
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.quadrules import tensor_rule
    from pyfr_gb300.solvers.elements import NavierStokesElements

    cfg, mesh = ns_tgv(n=48, order=3, dt=5e-4)
    u0 = NavierStokesElements('hex', mesh.spts['hex'], cfg).set_ics_from_cfg()
    co = _c_oracle(mesh, cfg, ns=True)
    _, qw = tensor_rule('gauss-legendre', 4, 3)
    ue = np.ascontiguousarray(u0.transpose(2, 0, 1))
    ints, states = [], {}
    for step in range(1, 201):
        ue = _rk45(co.rhs_native, ue, 5e-4)
        ints.append(co.integrals_native(ue, qw))
        if step in (20, 200):
            states[step] = ue.transpose(1, 2, 0).copy()
    return dict(states=states, ints=np.array(ints))


def test_tgv_48_plain_20_steps_with_integrals(tgv48_oracle):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.plugins import FieldIntegrals
    from pyfr_gb300.solvers.system import NavierStokesSystem

    cfg, mesh = ns_tgv(n=48, order=3, dt=5e-4)
    intg = RKVdH2Integrator(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
    fi = FieldIntegrals(intg)
    got = []
    for _ in range(20):
        intg.run_steps(1)
        r = fi()
        got.append((r['E'], r['enst'], r['vol']))
    (ug,) = intg.soln

    assert _relerr_per_var(ug, tgv48_oracle['states'][20]) < TOL
    got, ref = np.array(got), tgv48_oracle['ints'][:20]
    assert np.all(np.abs(got - ref) <= TOL*np.abs(ref)), \
        np.abs(got - ref).max(axis=0)/np.abs(ref).max(axis=0)


def test_tgv_48_chosen_form_200_steps(tgv48_oracle):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.cases import ns_tgv
    from pyfr_gb300.integrators import MixedRKIntegrator
    from pyfr_gb300.plugins import FieldIntegrals
    from pyfr_gb300.solvers.system import NavierStokesSystem

    cfg, mesh = ns_tgv(n=48, order=3, dt=5e-4, precision='single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '5')
    intg = MixedRKIntegrator(B200Backend(cfg), NavierStokesSystem, mesh, cfg)
    fi = FieldIntegrals(intg)
    ke = []
    for _ in range(200):
        intg.run_steps(1)
        r = fi()
        ke.append(0.5*r['E']/r['vol'])
    (uc,) = intg.soln

    ref = tgv48_oracle['states'][200]
    l2 = np.linalg.norm((uc - ref).ravel())/np.linalg.norm(ref.ravel())
    ints = tgv48_oracle['ints']
    ke_ref = 0.5*ints[:, 0]/ints[:, 2]
    ke_err = np.abs(np.array(ke) - ke_ref).max()
    assert l2 <= 1e-6, l2
    assert ke_err <= 1e-8, ke_err
