"""Boundary conditions through the CUDA path against the oracle
(pyfr/solvers/euler/kernels/bccflux.mako, pyfr/solvers/navstokes/kernels/
{bcconu,bccflux}.mako and the boundary states of */kernels/bcs/*.mako).

Plain FP64: relative max-norm 1e-10 on the right-hand side of boxes bounded
in one direction, for every boundary type, with a non-uniform state; three
RK45 steps with walls; the split-BF16 form against FP64."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step
from tests.bc_cases import FREE, GAS, TOTAL, vc as _vc
from tests.bc_cases import bc_cfg as _cfg
from tests.test_oracle import bc_disc

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


def _backend(cfg):
    from pyfr_gb300.backend import B200Backend
    return B200Backend(cfg)


EULER = [('sup-in-fa', 'sup-out-fn'), ('char-riem-inv', 'char-riem-inv'),
         ('slp-adia-wall', 'slp-adia-wall'), ('sup-out-fn', 'char-riem-inv')]


@pytest.mark.parametrize('types', EULER)
@pytest.mark.parametrize('rsolver', ['rusanov', 'hllc'])
def test_euler_bcs_rhs(built, types, rsolver):
    from pyfr_gb300.solvers.system import EulerSystem
    specs = {'ylo': dict(type=types[0], **FREE),
             'yhi': dict(type=types[1], **FREE)}
    d, mesh = bc_disc('quad', (4, 3), (True, False), specs)
    cfg = _cfg(2, specs, rsolver)
    s = EulerSystem(_backend(cfg), mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    assert _relerr(r, d.rhs_euler(u, GAS, rsolver)) < TOL


NS = [('no-slp-adia-wall', 'no-slp-adia-wall'),
      ('no-slp-isot-wall', 'slp-adia-wall'),
      ('sup-in-fa', 'sup-out-fn'), ('char-riem-inv', 'no-slp-isot-wall'),
      ('sub-in-frv', 'sub-out-fp'), ('sub-in-ftpttang', 'sup-out-fn')]

@pytest.mark.parametrize('types', NS)
def test_ns_bcs_rhs(built, types):
    from pyfr_gb300.solvers.system import NavierStokesSystem
    extra = dict(TOTAL, vc=_vc(TOTAL['theta'], TOTAL['phi']))
    specs = {'zlo': dict(type=types[0], cpTw=3.2, **FREE, **extra),
             'zhi': dict(type=types[1], cpTw=3.6, **FREE, **extra)}
    d, mesh = bc_disc('hex', (2, 2, 3), (True, True, False), specs, ns=True)
    cfg = _cfg(3, specs, ns=True)
    s = NavierStokesSystem(_backend(cfg), mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    assert _relerr(r, d.rhs_ns(u, GAS)) < TOL


def test_ns_walls_rk45(built):
    """Three RK45 steps of a channel between an adiabatic and an
    isothermal no-slip wall (CUDA graphs on)."""
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import NavierStokesSystem
    specs = {'zlo': dict(type='no-slp-adia-wall'),
             'zhi': dict(type='no-slp-isot-wall', cpTw=3.4, u=[0.2, 0, 0])}
    d, mesh = bc_disc('hex', (2, 2, 3), (True, True, False), specs, ns=True)
    cfg = _cfg(3, specs, ns=True)
    intg = RKVdH2Integrator(_backend(cfg), NavierStokesSystem, mesh, cfg)
    (u0,) = intg.soln
    intg.run_steps(3)
    (got,) = intg.soln
    u = u0
    for _ in range(3):
        u = rk45_step(lambda x: d.rhs_ns(x, GAS), u, 1e-3)
    assert _relerr(got, u) < TOL


@pytest.mark.parametrize('types', [EULER[2], EULER[1]])
def test_euler_bcs_chosen_form(built, types):
    """The chosen form with boundaries (no reference-state shift) stays
    within FP32 accuracy of FP64 over ten steps."""
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.mesh import box
    from pyfr_gb300.solvers.system import EulerSystem
    specs = {'ylo': dict(type=types[0], **FREE),
             'yhi': dict(type=types[1], **FREE)}
    mesh = box('quad', (6, 5), 0.0, 1.0, (True, False))
    plain = RKVdH2Integrator(_backend(_cfg(2, specs)), EulerSystem, mesh,
                             _cfg(2, specs))
    cfg = _cfg(2, specs, precision='single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '5')
    chosen = MixedRKIntegrator(_backend(cfg), EulerSystem, mesh, cfg)
    plain.run_steps(10)
    chosen.run_steps(10)
    (a,), (b,) = chosen.soln, plain.soln
    assert np.linalg.norm(a - b)/np.linalg.norm(b) < 1e-6


@pytest.mark.parametrize('kind,types', [
    ('euler', ('char-riem-inv-mass-flow', 'sup-out-fn')),
    ('euler', ('char-riem-inv-pressure', 'char-riem-inv')),
    ('ns', ('char-riem-inv-pressure', 'no-slp-adia-wall')),
    ('ns', ('no-slp-isot-wall', 'char-riem-inv-mass-flow'))])
def test_controlled_bcs_rhs(built, kind, types):
    """The controlled characteristic boundaries' ghost state with the
    pressure p(t) = ic + im*t of their controller (set here, with the
    controller between updates) against the oracle's char-riem-inv at that
    pressure, t = 0.3."""
    from pyfr_gb300.solvers.system import EulerSystem, NavierStokesSystem
    from tests.bc_cases import bc_case
    cfg, mesh, specs = bc_case(kind, types)
    cls = EulerSystem if kind == 'euler' else NavierStokesSystem
    s = cls(_backend(cfg), mesh, None, 2, cfg)
    s.commit()
    ctrls = s.controlled_bcs
    assert len(ctrls) == 1 and s.time_dependent
    (c,) = ctrls
    c.interp_c, c.interp_m = 0.8, 0.5
    c.tprev, c.nstep_counter = 0.1, 1
    s.rhs(0.3, 0, 1)
    assert c.nstep_counter == 2 and not c.history
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    ospecs = {n: dict(sp, type='char-riem-inv', p=0.8 + 0.5*0.3)
              if sp['type'].startswith('char-riem-inv-') else sp
              for n, sp in specs.items()}
    if kind == 'euler':
        d, _ = bc_disc('quad', (4, 3), (True, False), ospecs)
        ref = d.rhs_euler(u, GAS)
    else:
        d, _ = bc_disc('hex', (2, 2, 3), (True, True, False), ospecs,
                       ns=True)
        ref = d.rhs_ns(u, GAS)
    assert _relerr(r, ref) < TOL
