"""Artificial viscosity through the CUDA path against the oracle
(pyfr/solvers/baseadvecdiff/artvisc.py, kernels/shocksensor.mako,
kernels/avfill.mako, kernels/artvisc.mako and its use in
pyfr/solvers/navstokes/kernels/{tflux,intcflux,bccflux}.mako).

Plain FP64: relative max-norm 1e-10 on the right-hand side for the decay-fit
sensor (orders 2 and 3) and the modal-ratio sensor (order 1, every branch
taken), on periodic boxes and on a box with walls and a characteristic
boundary; three RK45 steps with CUDA graphs."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step, shock_sensor
from tests.test_artvisc import AV_C, av_case

pytestmark = pytest.mark.gpu

TOL = 1e-10
GAS = dict(gamma=1.4, mu=0.005, Pr=0.72, **{'ldg-beta': 0.5,
                                            'ldg-tau': 0.1})


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/np.abs(b).max()


def _cfg(order, c, cfg=None):
    from pyfr_gb300.inifile import Inifile
    if cfg is None:
        cfg = Inifile()
        cfg.set('backend', 'precision', 'double')
        for k in ('gamma', 'mu', 'Pr'):
            cfg.set('constants', k, GAS[k])
        cfg.set('solver-interfaces', 'riemann-solver', 'rusanov')
        for k in ('ldg-beta', 'ldg-tau'):
            cfg.set('solver-interfaces', k, GAS[k])
        cfg.set('solver-time-integrator', 'dt', 1e-4)
    cfg.set('constants', 'mu', GAS['mu'])
    cfg.set('solver', 'order', order)
    cfg.set('solver', 'shock-capturing', 'artificial-viscosity')
    for k, v in c.items():
        cfg.set('solver-artificial-viscosity', k, v)
    return cfg


def _backend(cfg):
    from pyfr_gb300.backend import B200Backend
    return B200Backend(cfg)


@pytest.mark.parametrize('et,n,order', [('hex', 4, 3), ('quad', 8, 2),
                                        ('quad', 8, 1)])
def test_ns_rhs_artvisc(built, et, n, order):
    from pyfr_gb300.mesh import periodic_box
    from pyfr_gb300.solvers.system import NavierStokesSystem
    from tests.oracle_util import disc_for_mesh

    mesh = periodic_box(et, n, 0.0, 1.0)
    av, u = av_case(et, mesh, order, AV_C[order])
    mu = shock_sensor(u, av)
    assert np.any(mu > 0)
    cfg = _cfg(order, AV_C[order])
    s = NavierStokesSystem(_backend(cfg), mesh, {et: u}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)

    # The vertex values on the device are the oracle's vertex maxima
    vtx = np.zeros(av['nnodes'])
    np.maximum.at(vtx, av['vnodes'].ravel(),
                  np.broadcast_to(mu, av['vnodes'].shape).ravel())
    assert _relerr(s._av.vertex_values(), vtx) < 1e-12

    d = disc_for_mesh(mesh, order, ns=True)
    assert _relerr(r, d.rhs_ns(u, GAS, av=av)) < TOL


def test_ns_rhs_artvisc_bcs(built):
    from pyfr_gb300.solvers.system import NavierStokesSystem
    from tests.test_gpu_bcs import FREE, _cfg as _bc_cfg
    from tests.test_oracle import bc_disc

    specs = {'zlo': dict(type='no-slp-isot-wall', cpTw=3.2, **FREE),
             'zhi': dict(type='char-riem-inv', **FREE)}
    d, mesh = bc_disc('hex', (3, 2, 3), (True, True, False), specs, ns=True)
    av, u = av_case('hex', mesh, 3, AV_C[3])
    cfg = _cfg(3, AV_C[3], _bc_cfg(3, specs, ns=True))
    s = NavierStokesSystem(_backend(cfg), mesh, {'hex': u}, 2, cfg)
    s.commit()
    s.rhs(0.0, 0, 1)
    (r,) = s.ele_scal_upts(1)
    assert _relerr(r, d.rhs_ns(u, GAS, av=av)) < TOL


def test_rk45_artvisc(built):
    """Three RK45 steps (CUDA graphs on)."""
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.mesh import periodic_box
    from pyfr_gb300.solvers.system import NavierStokesSystem
    from tests.oracle_util import disc_for_mesh

    mesh = periodic_box('quad', 8, 0.0, 1.0)
    av, u0 = av_case('quad', mesh, 2, AV_C[2])
    cfg = _cfg(2, AV_C[2])
    intg = RKVdH2Integrator(_backend(cfg), NavierStokesSystem, mesh, cfg,
                            {'quad': u0})
    intg.run_steps(3)
    (got,) = intg.soln

    d = disc_for_mesh(mesh, 2, ns=True)
    u = u0
    for _ in range(3):
        u = rk45_step(lambda x: d.rhs_ns(x, GAS, av=av), u, 1e-4)
    assert _relerr(got, u) < TOL


def test_chosen_form_artvisc(built):
    """Artificial viscosity in the chosen form (split-BF16 operators, FP32
    fluxes and sensor, FP64 accumulation; no reference-state shift): ten
    steps of the 5^3 hex box with a steep front within the chosen form's
    L2 bound of the FP64 plain form."""
    from pyfr_gb300.integrators import MixedRKIntegrator, RKVdH2Integrator
    from pyfr_gb300.mesh import periodic_box
    from pyfr_gb300.solvers.system import NavierStokesSystem

    mesh = periodic_box('hex', 5, 0.0, 1.0)
    av, u0 = av_case('hex', mesh, 3, AV_C[3])
    assert np.any(shock_sensor(u0, av) > 0)
    cfg = _cfg(3, AV_C[3])
    plain = RKVdH2Integrator(_backend(cfg), NavierStokesSystem, mesh, cfg,
                             {'hex': u0})
    cfg = _cfg(3, AV_C[3])
    cfg.set('backend', 'precision', 'single')
    cfg.set('backend-b200', 'mul-precision', 'bf16x3')
    cfg.set('backend-b200', 'split-products', '5')
    chosen = MixedRKIntegrator(_backend(cfg), NavierStokesSystem, mesh, cfg,
                               {'hex': u0})
    assert chosen.uref is None
    plain.run_steps(10)
    chosen.run_steps(10)
    (a,), (b,) = chosen.soln, plain.soln
    assert np.linalg.norm(a - b)/np.linalg.norm(b) < 1e-6
