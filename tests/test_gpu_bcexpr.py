"""Boundary values given as expressions of position and time (the
reference's [soln-bcs-<name>] expressions, pyfr/solvers/baseadvec/
inters.py:95-116) through the CUDA path against the oracle, which
evaluates the same text with numpy at the boundary points.

Plain FP64, relative max-norm 1e-10: the right-hand side at t = 0.3 for
Euler and Navier-Stokes boundaries whose values vary in space and time,
and three RK45 steps with a time-dependent inflow, where each stage sees
its own time t + c_i dt (CUDA graphs on and off)."""
import numpy as np
import pytest

from oracle.fr_oracle import rk45_step_t
from tests.test_oracle import bc_disc

pytestmark = pytest.mark.gpu

TOL = 1e-10
GAS = dict(gamma=1.4, mu=0.02, Pr=0.72, **{'ldg-beta': 0.5, 'ldg-tau': 0.1})
NP = dict(sin=np.sin, cos=np.cos, exp=np.exp, tanh=np.tanh, sqrt=np.sqrt,
          fabs=np.abs, pow=np.power, pi=np.pi)


@pytest.fixture(scope='module')
def built():
    import __graft_entry__ as ge
    ge.build_library()


def _relerr(a, b):
    return np.abs(a - b).max()/max(np.abs(b).max(), 1e-300)


def _fn(text, consts):
    """numpy evaluation of a boundary expression: f(x, t)."""
    def f(x, t):
        env = NP | consts | dict(x=x[0], y=x[1], t=t)
        if len(x) == 3:
            env['z'] = x[2]
        v = eval(text, {'__builtins__': {}}, env)
        return np.broadcast_to(np.asarray(v, dtype=float), x.shape[1:])
    return f


def _setup(ndims, specs, graphs=True):
    from tests.test_gpu_bcs import _cfg
    cfg = _cfg(ndims, {}, ns=True)
    cfg.set('constants', 'amp', 0.1)
    cfg.set('backend-b200', 'cuda-graphs', str(graphs).lower())
    for name, spec in specs.items():
        sect = f'soln-bcs-{name}'
        cfg.set(sect, 'type', spec['type'])
        for k, v in spec.items():
            if k == 'type':
                continue
            if k == 'u':
                for c, vv in zip('uvw', v):
                    cfg.set(sect, c, vv)
            else:
                cfg.set(sect, k, v)
    return cfg


def _oracle_specs(specs):
    consts = dict(amp=0.1)
    out = {}
    for name, spec in specs.items():
        o = {}
        for k, v in spec.items():
            if k == 'type':
                o[k] = v
            elif k == 'u':
                o[k] = [_fn(str(vv), consts) for vv in v]
            else:
                o[k] = _fn(str(v), consts)
        out[name] = o
    return out


EULER = {'ylo': dict(type='sup-in-fa', rho='1 + amp*sin(2*pi*x - t)',
                     p='1 + 0.05*cos(2*pi*x)*exp(-t)',
                     u=['0.4 + 0.1*t', '0.3 + 0.05*x']),
         'yhi': dict(type='char-riem-inv', rho='1.1', p='0.9 + 0.1*t*t',
                     u=['0.35', '-0.15*tanh(4*(x - 0.5))'])}

NS = {'zlo': dict(type='no-slp-isot-wall', cpTw='3.2 + 0.2*sin(pi*x*y)',
                  u=['0.1*sin(2*pi*y)', '0', '0']),
      'zhi': dict(type='sub-in-frv', rho='1 + amp*x*y*t',
                  u=['0.3', '0.1*cos(2*pi*x)', '-0.1 - 0.05*t'])}


def test_euler_bc_expressions_rhs(built):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.solvers.system import EulerSystem
    cfg = _setup(2, EULER)
    d, mesh = bc_disc('quad', (4, 3), (True, False),
                      _oracle_specs(EULER))
    s = EulerSystem(B200Backend(cfg), mesh, None, 2, cfg)
    s.commit()
    assert s.time_dependent
    s.rhs(0.3, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    assert _relerr(r, d.rhs_euler(u, GAS, 'rusanov', t=0.3)) < TOL


def test_ns_bc_expressions_rhs(built):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.solvers.system import NavierStokesSystem
    cfg = _setup(3, NS)
    d, mesh = bc_disc('hex', (2, 2, 3), (True, True, False),
                      _oracle_specs(NS), ns=True)
    s = NavierStokesSystem(B200Backend(cfg), mesh, None, 2, cfg)
    s.commit()
    s.rhs(0.3, 0, 1)
    (u,), (r,) = s.ele_scal_upts(0), s.ele_scal_upts(1)
    assert _relerr(r, d.rhs_ns(u, GAS, t=0.3)) < TOL


@pytest.mark.parametrize('graphs', [True, False])
def test_rk45_time_dependent_inflow(built, graphs):
    from pyfr_gb300.backend import B200Backend
    from pyfr_gb300.integrators import RKVdH2Integrator
    from pyfr_gb300.solvers.system import EulerSystem
    cfg = _setup(2, EULER, graphs)
    cfg.set('solver-time-integrator', 'tstart', 0.2)
    d, mesh = bc_disc('quad', (4, 3), (True, False),
                      _oracle_specs(EULER))
    intg = RKVdH2Integrator(B200Backend(cfg), EulerSystem, mesh, cfg)
    (u,) = intg.soln
    intg.run_steps(3)
    (got,) = intg.soln
    t, dt = 0.2, intg.dt
    for _ in range(3):
        u = rk45_step_t(lambda x, tt: d.rhs_euler(x, GAS, 'rusanov', t=tt),
                        u, t, dt)
        t += dt
    assert _relerr(got, u) < TOL
